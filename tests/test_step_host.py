"""ast_step_host: one step from host arrays to host arrays.  Page-locked
arrays are moved in bands of tile rows, the copies in, the banded step and
the copies out overlapping on three streams; every band's launch steps its
tiles with the same kernel as a whole-grid launch and all of them report to
one clock, so the result must equal ast_set_state + ast_step(1) +
ast_get_state bit for bit, clock included, for every kernel (FP32
persistent and per-tile, FP64 with 32x16 and 16x16 tiles), for grids with
fewer tile rows than bands and ragged edges, in place and apart, and over
consecutive calls.  Pageable arrays and the inflow rule take the three
calls in turn."""
import os

import numpy as np
import pytest

from asteriy_2d_gb300 import abi as A
from asteriy_2d_gb300 import problems, solver

pytestmark = pytest.mark.gpu


def pinned(shape):
    torch = pytest.importorskip("torch")
    return torch.zeros(shape, dtype=torch.float64, pin_memory=True)


def reference_run(cfg, s0, u0, nsteps, params=None):
    """nsteps of set_state + step(1) + get_state"""
    out = []
    with solver.Solver(cfg) as S:
        if params is not None:
            S.set_mlp(params)
        s, u = s0, u0
        for _ in range(nsteps):
            S.set_state(s, u)
            S.step(1)
            s, u = S.get_state()
            out.append((s, u, S.clock()))
    return out


def host_run(cfg, s0, u0, nsteps, params=None, in_place=False):
    K = cfg.N * cfg.M
    a_s, a_u, b_s, b_u = (pinned((K, 2)) for _ in range(4))
    a_s.numpy()[:] = s0
    a_u.numpy()[:] = u0
    out = []
    with solver.Solver(cfg) as S:
        if params is not None:
            S.set_mlp(params)
        for _ in range(nsteps):
            if in_place:
                S.step_host(a_s.data_ptr(), a_u.data_ptr(), a_s.data_ptr(), a_u.data_ptr())
                out.append((a_s.numpy().copy(), a_u.numpy().copy(), S.clock()))
            else:
                S.step_host(a_s.data_ptr(), a_u.data_ptr(), b_s.data_ptr(), b_u.data_ptr())
                out.append((b_s.numpy().copy(), b_u.numpy().copy(), S.clock()))
                a_s, b_s, a_u, b_u = b_s, a_s, b_u, a_u
        S.synchronize()
    return out


def assert_same(ref, got):
    assert len(ref) == len(got)
    for i, ((s1, u1, c1), (s2, u2, c2)) in enumerate(zip(ref, got)):
        assert np.array_equal(s1, s2) and np.array_equal(u1, u2), i
        assert c1 == c2, (i, c1, c2)


CASES = [
    # (precision, persistent, flux, grid)
    (A.PREC_FP32, 1, A.FLUX_HLL, (512, 384)),       # 24 tile rows: 16 bands of 1-2
    (A.PREC_FP32, 1, A.FLUX_HLLC, (64, 3200)),      # 200 tile rows: 16 bands of 12-13
    (A.PREC_FP32, 1, A.FLUX_GODUNOV, (300, 130)),   # 9 tile rows, ragged edges
    (A.PREC_FP32, 0, A.FLUX_HLLC, (256, 272)),      # per-tile FP32 kernel, 17 tile rows
    (A.PREC_FP64, 0, A.FLUX_HLLC, (1024, 512)),     # FP64, 32x16 tiles
    (A.PREC_FP64, 0, A.FLUX_GODUNOV, (97, 45)),     # FP64, 16x16 tiles, 3 tile rows
    (A.PREC_FP32, 1, A.FLUX_HLLC_A, (40, 7)),       # one tile row: one band
    (A.PREC_FP32, 2, A.FLUX_HLL, (512, 384)),       # strip kernel, 16 bands (strips cut at band edges)
    (A.PREC_FP32, 2, A.FLUX_HLLC, (64, 3200)),      # strip kernel, bands of 12-13 tile rows
    (A.PREC_FP32, 2, A.FLUX_HLLC_A, (300, 130)),    # strip kernel, ragged edges
]


@pytest.mark.parametrize("prec,persistent,flux,grid", CASES)
def test_banded_host_step_equals_set_step_get(prec, persistent, flux, grid):
    cfg = problems.blast_config(*grid, flux=flux, precision=prec)
    cfg.persistent = persistent
    s0, u0 = solver.fill_blast(cfg)
    u0[:, 0] = np.linspace(-0.3, 0.4, len(u0))
    u0[:, 1] = 0.1
    assert_same(reference_run(cfg, s0, u0, 5), host_run(cfg, s0, u0, 5))


def test_uniform_tile_variant_and_stats():
    # the persistent kernel's skip_uniform variant in bands; the counters
    # of the banded step equal those of the whole-grid step
    cfg = problems.blast_config(640, 320, flux=A.FLUX_GODUNOV, precision=A.PREC_FP32)
    cfg.skip_uniform, cfg.collect_stats = 1, 1
    s0, u0 = solver.fill_blast(cfg)
    ref = reference_run(cfg, s0, u0, 3)
    assert_same(ref, host_run(cfg, s0, u0, 3))
    K = cfg.N * cfg.M
    a = [pinned((K, 2)) for _ in range(4)]
    a[0].numpy()[:] = s0
    a[1].numpy()[:] = u0
    with solver.Solver(cfg) as S:
        S.step_host(*(t.data_ptr() for t in a))
        st_host = S.stats()
    with solver.Solver(cfg) as S:
        S.set_state(s0, u0)
        S.step(1)
        st_plain = S.stats()
    assert st_host == st_plain


@pytest.mark.parametrize("prec", [A.PREC_FP32, A.PREC_FP64])
def test_in_place(prec):
    cfg = problems.wind_config(256, 160, precision=prec)
    s0, u0 = solver.fill_wind(cfg)
    assert_same(reference_run(cfg, s0, u0, 4), host_run(cfg, s0, u0, 4, in_place=True))


def test_learned_start_value():
    params = np.load(os.path.join(os.path.dirname(solver.__file__), "data", "guess_blast.npy"))
    cfg = problems.blast_config(512, 256, flux=A.FLUX_GODUNOV, precision=A.PREC_FP32)
    cfg.guess, cfg.riemann_tol = A.GUESS_MLP, 1e-8
    s0, u0 = solver.fill_blast(cfg)
    assert_same(reference_run(cfg, s0, u0, 3, params), host_run(cfg, s0, u0, 3, params))


def test_pageable_and_inflow_take_the_plain_calls():
    cfg = problems.blast_config(128, 64, flux=A.FLUX_HLLC, precision=A.PREC_FP64)
    s0, u0 = solver.fill_blast(cfg)
    ref = reference_run(cfg, s0, u0, 1)[0]
    with solver.Solver(cfg) as S:
        s, u = np.empty_like(s0), np.empty_like(u0)
        S.step_host(s0.ctypes.data, u0.ctypes.data, s.ctypes.data, u.ctypes.data)
        assert np.array_equal(s, ref[0]) and np.array_equal(u, ref[1]) and S.clock() == ref[2]
    cfg.inflow_p, cfg.inflow_v = 7.0, 1.0
    ref = reference_run(cfg, s0, u0, 2)
    assert_same(ref, host_run(cfg, s0, u0, 2))


def test_overlapping_arrays_are_refused():
    cfg = problems.blast_config(64, 32, precision=A.PREC_FP64)
    K = cfg.N * cfg.M
    big = pinned((3 * K, 2))
    p = big.data_ptr()
    with solver.Solver(cfg) as S:
        with pytest.raises(solver.AstError):
            # s_out starts half way into s_in
            S.step_host(p, p + K * 16, p + K * 8, p + 2 * K * 16)
        with pytest.raises(solver.AstError):
            S.step_host(p, p + K * 16, p + 2 * K * 16, p + 2 * K * 16)


@pytest.mark.parametrize("prec,persistent,grid,in_place", [
    (A.PREC_FP32, 1, (512, 384), False),
    (A.PREC_FP32, 1, (300, 130), True),
    (A.PREC_FP64, 0, (256, 160), False),
])
def test_n_steps_chain_equals_single_steps(prec, persistent, grid, in_place):
    # ast_step_host_n: the copies of consecutive steps overlap; every step's
    # result must still equal the step-by-step one, and the last result
    # lies in the pair the step count's parity names
    cfg = problems.blast_config(*grid, flux=A.FLUX_GODUNOV, precision=prec)
    cfg.persistent = persistent
    s0, u0 = solver.fill_blast(cfg)
    u0[:, 0] = np.linspace(-0.3, 0.4, len(u0))
    K = cfg.N * cfg.M
    for n in (1, 4, 7):
        ref = reference_run(cfg, s0, u0, n)[-1]
        a_s, a_u, b_s, b_u = (pinned((K, 2)) for _ in range(4))
        a_s.numpy()[:] = s0
        a_u.numpy()[:] = u0
        if in_place:
            b_s, b_u = a_s, a_u
        with solver.Solver(cfg) as S:
            S.step_host_n(n, a_s.data_ptr(), a_u.data_ptr(), b_s.data_ptr(), b_u.data_ptr())
            clk = S.clock()
        s, u = (b_s, b_u) if n % 2 else (a_s, a_u)
        assert np.array_equal(s.numpy(), ref[0]) and np.array_equal(u.numpy(), ref[1]), n
        assert clk == ref[2]


def test_n_steps_pageable_takes_the_plain_calls():
    cfg = problems.blast_config(128, 64, flux=A.FLUX_HLLC, precision=A.PREC_FP32)
    s0, u0 = solver.fill_blast(cfg)
    ref = reference_run(cfg, s0, u0, 3)[-1]
    a_s, a_u = s0.copy(), u0.copy()
    b_s, b_u = np.empty_like(s0), np.empty_like(u0)
    with solver.Solver(cfg) as S:
        S.step_host_n(3, a_s.ctypes.data, a_u.ctypes.data, b_s.ctypes.data, b_u.ctypes.data)
        clk = S.clock()
    assert np.array_equal(b_s, ref[0]) and np.array_equal(b_u, ref[1]) and clk == ref[2]
    with solver.Solver(cfg) as S:
        S.step_host_n(0, a_s.ctypes.data, a_u.ctypes.data, b_s.ctypes.data, b_u.ctypes.data)
        assert S.clock()[2] == 0
        with pytest.raises(solver.AstError):
            S.step_host_n(-1, a_s.ctypes.data, a_u.ctypes.data, b_s.ctypes.data, b_u.ctypes.data)
