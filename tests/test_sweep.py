"""The FP32 solver's strip kernel (persistent = 2: each warp sweeps a strip
of 30 columns up its rows, stencil, fluxes and update in registers) against
the persistent tile kernel (persistent = 1) and the one-CTA-per-tile kernel
(persistent = 0).  Every face and cell is evaluated by the same device
functions in the same order, so the kernels agree to rounding (the compiler
may fuse a multiply and an add differently in different kernels), on the
blast and wind problems, ragged grids, grids of a few cells, every
boundary kind, the fixed region, region selection, the body force and
planar geometry; and the oracle bounds the FP32 strip kernel's error as it
bounds the others'."""
import os

import numpy as np
import pytest

import pyoracle as O
from asteriy_2d_gb300 import abi as A
from asteriy_2d_gb300 import problems, solver

pytestmark = pytest.mark.gpu
TOL, CTOL = 1e-5, 1e-6
FLUXES = [A.FLUX_HLL, A.FLUX_HLLC, A.FLUX_HLLC_A, A.FLUX_GODUNOV]


def run(cfg, s0, u0, nsteps, persistent, params=None):
    c = cfg.copy()
    c.persistent = persistent
    c.collect_stats = 1
    with solver.Solver(c) as S:
        if params is not None:
            S.set_mlp(params)
        S.set_state(s0, u0)
        S.step(nsteps)
        s, u = S.get_state()
        return s, u, S.clock(), S.stats()


def assert_agree(cfg, s0, u0, nsteps, other=1, params=None):
    s2, u2, c2, st2 = run(cfg, s0, u0, nsteps, 2, params)
    s1, u1, c1, st1 = run(cfg, s0, u0, nsteps, other, params)
    for a, b in ((s2, s1), (u2, u1)):
        err = np.max(np.abs(a - b), axis=0) / np.maximum(np.max(np.abs(b), axis=0), 1e-300)
        assert np.all(err <= TOL), err
    assert c2[2] == c1[2] == nsteps
    assert abs(c2[0] - c1[0]) <= CTOL * c1[0] and abs(c2[1] - c1[1]) <= CTOL * c1[1], (c2, c1)
    assert st2["rho_floor"] == st1["rho_floor"] and st2["p_floor"] == st1["p_floor"]
    assert not st2["status"] & (A.AST_ST_NONFINITE | A.AST_ST_TIMEOUT), st2["status"]
    return s2, u2


@pytest.mark.parametrize("flux", FLUXES)
@pytest.mark.parametrize("grid", [(256, 128), (150, 70), (33, 17), (4, 4), (97, 5), (61, 200)])
def test_blast_strip_kernel_agrees(flux, grid):
    cfg = problems.blast_config(*grid, flux=flux, precision=A.PREC_FP32)
    s0, u0 = solver.fill_blast(cfg)
    s, _ = assert_agree(cfg, s0, u0, 40)
    assert np.all(np.isfinite(s))


@pytest.mark.parametrize("recon", [A.RECON_MINMOD, A.RECON_NONE])
def test_wind_strip_kernel_agrees(recon):
    cfg = problems.wind_config(300, 150, precision=A.PREC_FP32)
    cfg.recon = recon
    s0, u0 = solver.fill_wind(cfg)
    assert_agree(cfg, s0, u0, 40)
    assert_agree(cfg, s0, u0, 40, other=0)


@pytest.mark.parametrize("kinds", [(A.BC_REFLECT,) * 4, (A.BC_OUTFLOW,) * 4,
                                   (A.BC_FIXED, A.BC_OUTFLOW, A.BC_REFLECT, A.BC_SUCTION),
                                   (A.BC_SUCTION, A.BC_FIXED, A.BC_SUCTION, A.BC_FIXED),
                                   (A.BC_NONREFLECT, A.BC_NONREFLECT, A.BC_REFLECT, A.BC_NONREFLECT)])
@pytest.mark.parametrize("flux", [A.FLUX_HLL, A.FLUX_HLLC])
def test_boundary_kinds_strip_kernel_agrees(kinds, flux):
    cfg = problems.blast_config(70, 45, flux=flux, precision=A.PREC_FP32)
    cfg.geom = A.GEOM_PLANAR
    for side, kind in enumerate(kinds):
        if kind == A.BC_FIXED:
            A.set_bc(cfg, side, kind, 1.2, 0.3, 0.1, -0.05)
        elif kind == A.BC_SUCTION:
            A.set_bc(cfg, side, kind, 0.0, 0.0, 0.02, -0.01)
        else:
            A.set_bc(cfg, side, kind)
    s0, u0 = solver.fill_blast(cfg)
    u0[:, 0] = 0.3
    u0[:, 1] = -0.2
    assert_agree(cfg, s0, u0, 30)


def test_region_select_and_body_force_strip_kernel_agrees():
    import golden_configs as G
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "step_tvd.npz"))
    cfg = G.tvd_config()
    cfg.precision = A.PREC_FP32
    cfg.flux = A.FLUX_HLLC
    assert cfg.region_select and cfg.body_force
    assert_agree(cfg, d["s0"], d["u0"], 20)


def test_strip_kernel_error_against_fp64_oracle():
    cfg = problems.blast_config(256, 128, flux=A.FLUX_HLL, precision=A.PREC_FP32)
    cfg.persistent = 2
    s0, u0 = solver.fill_blast(cfg)
    with solver.Solver(cfg) as S:
        S.set_state(s0, u0)
        S.step(100)
        s, _ = S.get_state()
    os_, *_ = O.run(problems.blast_config(256, 128, flux=A.FLUX_HLL), s0, u0, 100, nthreads=os.cpu_count() or 1)
    l1 = np.sum(np.abs(s[:, 0] - os_[:, 0])) / np.sum(np.abs(os_[:, 0]))
    assert l1 < 1e-4, l1


def test_strip_kernel_many_steps_and_graph_blocks():
    # 37 steps: two captured blocks of 16 and five single launches; the strip
    # counter must rewind every step
    cfg = problems.blast_config(512, 256, flux=A.FLUX_HLL, precision=A.PREC_FP32)
    s0, u0 = solver.fill_blast(cfg)
    assert_agree(cfg, s0, u0, 37)


def test_learned_start_strip_kernel_agrees():
    # the strip kernel evaluates the network in FP32, the tile kernels in
    # f16 tensor-core tiles: the start values differ, the Newton iteration
    # converges to the same tolerance
    params = np.load(os.path.join(os.path.dirname(solver.__file__), "data", "guess_blast.npy"))
    cfg = problems.blast_config(256, 128, flux=A.FLUX_GODUNOV, precision=A.PREC_FP32)
    cfg.guess, cfg.riemann_tol = A.GUESS_MLP, 1e-8
    s0, u0 = solver.fill_blast(cfg)
    assert_agree(cfg, s0, u0, 60, params=params)
    _, _, _, st = run(cfg, s0, u0, 60, 2, params)
    assert st["strong_calls"] > 0 and st["mlp_fallback"] == 0
