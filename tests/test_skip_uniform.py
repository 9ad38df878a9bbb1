"""skip_uniform: tiles whose staged cells are all bit-identical skip the
face pass and update on zero flux differences.  The results must be
identical, bit for bit, to the full computation: state, clock and counters,
for every flux, both precisions, both FP32 kernels, boundary kinds that
produce uniform ghost cells and ones that do not, and the batch."""
import numpy as np
import pytest

from asteriy_2d_gb300 import abi as A
from asteriy_2d_gb300 import problems, solver

pytestmark = pytest.mark.gpu


def run(cfg, s0, u0, nsteps, skip, params=None):
    c = cfg.copy()
    c.skip_uniform = skip
    c.collect_stats = 1
    with solver.Solver(c) as S:
        if params is not None:
            S.set_mlp(params)
        S.set_state(s0, u0)
        S.step(nsteps)
        s, u = S.get_state()
        return s, u, S.clock(), S.stats()


def assert_identical(cfg, s0, u0, nsteps, params=None):
    a = run(cfg, s0, u0, nsteps, 0, params)
    b = run(cfg, s0, u0, nsteps, 1, params)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert a[2] == b[2]
    assert a[3] == b[3]
    return a


@pytest.mark.parametrize("precision", [A.PREC_FP32, A.PREC_FP64])
@pytest.mark.parametrize("flux", [A.FLUX_HLL, A.FLUX_HLLC, A.FLUX_GODUNOV, A.FLUX_HLLC_A])
def test_blast_skip_uniform_identical(precision, flux):
    # the blast at rest around a small hot sphere: most tiles uniform
    cfg = problems.blast_config(384, 192, flux=flux, precision=precision)
    s0, u0 = solver.fill_blast(cfg)
    s, _, _, _ = assert_identical(cfg, s0, u0, 60)
    assert np.all(np.isfinite(s))


@pytest.mark.parametrize("persistent", [0, 1])
@pytest.mark.parametrize("flux", [A.FLUX_HLL, A.FLUX_GODUNOV])
def test_negative_zero_velocities_skip_uniform_identical(persistent, flux):
    # every velocity -0: the FP32 HLL face pairs' one-state path must not
    # take such stencils (the reconstruction gives +0 on one side and -0 on
    # the other, which the plain path does not find equal), so the results
    # stay bit-identical to the full computation
    cfg = problems.blast_config(384, 192, flux=flux, precision=A.PREC_FP32)
    cfg.persistent = persistent
    s0, u0 = solver.fill_blast(cfg)
    u0 = np.full_like(u0, -0.0)
    s, u, _, _ = assert_identical(cfg, s0, u0, 30)
    assert np.all(np.isfinite(s)) and np.all(np.isfinite(u))


@pytest.mark.parametrize("persistent", [0, 1])
@pytest.mark.parametrize("grid", [(150, 70), (97, 33), (33, 17)])
def test_ragged_grids_and_both_fp32_kernels(persistent, grid):
    cfg = problems.blast_config(*grid, flux=A.FLUX_GODUNOV, precision=A.PREC_FP32)
    cfg.persistent = persistent
    s0, u0 = solver.fill_blast(cfg)
    assert_identical(cfg, s0, u0, 40)


@pytest.mark.parametrize("kinds", [(A.BC_REFLECT,) * 4, (A.BC_OUTFLOW,) * 4,
                                   (A.BC_FIXED, A.BC_OUTFLOW, A.BC_REFLECT, A.BC_SUCTION),
                                   (A.BC_NONREFLECT, A.BC_FIXED, A.BC_REFLECT, A.BC_OUTFLOW)])
def test_boundary_kinds_skip_uniform_identical(kinds):
    # a uniform moving gas: reflecting walls flip a velocity in the ghost
    # cells (those tiles are not uniform), fixed sides may differ
    cfg = problems.blast_config(160, 96, flux=A.FLUX_HLLC, precision=A.PREC_FP32)
    cfg.geom = A.GEOM_PLANAR
    for side, kind in enumerate(kinds):
        if kind == A.BC_FIXED:
            A.set_bc(cfg, side, kind, 1.0, 0.1, 0.3, -0.2)
        elif kind == A.BC_SUCTION:
            A.set_bc(cfg, side, kind, 0.0, 0.0, 0.02, -0.01)
        else:
            A.set_bc(cfg, side, kind)
    s0, u0 = solver.fill_blast(cfg)
    u0[:, 0] = 0.3
    u0[:, 1] = -0.2
    assert_identical(cfg, s0, u0, 30)


def test_learned_start_and_wind_skip_uniform_identical():
    import os
    params = np.load(os.path.join(os.path.dirname(solver.__file__), "data", "guess_blast.npy"))
    cfg = problems.blast_config(256, 128, flux=A.FLUX_GODUNOV, precision=A.PREC_FP32)
    cfg.guess, cfg.riemann_tol = A.GUESS_MLP, 1e-8
    s0, u0 = solver.fill_blast(cfg)
    assert_identical(cfg, s0, u0, 80, params)
    # the wind: a fixed region and seeded noise (no uniform tiles off the
    # far field)
    cfg = problems.wind_config(200, 100, precision=A.PREC_FP32)
    s0, u0 = solver.fill_wind(cfg)
    assert_identical(cfg, s0, u0, 30)


def test_region_select_takes_the_full_path():
    cfg = problems.blast_config(128, 64, flux=A.FLUX_GODUNOV, precision=A.PREC_FP64)
    cfg.region_select, cfg.region_lo, cfg.region_hi = 1, -0.5, 0.5
    s0, u0 = solver.fill_blast(cfg)
    assert_identical(cfg, s0, u0, 20)


def test_batch_skip_uniform_identical():
    ps = solver.problem_set(64, 6)
    cfgs = []
    for p in ps:
        p.cfg.M = min(p.cfg.M, 96)
        p.cfg.N = 2 * p.cfg.M
        cfgs.append(p.cfg)
    init = [solver.problem_fill(p) for p in ps]
    out = []
    for skip in (0, 1):
        cs = [c.copy() for c in cfgs]
        for c in cs:
            c.skip_uniform = skip
        with solver.Batch(cs) as B:
            for i, (s0, u0) in enumerate(init):
                B.set_state(i, s0, u0)
            B.step(20)
            out.append([(B.get_state(i), B.clock(i)) for i in range(len(cs))])
    for (sa, ca), (sb, cb) in zip(*out):
        assert np.array_equal(sa[0], sb[0]) and np.array_equal(sa[1], sb[1])
        assert ca == cb

