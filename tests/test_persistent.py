"""The FP32 solver's persistent kernel (tiles staged and stored by bulk-tensor
copies, ghost cells filled from the staged tile) against the one-CTA-per-
tile kernel: the same device code for faces and updates, so the two agree to
rounding (the compiler may fuse a multiply and an add differently in the two
kernels), on grids whose tiles are mostly or entirely boundary tiles, ragged
grids, every boundary kind and the fixed region."""
import numpy as np
import pytest

from asteriy_2d_gb300 import abi as A
from asteriy_2d_gb300 import problems, solver

pytestmark = pytest.mark.gpu

TOL, CTOL = 1e-5, 1e-6


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


def assert_agree(cfg, s0, u0, nsteps, params=None):
    s1, u1, c1, st1 = run(cfg, s0, u0, nsteps, 1, params)
    s0_, u0_, c0, st0 = run(cfg, s0, u0, nsteps, 0, params)
    for a, b in ((s1, s0_), (u1, u0_)):
        err = np.max(np.abs(a - b), axis=0) / np.maximum(np.max(np.abs(b), axis=0), 1e-300)
        assert np.all(err <= TOL), err
    assert c1[2] == c0[2] == nsteps
    assert abs(c1[0] - c0[0]) <= CTOL * c0[0] and abs(c1[1] - c0[1]) <= CTOL * c0[1], (c1, c0)
    # status bits can differ through faces no updated cell uses (the two
    # kernels fill ghost layers beyond the second differently); none may be
    # non-finite or timed out
    for st in (st1, st0):
        assert not st["status"] & (A.AST_ST_NONFINITE | A.AST_ST_TIMEOUT), st["status"]
    return s1


@pytest.mark.parametrize("flux", [A.FLUX_HLL, A.FLUX_HLLC, A.FLUX_GODUNOV])
@pytest.mark.parametrize("grid", [(256, 128), (150, 70), (33, 17), (4, 4), (97, 5)])
def test_blast_fp32_persistent_agrees(flux, grid):
    cfg = problems.blast_config(*grid, flux=flux, precision=A.PREC_FP32)
    s0, u0 = solver.fill_blast(cfg)
    s = assert_agree(cfg, s0, u0, 40)
    assert np.all(np.isfinite(s))


def test_wind_fp32_persistent_agrees():
    cfg = problems.wind_config(300, 150, precision=A.PREC_FP32)
    s0, u0 = solver.fill_wind(cfg)
    assert_agree(cfg, s0, u0, 40)


@pytest.mark.parametrize("kinds", [(A.BC_REFLECT,) * 4, (A.BC_OUTFLOW,) * 4,
                                   (A.BC_FIXED, A.BC_OUTFLOW, A.BC_REFLECT, A.BC_SUCTION),
                                   (A.BC_SUCTION, A.BC_FIXED, A.BC_SUCTION, A.BC_FIXED)])
def test_boundary_kinds_persistent_agree(kinds):
    cfg = problems.blast_config(70, 45, flux=A.FLUX_HLLC, precision=A.PREC_FP32)
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


def test_learned_guess_persistent_agrees():
    import os
    params = np.load(os.path.join(os.path.dirname(solver.__file__), "data", "guess_blast.npy"))
    cfg = problems.blast_config(256, 128, flux=A.FLUX_GODUNOV, precision=A.PREC_FP32)
    cfg.guess, cfg.riemann_tol = A.GUESS_MLP, 1e-8
    s0, u0 = solver.fill_blast(cfg)
    assert_agree(cfg, s0, u0, 60, params)


def test_persistent_many_steps_and_graph_blocks():
    # 37 steps: two captured blocks of 16 and five single launches; the tile
    # counter must rewind every step
    cfg = problems.blast_config(512, 256, flux=A.FLUX_GODUNOV, precision=A.PREC_FP32)
    s0, u0 = solver.fill_blast(cfg)
    assert_agree(cfg, s0, u0, 37)
