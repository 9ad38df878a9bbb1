"""Failure detection on the GPU, with no GPU fault: every failure here is
made on the host (tolerances, iteration caps, non-finite or negative input,
an oversized first time step) or by a short wait limit, and the tests check
the status bits and error codes the library reports.

  - iteration caps (riemann_max_iter = 1, tolerance 1e-300, which no
    iterate meets): the Newton and
    bisection caps set AST_ST_NEWTON_CAP / AST_ST_BISECT_CAP, as the
    reference's 1100-iteration prints mark non-convergence
    (kernel.cu:651, 667, 715); the state still equals the oracle's;
  - a NaN cell: AST_ST_NONFINITE, and ast_synchronize returns
    AST_ERR_NUMERIC; a cell with negative pressure (no real sound speed):
    with HLLC the pressure floor catches it, with HLL its NaN sound speed
    spreads, in both cases as in the oracle;
  - the density and pressure floors (kernel.cu:3060-3064, 3070-3073): a
    first step far above the CFL limit drives cells negative; the GPU counts
    the same floor hits as the oracle and sets AST_ST_RHO_FLOOR /
    AST_ST_P_FLOOR;
  - a bulk tile copy that does not arrive within the wait limit
    (copy_wait_polls = 1 poll): AST_ST_TIMEOUT and AST_ERR_CUDA from the
    synchronize call; the kernel then waits for the copy with its long
    limit, so the step's result equals the normal run's bit for bit and the
    context stays usable.
"""
import os

import numpy as np
import pytest

import golden_configs as G
import pyoracle as O
from asteriy_2d_gb300 import abi as A
from asteriy_2d_gb300 import problems, solver

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 1
TOL = 1e-10


def rel_linf(a, b):
    return np.max(np.abs(a - b), axis=0) / np.maximum(np.max(np.abs(b), axis=0), 1e-300)


def random_cfg(precision=A.PREC_FP64):
    cfg = problems.blast_config(64, 32, flux=A.FLUX_GODUNOV, precision=precision)
    s0, u0 = G.random_state(64 * 32, np.random.default_rng(11))
    return cfg, s0, u0


def test_iteration_caps_set_status_bits_fp64():
    cfg, s0, u0 = random_cfg()
    cfg.riemann_tol = 1e-300
    cfg.riemann_max_iter = 1
    cfg.collect_stats = 1
    with solver.Solver(cfg) as S:
        S.set_state(s0, u0)
        S.step(2)
        s, u = S.get_state()
        st = S.stats()
    assert st["status"] & A.AST_ST_NEWTON_CAP and st["status"] & A.AST_ST_BISECT_CAP
    assert st["newton_max_iters"] == 1
    os_, ou, _, _, _, cnt = O.run(cfg, s0, u0, 2, nthreads=NT)
    assert cnt[4] > 0 and cnt[7] > 0          # the oracle's newton_cap, bisect_cap
    assert np.all(rel_linf(s, os_) <= TOL) and np.all(rel_linf(u, ou) <= TOL)


@pytest.mark.parametrize("persistent", [0, 1])
def test_iteration_cap_sets_status_bit_fp32(persistent):
    cfg, s0, u0 = random_cfg(A.PREC_FP32)
    cfg.riemann_tol = 1e-300
    cfg.riemann_max_iter = 1
    cfg.persistent = persistent
    with solver.Solver(cfg) as S:
        S.set_state(s0, u0)
        S.step(2)
        assert S.stats()["status"] & A.AST_ST_NEWTON_CAP


@pytest.mark.parametrize("precision,persistent", [(A.PREC_FP64, 0), (A.PREC_FP32, 0), (A.PREC_FP32, 1),
                                                  (A.PREC_FP32, 2)])
def test_nan_cell_reports_numeric_error(precision, persistent):
    cfg = problems.blast_config(96, 48, flux=A.FLUX_HLLC, precision=precision)
    cfg.persistent = persistent
    s0, u0 = solver.fill_blast(cfg)
    s0[20 * 96 + 40, 0] = np.nan
    with solver.Solver(cfg) as S:
        S.set_state(s0, u0)
        S.step(1, sync=False)
        with pytest.raises(solver.AstError) as e:
            S.synchronize()
        assert e.value.code == A.AST_ERR_NUMERIC
        assert S.stats()["status"] & A.AST_ST_NONFINITE
    # the oracle's state is not finite there either
    os_, ou, *_ = O.run(problems.blast_config(96, 48, flux=A.FLUX_HLLC), s0, u0, 1, nthreads=NT)
    assert not np.all(np.isfinite(os_))


def negative_pressure_case(flux):
    cfg = problems.blast_config(96, 48, flux=flux)
    cfg.collect_stats = 1
    s0, u0 = solver.fill_blast(cfg)
    s0[20 * 96 + 40, 1] = -1.0
    return cfg, s0, u0


@pytest.mark.parametrize("flux", [A.FLUX_HLLC, A.FLUX_HLLC_A])
def test_negative_pressure_input_floored_like_the_oracle(flux):
    # a cell with p < 0 has no real sound speed; the HLLC bounds take the
    # larger of the two sides' speeds with CUDA's max (NaN dropped), so the
    # step stays finite and the pressure floor (kernel.cu:3070-3073)
    # catches the negative pressure: the GPU counts the oracle's floor hits
    # and matches its state
    cfg, s0, u0 = negative_pressure_case(flux)
    with solver.Solver(cfg) as S:
        S.set_state(s0, u0)
        S.step(1)
        s, u = S.get_state()
        st = S.stats()
    os_, ou, _, _, _, cnt = O.run(cfg, s0, u0, 1, nthreads=NT)
    assert np.all(np.isfinite(os_)) and cnt[1] > 0
    assert st["p_floor"] == cnt[1] and st["status"] & A.AST_ST_P_FLOOR
    assert not st["status"] & A.AST_ST_NONFINITE
    assert np.all(rel_linf(s, os_) <= TOL) and np.all(rel_linf(u, ou) <= TOL)


def test_negative_pressure_input_hll_reports_numeric_error_like_the_oracle():
    # the reference's HLL selects the larger sound speed with a comparison,
    # which passes a NaN from the right side on: its state becomes non-
    # finite, and the GPU's HLL (the same selects) reports AST_ERR_NUMERIC
    cfg, s0, u0 = negative_pressure_case(A.FLUX_HLL)
    os_, *_ = O.run(cfg, s0, u0, 1, nthreads=NT)
    assert not np.all(np.isfinite(os_))
    with solver.Solver(cfg) as S:
        S.set_state(s0, u0)
        S.step(1, sync=False)
        with pytest.raises(solver.AstError) as e:
            S.synchronize()
        assert e.value.code == A.AST_ERR_NUMERIC


@pytest.mark.parametrize("flux", [A.FLUX_HLL, A.FLUX_GODUNOV])
def test_floors_counted_like_the_oracle(flux):
    # a first step of dt 0.05 on cells of ~0.03 with flows of Mach ~3 empties
    # cells: densities and pressures that would go negative are floored
    cfg = problems.blast_config(64, 32, flux=flux)
    cfg.geom = A.GEOM_PLANAR
    cfg.dt_first = 0.05
    cfg.collect_stats = 1
    rng = np.random.default_rng(3)
    K = 64 * 32
    s0 = np.stack([rng.uniform(0.2, 1.0, K), rng.uniform(0.05, 0.2, K)], 1)
    u0 = np.stack([rng.uniform(-1.5, 1.5, K), rng.uniform(-1.5, 1.5, K)], 1)
    with solver.Solver(cfg) as S:
        S.set_state(s0, u0)
        S.step(1)
        s, u = S.get_state()
        st = S.stats()
    os_, ou, _, _, _, cnt = O.run(cfg, s0, u0, 1, nthreads=NT)
    assert cnt[0] > 0 and cnt[1] > 0
    assert st["rho_floor"] == cnt[0] and st["p_floor"] == cnt[1]
    assert st["status"] & A.AST_ST_RHO_FLOOR and st["status"] & A.AST_ST_P_FLOOR
    assert np.all(rel_linf(s, os_) <= TOL) and np.all(rel_linf(u, ou) <= TOL)


@pytest.mark.parametrize("flux", [A.FLUX_HLL, A.FLUX_GODUNOV])
def test_copy_wait_timeout_reported_and_result_unchanged(flux):
    cfg = problems.blast_config(512, 256, flux=flux, precision=A.PREC_FP32)
    cfg.persistent = 1
    s0, u0 = solver.fill_blast(cfg)
    with solver.Solver(cfg) as S:
        S.set_state(s0, u0)
        S.step(3)
        ref = S.get_state()
    short = cfg.copy()
    short.copy_wait_polls = 1
    with solver.Solver(short) as S:
        S.set_state(s0, u0)
        S.step(3, sync=False)
        with pytest.raises(solver.AstError) as e:
            S.synchronize()
        assert e.value.code == A.AST_ERR_CUDA
        assert S.stats()["status"] & A.AST_ST_TIMEOUT
        s, u = S.get_state()
    assert np.array_equal(s, ref[0]) and np.array_equal(u, ref[1])
    # the context is usable: a new solver steps as before
    with solver.Solver(cfg) as S:
        S.set_state(s0, u0)
        S.step(3)
        again = S.get_state()
    assert np.array_equal(again[0], ref[0])


@pytest.mark.parametrize("one_launch", [False, True])
def test_batch_copy_wait_timeout_reported_and_result_unchanged(one_launch):
    """The persistent batch kernel, per class and in one launch for the whole
    batch: a copy wait that runs out is reported and the step completes."""
    probs = solver.problem_set(64, 6, A.PREC_FP32)
    init = [solver.problem_fill(p) for p in probs]

    def run(polls):
        cfgs = []
        for p in probs:
            c = p.cfg.copy()
            c.copy_wait_polls = polls
            cfgs.append(c)
        with solver.Batch(cfgs) as B:
            for i, (s0, u0) in enumerate(init):
                B.set_state(i, s0, u0)
            if one_launch:
                B.set_mixed(2)   # the persistent kernel over every problem
            else:
                for cls in range(B.info()["launches_per_step"]):
                    B.set_schedule(cls, solver.PERSISTENT)
            B.step(2, sync=False)
            err = None
            try:
                B.synchronize()
            except solver.AstError as e:
                err = e.code
            status = [B.stats(i)["status"] for i in range(len(probs))]
            return err, status, [B.get_state(i)[0] for i in range(len(probs))]

    err0, st0, ref = run(0)
    err1, st1, got = run(1)
    assert err0 is None and all(not (s & A.AST_ST_TIMEOUT) for s in st0)
    assert err1 == A.AST_ERR_CUDA and any(s & A.AST_ST_TIMEOUT for s in st1)
    assert all(np.array_equal(a, b) for a, b in zip(got, ref))
