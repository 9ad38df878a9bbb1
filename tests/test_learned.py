"""The learned start value end to end on the GPU: record exact-solver faces
from the FP64 solver, train the network with the CUDA kernels, and compare
the FP32 Godunov solver started from the network with the same solver
started from the acoustic (PVRS-type) value at the same Newton tolerance."""
import os

import numpy as np
import pytest

import pyoracle as O
from asteriy_2d_gb300 import abi as A
from asteriy_2d_gb300 import learned, problems, solver

pytestmark = pytest.mark.gpu


def fp32_run(cfg, s0, u0, nsteps, params=None):
    c = cfg.copy()
    c.precision = A.PREC_FP32
    c.collect_stats = 1
    c.riemann_tol = 1e-8
    c.guess = A.GUESS_MLP if params is not None else A.GUESS_PVRS
    with solver.Solver(c) as S:
        if params is not None:
            S.set_mlp(params)
        S.set_state(s0, u0)
        S.step(nsteps)
        s, u = S.get_state()
        st = S.stats()
    return s, u, st


def test_recorder_trainer_and_learned_guess():
    cfg = problems.blast_config(128, 64, flux=A.FLUX_GODUNOV)
    s0, u0 = solver.fill_blast(cfg)
    rec, offered = learned.record_faces(cfg, s0, u0, 150, every=1, capacity=1 << 20)
    assert offered == len(rec) > 1000
    assert np.all(np.isfinite(rec[:, :7]))
    pat = rec[:, 9].view(np.int32)
    assert set(np.unique(pat)) <= {2, 3}
    strong = learned.strong_records(rec, 0.2)
    assert len(strong) > 500
    # the recorder's own gate keeps the same faces (up to rounding of the
    # strength right at the gate: the kernel tests it in FP64 state, the
    # filter here from the float records)
    gated, offered_g = learned.record_faces(cfg, s0, u0, 150, every=1, capacity=1 << 20, min_strength=0.2)
    assert offered_g == len(gated)
    assert abs(len(gated) - len(strong)) <= max(2, len(strong) // 1000), (len(gated), len(strong))
    key = lambda r: set(zip(r[:, 7].view(np.int32).tolist(), r[:, 8].view(np.int32).tolist()))
    assert len(key(gated) ^ key(strong)) <= max(4, len(strong) // 500)
    samples = learned.sample_records(strong, min(len(strong), 1 << 16), seed=7)
    params, losses = learned.train_guess(samples, epochs=60, batch=1024, lr=3e-3, seed=7)
    assert losses[-1] < 0.7 * losses[0], losses

    # same problem, FP32 solver: learned vs acoustic start value; the faces
    # above the gate are the ones the network serves, counted in both runs
    sp, up, st_p = fp32_run(cfg, s0, u0, 150)
    sm, um, st_m = fp32_run(cfg, s0, u0, 150, params)
    it_p = st_p["strong_iters"] / st_p["strong_calls"]
    it_m = st_m["strong_iters"] / st_m["strong_calls"]
    fb = st_m["mlp_fallback"] / st_m["strong_calls"]
    print(f"mean Newton iterations on faces above the gate: PVRS {it_p:.3f}, learned {it_m:.3f}; "
          f"fallback rate {fb:.4f}; all faces PVRS {st_p['newton_iters'] / st_p['newton_calls']:.3f} "
          f"learned {st_m['newton_iters'] / st_m['newton_calls']:.3f}")
    assert st_p["strong_calls"] > 0 and abs(st_p["strong_calls"] - st_m["strong_calls"]) < 0.2 * st_p["strong_calls"]
    assert it_m < it_p
    assert fb < 0.1
    # both stay within the FP32 form's error bound against the FP64 oracle
    os_, ou, *_ = O.run(cfg, s0, u0, 150, nthreads=os.cpu_count() or 1)
    for s in (sp, sm):
        l1 = np.sum(np.abs(s[:, 0] - os_[:, 0])) / np.sum(np.abs(os_[:, 0]))
        assert l1 < 1e-4, l1


def test_recorder_is_fp64_only():
    # the recorder's records are training targets: FP64 exact-solver
    # solvers only; FP32 and HLL solvers refuse it
    for prec, flux in ((A.PREC_FP32, A.FLUX_GODUNOV), (A.PREC_FP64, A.FLUX_HLL)):
        cfg = problems.blast_config(64, 32, flux=flux, precision=prec)
        with solver.Solver(cfg) as S:
            with pytest.raises(solver.AstError) as e:
                S.record_start(1024)
            assert e.value.code == A.AST_ERR_UNSUPPORTED
