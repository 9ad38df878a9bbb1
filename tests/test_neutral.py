"""The neutral-coupling momentum source of add_MK (kernel.cu:2495-2496):
T_do * (rho * n_H / Kn) * nn2.(x, y) added to the momentum.  The golden
vectors are 20 launches of the reference's own add_MK with a random nn2
(tests/golden/make_golden.py); the solver (ast_set_neutral, FP64 and the
FP32 form, both FP32 kernels) and the raw drop-in (ast_add_mk_raw) are
compared with them and with the oracle."""
import numpy as np
import pytest

from asteriy_2d_gb300 import abi as A
from asteriy_2d_gb300 import solver

import golden_configs as G
from conftest import golden
import pyoracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-10


def rel_linf(a, b):
    return np.max(np.abs(a - b), axis=0) / np.maximum(np.max(np.abs(b), axis=0), 1e-300)


def run(cfg, s0, u0, nn2, nsteps, device_src=False):
    with solver.Solver(cfg) as S:
        if device_src:
            import torch
            t = torch.tensor(np.ascontiguousarray(nn2), device="cuda:0")
            S.set_neutral_device(t.data_ptr())
        else:
            S.set_neutral(nn2)
        S.set_state(s0, u0)
        S.step(nsteps)
        s, u = S.get_state()
        return s, u, S.clock()


@pytest.mark.parametrize("device_src", [False, True])
def test_solver_matches_reference_add_mk(device_src):
    d = golden("step_mk_neutral.npz")
    cfg = G.add_mk_config(0)
    s, u, (tdo, tt, step) = run(cfg, d["s0"], d["u0"], d["nn2"], int(d["nsteps"]), device_src)
    assert np.all(rel_linf(s, d["s"]) <= TOL) and np.all(rel_linf(u, d["u"]) <= TOL)
    assert step == int(d["steps"]) and abs(tdo - float(d["T_do"])) <= 1e-12 * float(d["T_do"])


def test_raw_drop_in_matches_reference_add_mk():
    import torch
    d = golden("step_mk_neutral.npz")
    cfg = G.add_mk_config(0)
    dev = torch.device("cuda:0")
    bufs = [torch.tensor(d["s0"], device=dev), torch.tensor(d["u0"], device=dev)]
    bufs2 = [torch.empty_like(bufs[0]), torch.empty_like(bufs[1])]
    nn2 = torch.tensor(d["nn2"], device=dev)
    T = torch.tensor([1e7], dtype=torch.float64, device=dev)
    T_do = torch.tensor([cfg.dt_first], dtype=torch.float64, device=dev)
    TT = torch.zeros(1, dtype=torch.float64, device=dev)
    i = torch.zeros(1, dtype=torch.int32, device=dev)
    for _ in range(int(d["nsteps"])):
        solver.add_mk_raw(bufs[0].data_ptr(), bufs[1].data_ptr(), bufs2[0].data_ptr(), bufs2[1].data_ptr(),
                          nn2.data_ptr(), T.data_ptr(), T_do.data_ptr(), cfg)
        solver.funk_time(T.data_ptr(), T_do.data_ptr(), TT.data_ptr(), i.data_ptr())
        bufs, bufs2 = bufs2, bufs
    torch.cuda.synchronize()
    s, u = bufs[0].cpu().numpy(), bufs[1].cpu().numpy()
    assert np.all(rel_linf(s, d["s"]) <= TOL) and np.all(rel_linf(u, d["u"]) <= TOL)
    assert int(i.item()) == int(d["steps"])
    assert abs(T_do.item() - float(d["T_do"])) <= 1e-12 * float(d["T_do"])


@pytest.mark.parametrize("flux", [A.FLUX_HLLC, A.FLUX_GODUNOV])
@pytest.mark.parametrize("geom", [A.GEOM_AXISYM, A.GEOM_PLANAR])
def test_fp64_solver_matches_oracle(flux, geom):
    cfg = G.add_mk_config(0, N=70, M=37)
    cfg.flux, cfg.recon, cfg.geom, cfg.riemann_tol = flux, A.RECON_MINMOD, geom, 1e-13
    rng = np.random.default_rng(flux * 10 + geom)
    s0, u0 = G.random_state(cfg.N * cfg.M, rng)
    nn2 = rng.uniform(-1.0, 1.0, (cfg.N * cfg.M, 3))
    s, u, (tdo, tt, step) = run(cfg, s0, u0, nn2, 15)
    os_, ou, otdo, ott, ost, _ = O.run(cfg, s0, u0, 15, nn2=nn2)
    assert np.all(rel_linf(s, os_) <= TOL) and np.all(rel_linf(u, ou) <= TOL)
    assert step == ost and abs(tdo - otdo) <= 1e-12 * otdo


@pytest.mark.parametrize("persistent", [1, 0])
def test_fp32_form_matches_oracle(persistent):
    cfg = G.add_mk_config(0, N=130, M=66)
    cfg.flux, cfg.recon, cfg.precision, cfg.persistent = A.FLUX_HLLC, A.RECON_MINMOD, A.PREC_FP32, persistent
    rng = np.random.default_rng(5)
    s0, u0 = G.random_state(cfg.N * cfg.M, rng)
    nn2 = rng.uniform(-1.0, 1.0, (cfg.N * cfg.M, 3))
    s, u, _ = run(cfg, s0, u0, nn2, 10)
    cfg64 = cfg.copy()
    cfg64.precision = A.PREC_FP64
    os_, ou, *_ = O.run(cfg64, s0, u0, 10, nn2=nn2)
    assert np.all(rel_linf(s, os_) <= 2e-5) and np.all(rel_linf(u, ou) <= 2e-5)
    # the source moved the state: the run without it differs
    s_no, u_no, _ = run(cfg, s0, u0, None, 10)
    assert np.max(np.abs(u_no - u)) > 1e-3


def test_removing_the_source_restores_the_plain_step():
    cfg = G.add_mk_config(0, N=64, M=32)
    rng = np.random.default_rng(9)
    s0, u0 = G.random_state(cfg.N * cfg.M, rng)
    nn2 = rng.uniform(-1.0, 1.0, (cfg.N * cfg.M, 3))
    plain = run(cfg, s0, u0, None, 32)
    with solver.Solver(cfg) as S:
        # 16 steps: a captured block, which must not outlive the source
        S.set_neutral(nn2)
        S.set_state(s0, u0)
        S.step(16)
        S.set_neutral(None)
        S.set_state(s0, u0)
        S.set_clock(cfg.dt_first, 0.0, 0)
        S.step(32)
        s, u = S.get_state()
    assert np.array_equal(s, plain[0]) and np.array_equal(u, plain[1])


def test_zero_kn_means_no_source():
    cfg = G.add_mk_config(0, N=40, M=20)
    cfg.neutral_kn = 0.0
    rng = np.random.default_rng(2)
    s0, u0 = G.random_state(cfg.N * cfg.M, rng)
    nn2 = rng.uniform(-1.0, 1.0, (cfg.N * cfg.M, 3))
    a = run(cfg, s0, u0, nn2, 5)
    b = run(cfg, s0, u0, None, 5)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


@pytest.mark.parametrize("prec", [A.PREC_FP64, A.PREC_FP32])
def test_host_step_with_source(prec):
    # FP64: the banded pipeline (the source inside every band's update);
    # FP32: the three calls (the source pass runs over the whole grid)
    torch = pytest.importorskip("torch")
    cfg = G.add_mk_config(0, N=96, M=80)
    cfg.precision = prec
    K = cfg.N * cfg.M
    rng = np.random.default_rng(17)
    s0, u0 = G.random_state(K, rng)
    nn2 = rng.uniform(-1.0, 1.0, (K, 3))
    ref = run(cfg, s0, u0, nn2, 1)
    hs, hu, os_, ou = (torch.zeros((K, 2), dtype=torch.float64, pin_memory=True) for _ in range(4))
    hs.numpy()[:] = s0
    hu.numpy()[:] = u0
    with solver.Solver(cfg) as S:
        S.set_neutral(nn2)
        S.step_host(hs.data_ptr(), hu.data_ptr(), os_.data_ptr(), ou.data_ptr())
        clk = S.clock()
    assert np.array_equal(os_.numpy(), ref[0]) and np.array_equal(ou.numpy(), ref[1]) and clk == ref[2]
