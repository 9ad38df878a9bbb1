"""The step that allocates nothing (ast_step_noalloc).

Some callers cannot call cudaMalloc while they step (a device-memory budget
owned by a different allocator, a real-time loop).  ast_step_noalloc does
one step and the dt shift with its reduction state in a static device array
(three kernels: clock in, step, clock out).  Here it is called twice in a
row through the C ABI and compared with the existing entry points
ast_step_raw + ast_funk_time on the same inputs: the states within the
parity tolerance, the clock (T_do, TT, step) equal.  This file is collected
last; it passes alone in a fresh process too.
"""
import numpy as np
import pytest

import golden_configs as G
from asteriy_2d_gb300 import abi as A
from asteriy_2d_gb300 import problems, solver

pytestmark = pytest.mark.gpu
TOL = 1e-10


def rel_linf(a, b):
    return np.max(np.abs(a - b), axis=0) / np.maximum(np.max(np.abs(b), axis=0), 1e-300)


@pytest.mark.parametrize("name", ["blast_hllc", "kernel_tvd"])
def test_noalloc_step_matches_raw_step_twice(name):
    import torch
    dev = torch.device("cuda:0")
    if name == "blast_hllc":
        cfg = problems.blast_config(96, 48, flux=A.FLUX_HLLC)
        s0, u0 = solver.fill_blast(cfg)
    else:
        cfg = G.tvd_config()
        s0, u0 = G.random_state(cfg.N * cfg.M, np.random.default_rng(5))

    # existing entry points: ast_step_raw + ast_funk_time, two steps
    a = [torch.tensor(s0, device=dev), torch.tensor(u0, device=dev)]
    b = [torch.empty_like(a[0]), torch.empty_like(a[1])]
    T = torch.tensor([1e7], dtype=torch.float64, device=dev)
    T_do = torch.tensor([cfg.dt_first], dtype=torch.float64, device=dev)
    TT = torch.zeros(1, dtype=torch.float64, device=dev)
    i = torch.zeros(1, dtype=torch.int32, device=dev)
    for _ in range(2):
        solver.step_raw(a[0].data_ptr(), a[1].data_ptr(), b[0].data_ptr(), b[1].data_ptr(), T.data_ptr(),
                        T_do.data_ptr(), TT.data_ptr(), cfg)
        solver.funk_time(T.data_ptr(), T_do.data_ptr(), TT.data_ptr(), i.data_ptr())
        a, b = b, a

    # the allocation-free entry point, two calls in a row
    c = [torch.tensor(s0, device=dev), torch.tensor(u0, device=dev)]
    d = [torch.empty_like(c[0]), torch.empty_like(c[1])]
    T_do2 = torch.tensor([cfg.dt_first], dtype=torch.float64, device=dev)
    TT2 = torch.zeros(1, dtype=torch.float64, device=dev)
    step2 = torch.zeros(1, dtype=torch.int64, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    for _ in range(2):
        solver.step_noalloc(c[0].data_ptr(), c[1].data_ptr(), d[0].data_ptr(), d[1].data_ptr(), T_do2.data_ptr(),
                            TT2.data_ptr(), step2.data_ptr(), cfg, status=status.data_ptr())
        c, d = d, c
    torch.cuda.synchronize()

    s_ref, u_ref = a[0].cpu().numpy(), a[1].cpu().numpy()
    s_new, u_new = c[0].cpu().numpy(), c[1].cpu().numpy()
    assert np.all(rel_linf(s_new, s_ref) <= TOL) and np.all(rel_linf(u_new, u_ref) <= TOL)
    assert abs(T_do2.item() - T_do.item()) <= 1e-12 * T_do.item()
    assert abs(TT2.item() - TT.item()) <= 1e-12 * TT.item()
    assert int(step2.item()) == int(i.item()) == 2
    assert int(status.item()) & A.AST_ST_NONFINITE == 0
