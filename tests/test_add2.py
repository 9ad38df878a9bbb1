"""The add2 drop-in (ast_add2_raw, kernel.cu:1928-2291) against the
reference's own add2 compiled for the host: 20 launches + funk_time on a
96x12 planar grid with a random state, method 0 and method 1 (the
time-dependent inflow density), recorded in tests/golden/step_add2_m*.npz.
add2's flux rule is not symmetric (the left face of a cell takes HLL inside
the region, the right face of its neighbour HLLC): the drop-in evaluates
each cell's four faces from the cell, as the reference does.  Bar: relative
L-infinity 1e-10, the clock to 1e-12."""
import numpy as np
import pytest

import golden_configs as G
from asteriy_2d_gb300 import solver
from conftest import golden

pytestmark = pytest.mark.gpu
TOL = 1e-10


def rel_linf(a, b):
    return np.max(np.abs(a - b), axis=0) / np.maximum(np.max(np.abs(b), axis=0), 1e-300)


@pytest.mark.parametrize("method", [0, 1])
def test_add2_raw_matches_reference(method):
    import torch
    d = golden(f"step_add2_m{method}.npz")
    cfg = G.add2_config()
    dev = torch.device("cuda:0")
    a = [torch.tensor(d["s0"], device=dev), torch.tensor(d["u0"], device=dev)]
    b = [torch.empty_like(a[0]), torch.empty_like(a[1])]
    T = torch.tensor([1e7], dtype=torch.float64, device=dev)
    T_do = torch.tensor([cfg.dt_first], dtype=torch.float64, device=dev)
    TT = torch.zeros(1, dtype=torch.float64, device=dev)
    i = torch.zeros(1, dtype=torch.int32, device=dev)
    for _ in range(int(d["nsteps"])):
        solver.add2_raw(a[0].data_ptr(), a[1].data_ptr(), b[0].data_ptr(), b[1].data_ptr(), T.data_ptr(),
                        T_do.data_ptr(), TT.data_ptr(), cfg, method=method)
        solver.funk_time(T.data_ptr(), T_do.data_ptr(), TT.data_ptr(), i.data_ptr())
        a, b = b, a
    torch.cuda.synchronize()
    s, u = a[0].cpu().numpy(), a[1].cpu().numpy()
    es, eu = rel_linf(s, d["s"]), rel_linf(u, d["u"])
    assert np.all(es <= TOL) and np.all(eu <= TOL), (es, eu)
    assert int(i.item()) == int(d["steps"])
    assert abs(T_do.item() - float(d["T_do"])) <= 1e-12 * float(d["T_do"])
    assert abs(TT.item() - float(d["TT"])) <= 1e-12 * float(d["TT"])


def test_add2_raw_rejects_configurations_it_does_not_reproduce():
    import torch
    cfg = G.add2_config()
    dev = torch.device("cuda:0")
    x = torch.zeros((cfg.N * cfg.M, 2), dtype=torch.float64, device=dev)
    t = torch.zeros(1, dtype=torch.float64, device=dev)
    for field, value in (("recon", 1), ("geom", 1), ("precision", 1)):
        c = cfg.copy()
        setattr(c, field, value)
        with pytest.raises(solver.AstError):
            solver.add2_raw(x.data_ptr(), x.data_ptr(), x.data_ptr(), x.data_ptr(), t.data_ptr(), t.data_ptr(),
                            t.data_ptr(), c)
