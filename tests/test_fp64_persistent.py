"""The FP64 solver's persistent tile kernel (the HLL family on grids of at
least two 32x16 tiles per SM): the same bits as one CTA per tile, through
ast_step and through the banded host-array step, and the oracle at 1e-10."""
import os

import numpy as np
import pytest

import pyoracle as O
from asteriy_2d_gb300 import abi as A
from asteriy_2d_gb300 import problems, solver

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 1


def run(cfg, s0, u0, n):
    with solver.Solver(cfg) as S:
        S.set_state(s0, u0)
        S.step(n)
        return S.get_state(), S.clock()


@pytest.mark.parametrize("flux", [A.FLUX_HLL, A.FLUX_HLLC, A.FLUX_HLLC_A, A.FLUX_HLLCQ])
def test_fp64_persistent_equals_per_tile(flux):
    cfg = problems.blast_config(1280, 256, flux=flux)   # 40 x 16 = 640 tiles of 32x16
    s0, u0 = solver.fill_blast(cfg, radius=0.3)
    (s, u), clk = run(cfg, s0, u0, 24)
    c0 = cfg.copy()
    c0.persistent = 0
    (rs, ru), rclk = run(c0, s0, u0, 24)
    assert np.array_equal(s, rs) and np.array_equal(u, ru) and clk == rclk


def test_fp64_persistent_host_steps_and_oracle():
    cfg = problems.blast_config(1280, 256, flux=A.FLUX_HLLC)
    s0, u0 = solver.fill_blast(cfg, radius=0.3)
    (s, u), (tdo, tt, st) = run(cfg, s0, u0, 3)
    # the banded host-array step (page-locked arrays) gives the same bits
    torch = pytest.importorskip("torch")
    K = cfg.N * cfg.M
    sa, ua, sb, ub = (torch.zeros((K, 2), dtype=torch.float64, pin_memory=True) for _ in range(4))
    sa.numpy()[:] = s0
    ua.numpy()[:] = u0
    with solver.Solver(cfg) as S:
        S.step_host_n(3, sa.data_ptr(), ua.data_ptr(), sb.data_ptr(), ub.data_ptr())
    assert np.array_equal(sb.numpy(), s) and np.array_equal(ub.numpy(), u)
    os_, ou, otdo, ott, ost, _ = O.run(cfg, s0, u0, 3, nthreads=NT)
    err = np.max(np.abs(s - os_), axis=0) / np.max(np.abs(os_), axis=0)
    assert np.all(err <= 1e-10), err
