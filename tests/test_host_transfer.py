"""ast_set_state / ast_get_state with host arrays: page-locked arrays are
read and written in place by the conversion kernels, pageable ones go
through the device staging buffers.  Both must give the same state, bit for
bit, in both precisions, also for arrays that start inside a larger
page-locked allocation."""
import ctypes as C

import numpy as np
import pytest

from asteriy_2d_gb300 import abi as A
from asteriy_2d_gb300 import problems, solver

pytestmark = pytest.mark.gpu


def pinned(a):
    torch = pytest.importorskip("torch")
    t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
    t.numpy()[:] = a
    return t


@pytest.mark.parametrize("precision", [A.PREC_FP32, A.PREC_FP64])
def test_pinned_and_pageable_transfers_agree(precision):
    cfg = problems.blast_config(300, 130, flux=A.FLUX_HLLC, precision=precision)
    s0, u0 = solver.fill_blast(cfg)
    u0[:, 0] = np.linspace(-0.3, 0.4, len(u0))
    lib = solver.load()
    with solver.Solver(cfg) as S:
        # pageable in, pageable out
        S.set_state(s0, u0)
        S.step(7)
        s_a, u_a = S.get_state()
        # page-locked in, page-locked out
        ps, pu = pinned(s0), pinned(u0)
        S.set_clock(cfg.dt_first, 0.0, 0)
        solver.check(lib.ast_set_state(S.h, ps.data_ptr(), pu.data_ptr(), 0), "set_state")
        S.step(7)
        solver.check(lib.ast_get_state(S.h, ps.data_ptr(), pu.data_ptr(), 0), "get_state")
        S.synchronize()
        s_b, u_b = ps.numpy().copy(), pu.numpy().copy()
        # page-locked in, pageable out, and the reverse
        S.set_clock(cfg.dt_first, 0.0, 0)
        ps.numpy()[:] = s0
        pu.numpy()[:] = u0
        solver.check(lib.ast_set_state(S.h, ps.data_ptr(), pu.data_ptr(), 0), "set_state")
        S.step(7)
        s_c, u_c = S.get_state()
    assert np.array_equal(s_a, s_b) and np.array_equal(u_a, u_b)
    assert np.array_equal(s_a, s_c) and np.array_equal(u_a, u_c)


def test_round_trip_through_pinned_arrays():
    cfg = problems.blast_config(97, 45, precision=A.PREC_FP64)
    rng = np.random.default_rng(3)
    s0 = rng.uniform(0.5, 2.0, (cfg.N * cfg.M, 2))
    u0 = rng.uniform(-1.0, 1.0, (cfg.N * cfg.M, 2))
    lib = solver.load()
    with solver.Solver(cfg) as S:
        ps, pu = pinned(s0), pinned(u0)
        solver.check(lib.ast_set_state(S.h, ps.data_ptr(), pu.data_ptr(), 0), "set_state")
        ps.numpy()[:] = 0.0
        pu.numpy()[:] = 0.0
        solver.check(lib.ast_get_state(S.h, ps.data_ptr(), pu.data_ptr(), 0), "get_state")
        assert np.array_equal(ps.numpy(), s0) and np.array_equal(pu.numpy(), u0)


def test_pinned_array_inside_a_larger_allocation():
    # the arrays start inside one page-locked allocation and end before its
    # end: read in place from their own offsets
    torch = pytest.importorskip("torch")
    cfg = problems.blast_config(64, 32, precision=A.PREC_FP64)
    K = cfg.N * cfg.M
    s0, u0 = solver.fill_blast(cfg)
    big = torch.zeros((3 * K + 8, 2), dtype=torch.float64, pin_memory=True)
    big.numpy()[4:4 + K] = s0
    big.numpy()[4 + K:4 + 2 * K] = u0
    lib = solver.load()
    with solver.Solver(cfg) as S:
        base = big.data_ptr() + 4 * 16
        solver.check(lib.ast_set_state(S.h, base, base + K * 16, 0), "set_state")
        S.synchronize()
        s, u = S.get_state()
        assert np.array_equal(s, s0) and np.array_equal(u, u0)
