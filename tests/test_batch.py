"""Batched problems: the seeded problem set (host, no GPU) and the batch
solver, whose every problem must evolve as the same problem does in its own
single-problem solver (the same device code compiled into another kernel:
the compiler may fuse a multiply and an add differently, so agreement is to
rounding, not bitwise), and whose FP64 problems match the oracle."""
import os

import numpy as np
import pytest

from asteriy_2d_gb300 import abi as A
from asteriy_2d_gb300 import solver


# ---------------------------------------------------------------- host side
def test_problem_set_is_seeded_and_in_range():
    a = solver.problem_set(64, 64)
    b = solver.problem_set(64, 64)
    c = solver.problem_set(65, 64)
    key = lambda ps: [(p.cfg.N, p.cfg.M, p.mach, p.cfg.gamma, p.setup, p.cfg.flux, p.seed) for p in ps]
    assert key(a) == key(b)
    assert key(a) != key(c)
    lib = solver.load()
    import ctypes as C
    for p in a:
        assert p.cfg.N == 2 * p.cfg.M and 64 <= p.cfg.M <= 512
        assert 1.5 <= p.mach <= 6.0
        assert p.cfg.gamma in (5.0 / 3.0, 1.4)
        assert p.setup in (A.SETUP_BLAST, A.SETUP_WIND)
        assert p.cfg.flux in (A.FLUX_HLLC, A.FLUX_GODUNOV)
        assert p.cfg.precision == A.PREC_FP32
        assert (p.cfg.cfl, p.cfg.recon, p.cfg.geom) == (0.4, A.RECON_MINMOD, A.GEOM_AXISYM)
        assert lib.ast_config_check(C.byref(p.cfg)) == A.AST_OK
        if p.setup == A.SETUP_WIND:
            bc = p.cfg.bc[A.Z_HI]
            assert (bc.kind, bc.rho, bc.p, bc.vz) == (A.BC_FIXED, 1.0, 1.0 / p.cfg.gamma, -p.mach)
            assert p.cfg.fixed_region == 1
        else:
            assert p.cfg.bc[A.Z_HI].kind == A.BC_OUTFLOW and p.cfg.fixed_region == 0
    # both setups, both fluxes and both gases occur; sizes span the range
    assert {p.setup for p in a} == {A.SETUP_BLAST, A.SETUP_WIND}
    assert {p.cfg.flux for p in a} == {A.FLUX_HLLC, A.FLUX_GODUNOV}
    assert {p.cfg.gamma for p in a} == {5.0 / 3.0, 1.4}
    Ms = [p.cfg.M for p in a]
    assert min(Ms) < 100 and max(Ms) > 350
    # the FP64 set is the same draw
    d = solver.problem_set(64, 64, A.PREC_FP64)
    assert [k[:-1] for k in key(d)] == [k[:-1] for k in key(a)]
    assert all(p.cfg.precision == A.PREC_FP64 for p in d)


def test_problem_fill_states():
    ps = solver.problem_set(64, 64)
    blast = next(p for p in ps if p.setup == A.SETUP_BLAST)
    s, u = solver.problem_fill(blast)
    g, m2 = blast.cfg.gamma, blast.mach ** 2
    p_in = 0.1 * (2 * g * m2 - (g - 1)) / (g + 1)
    assert np.all(s[:, 0] == 1.0) and np.all(u == 0.0)
    assert set(np.unique(s[:, 1])) == {0.1, p_in}
    wind = next(p for p in ps if p.setup == A.SETUP_WIND)
    s, u = solver.problem_fill(wind)
    ref_s, ref_u = solver.fill_wind(wind.cfg, v_inf=-wind.mach, seed=wind.seed)
    assert np.array_equal(s, ref_s) and np.array_equal(u, ref_u)
    far = np.abs(s[:, 0] - 1.0) <= 0.01 + 1e-15
    assert far.mean() > 0.9 and np.all(u[far, 0] == -wind.mach)


def test_batch_rejects_bad_sets():
    import ctypes as C
    lib = solver.load()
    ps = solver.problem_set(64, 2)
    arr = (A.ast_config * 2)(ps[0].cfg, ps[1].cfg)
    arr[1].precision = A.PREC_FP64
    h = C.c_void_p()
    assert lib.ast_batch_create(arr, 2, C.byref(h)) == A.AST_ERR_INVALID
    arr[1].precision = A.PREC_FP32
    arr[1].gamma = 1.0
    assert lib.ast_batch_create(arr, 2, C.byref(h)) == A.AST_ERR_INVALID
    assert lib.ast_batch_create(arr, 0, C.byref(h)) == A.AST_ERR_INVALID


# ---------------------------------------------------------------- GPU
def small_set(precision, n=8, max_m=96, seed=64):
    """The first n problems of the seeded set, shrunk to at most
    2*max_m x max_m cells so that every test stays fast."""
    out = []
    for p in solver.problem_set(seed, 64, precision):
        if len(out) == n:
            break
        p.cfg.M = min(p.cfg.M, max_m)
        p.cfg.N = 2 * p.cfg.M
        out.append(p)
    return out


# batch vs single-problem solver after a few dozen steps: relative
# L-infinity per variable, and the clock (T_do, TT) relative
AGREE = {A.PREC_FP64: (1e-11, 1e-13), A.PREC_FP32: (1e-5, 1e-6)}


def assert_agree(prec, got, ref, clock, rclock, what):
    tol, ctol = AGREE[prec]
    for g, r in zip(got, ref):
        err = np.max(np.abs(g - r), axis=0) / np.maximum(np.max(np.abs(r), axis=0), 1e-300)
        assert np.all(err <= tol), (what, err)
    assert clock[2] == rclock[2], what
    assert abs(clock[0] - rclock[0]) <= ctol * rclock[0] and abs(clock[1] - rclock[1]) <= ctol * rclock[1], \
        (what, clock, rclock)


def single_run(cfg, s0, u0, steps, params=None):
    with solver.Solver(cfg) as S:
        if params is not None:
            S.set_mlp(params)
        S.set_state(s0, u0)
        S.step(steps)
        s, u = S.get_state()
        return s, u, S.clock()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [A.PREC_FP64, A.PREC_FP32])
def test_batch_matches_single_solvers(precision):
    probs = small_set(precision)
    # odd sizes as well (ragged tiles), and an HLL member
    probs[0].cfg.N, probs[0].cfg.M = 150, 70
    probs[1].cfg.flux = A.FLUX_HLL
    cfgs = [p.cfg for p in probs]
    init = [solver.problem_fill(p) for p in probs]
    steps = 37      # two captured blocks of 16 and five single steps
    with solver.Batch(cfgs) as B:
        info = B.info()
        assert info["cells"] == sum(c.N * c.M for c in cfgs)
        assert info["launches_per_step"] == len({(c.flux, c.recon) for c in cfgs})
        for i, (s0, u0) in enumerate(init):
            B.set_state(i, s0, u0)
        B.step(16)
        B.step(steps - 16)
        for i, c in enumerate(cfgs):
            s, u = B.get_state(i)
            rs, ru, rclock = single_run(c, *init[i], steps)
            assert_agree(precision, (s, u), (rs, ru), B.clock(i), rclock, i)


@pytest.mark.gpu
def test_batch_fp64_matches_oracle():
    import pyoracle as O
    probs = small_set(A.PREC_FP64, n=4, max_m=48)
    cfgs = [p.cfg for p in probs]
    init = [solver.problem_fill(p) for p in probs]
    steps = 20
    with solver.Batch(cfgs) as B:
        for i, (s0, u0) in enumerate(init):
            B.set_state(i, s0, u0)
        B.step(steps)
        for i, c in enumerate(cfgs):
            s, u = B.get_state(i)
            os_, ou, T_do, TT = O.run(c, *init[i], steps, nthreads=os.cpu_count() or 1)[:4]
            # the bars of the single-problem parity tests: 1e-10 relative
            # L-infinity per variable, 1e-9 for the exact solver at the
            # reference's absolute bisection tolerance
            tol = 1e-9 if c.flux == A.FLUX_GODUNOV else 1e-10
            for got, ref in ((s, os_), (u, ou)):
                err = np.max(np.abs(got - ref), axis=0) / np.maximum(np.max(np.abs(ref), axis=0), 1e-300)
                assert np.all(err <= tol), (i, c.flux, err)
            assert abs(B.clock(i)[1] - TT) <= 10 * tol * TT


@pytest.mark.gpu
def test_batch_clocks_are_per_problem():
    probs = small_set(A.PREC_FP32, n=3)
    cfgs = [p.cfg for p in probs]
    with solver.Batch(cfgs) as B:
        for i, p in enumerate(probs):
            B.set_state(i, *solver.problem_fill(p))
        B.set_clock(1, 1e-6, 5.0, 100)
        B.step(3)
        t0, t1 = B.clock(0), B.clock(1)
        assert t0[2] == 3 and t1[2] == 103
        assert t1[1] > 5.0 and t0[1] < 1.0
        assert t0[0] != t1[0]


@pytest.mark.gpu
def test_batch_stats_and_learned_guess():
    probs = [p for p in small_set(A.PREC_FP32, n=16) if p.cfg.flux == A.FLUX_GODUNOV][:3]
    assert probs
    params = np.load(os.path.join(os.path.dirname(solver.__file__), "data", "guess_blast.npy"))
    cfgs = []
    for p in probs:
        c = p.cfg.copy()
        c.guess, c.collect_stats, c.riemann_tol = A.GUESS_MLP, 1, 1e-8
        cfgs.append(c)
    init = [solver.problem_fill(p) for p in probs]
    with solver.Batch(cfgs) as B:
        with pytest.raises(solver.AstError):
            B.step(1)
        B.set_mlp(params)
        for i, (s0, u0) in enumerate(init):
            B.set_state(i, s0, u0)
        B.step(40)
        for i, c in enumerate(cfgs):
            st = B.stats(i)
            assert st["newton_calls"] > 0
            assert st["mlp_fallback"] <= st["strong_calls"]
            s, u = B.get_state(i)
            rs, ru, rclock = single_run(c, *init[i], 40, params)
            assert_agree(A.PREC_FP32, (s, u), (rs, ru), B.clock(i), rclock, i)


@pytest.mark.gpu
@pytest.mark.parametrize("schedule", range(len(solver.SCHEDULES)))
def test_batch_schedules_agree(schedule):
    """Every schedule (one CTA per tile with each tile shape, the persistent
    kernel) gives the single-problem results, on ragged and tiny grids."""
    probs = small_set(A.PREC_FP32, n=6)
    probs[0].cfg.N, probs[0].cfg.M = 150, 70
    probs[1].cfg.N, probs[1].cfg.M = 33, 17
    probs[2].cfg.flux = A.FLUX_HLLC_A
    cfgs = [p.cfg for p in probs]
    init = [solver.problem_fill(p) for p in probs]
    with solver.Batch(cfgs) as B:
        assert all(c["schedule"] == solver.PERSISTENT for c in B.classes())   # the FP32 default
        for k in range(B.info()["launches_per_step"]):
            B.set_schedule(k, schedule)
        assert all(c["schedule"] == schedule for c in B.classes())
        if schedule < len(solver.TILE_SHAPES):
            assert all(c["tile"] == solver.TILE_SHAPES[schedule] for c in B.classes())
        for i, (s0, u0) in enumerate(init):
            B.set_state(i, s0, u0)
        B.step(21)
        for i, c in enumerate(cfgs):
            rs, ru, rclock = single_run(c, *init[i], 21)
            assert_agree(A.PREC_FP32, B.get_state(i), (rs, ru), B.clock(i), rclock, (schedule, i))
    with solver.Batch(cfgs[:1]) as B:
        with pytest.raises(solver.AstError):
            B.set_tiles(0, 8, 8)
    c64 = cfgs[0].copy()
    c64.precision = A.PREC_FP64
    with solver.Batch([c64]) as B:
        assert B.classes()[0]["schedule"] == 0
        with pytest.raises(solver.AstError):
            B.set_schedule(0, solver.PERSISTENT)


@pytest.mark.gpu
def test_autotune_leaves_the_run_unchanged():
    probs = small_set(A.PREC_FP32, n=6)
    cfgs = [p.cfg for p in probs]
    init = [solver.problem_fill(p) for p in probs]
    with solver.Batch(cfgs) as T, solver.Batch(cfgs) as U:
        for Bt in (T, U):
            for i, (s0, u0) in enumerate(init):
                Bt.set_state(i, s0, u0)
            Bt.step(10)
        before = [(T.get_state(i), T.clock(i), T.stats(i)) for i in range(len(cfgs))]
        classes = T.autotune(2)
        for c in classes:
            assert c["tile"] in solver.TILE_SHAPES
            assert all(ms > 0 for ms in c["ms_per_schedule"])
            assert min(c["ms_per_schedule"]) == c["ms_per_schedule"][c["schedule"]]
        for i in range(len(cfgs)):
            s, u = T.get_state(i)
            assert np.array_equal(s, before[i][0][0]) and np.array_equal(u, before[i][0][1])
            assert T.clock(i) == before[i][1] and T.stats(i) == before[i][2]
        T.step(20)
        U.step(20)
        for i in range(len(cfgs)):
            assert_agree(A.PREC_FP32, T.get_state(i), U.get_state(i), T.clock(i), U.clock(i), i)


@pytest.mark.gpu
def test_one_launch_mode():
    """Every problem in one launch, with a CTA per tile (mode 1) and with the
    persistent kernel (mode 2; tiles from one counter, staged by bulk-tensor
    copies): each tile stepped by the tile code of its problem's flux, as
    schedule 0 of every class steps it, bit for bit."""
    probs = small_set(A.PREC_FP32, n=7)
    probs[0].cfg.N, probs[0].cfg.M = 150, 70
    probs[1].cfg.N, probs[1].cfg.M = 33, 17
    probs[2].cfg.flux = A.FLUX_HLLC_A
    probs[3].cfg.flux = A.FLUX_HLL
    cfgs = [p.cfg for p in probs]
    init = [solver.problem_fill(p) for p in probs]
    states = []
    for mode in (1, 2, 0):
        with solver.Batch(cfgs) as B:
            if mode:
                B.set_mixed(mode)
                assert B.info()["launches_per_step"] == 1 and B.mixed()[0] == mode
            else:
                for k in range(B.info()["launches_per_step"]):
                    B.set_schedule(k, 0)
            for i, (s0, u0) in enumerate(init):
                B.set_state(i, s0, u0)
            B.step(21)
            states.append([(B.get_state(i), B.clock(i)) for i in range(len(cfgs))])
    for run in states[:2]:
        bitwise = True
        for i in range(len(cfgs)):
            (s, u), clk = run[i]
            (rs, ru), rclk = states[2][i]
            assert_agree(A.PREC_FP32, (s, u), (rs, ru), clk, rclk, i)
            bitwise = bitwise and np.array_equal(s, rs) and np.array_equal(u, ru) and clk == rclk
        # the same tile code for each flux as schedule 0's kernels
        assert bitwise
    # the tuner times both ways and keeps the faster
    with solver.Batch(cfgs) as B:
        for i, (s0, u0) in enumerate(init):
            B.set_state(i, s0, u0)
        B.autotune(2)
        on, ms_mixed, ms_split = B.mixed()
        assert ms_mixed > 0 and ms_split > 0 and bool(on) == (ms_mixed < ms_split)
        assert B.info()["launches_per_step"] == (1 if on else B.lib.ast_batch_num_classes(B.h))
    # FP64 batches, and problems of different reconstructions, keep one
    # launch per class
    c64 = [c.copy() for c in cfgs[:2]]
    for c in c64:
        c.precision = A.PREC_FP64
    with solver.Batch(c64) as B:
        with pytest.raises(solver.AstError):
            B.set_mixed(True)
    two = [cfgs[0].copy(), cfgs[1].copy()]
    two[1].recon = A.RECON_NONE
    with solver.Batch(two) as B:
        with pytest.raises(solver.AstError):
            B.set_mixed(True)


@pytest.mark.gpu
def test_one_launch_mode_with_learned_guess():
    """The mixed kernel with exact-Godunov problems on the learned start
    value next to HLLC problems: bit for bit schedule 0, counters included."""
    probs = small_set(A.PREC_FP32, n=8)
    params = np.load(os.path.join(os.path.dirname(solver.__file__), "data", "guess_blast.npy"))
    cfgs = []
    for p in probs:
        c = p.cfg.copy()
        c.collect_stats = 1
        if c.flux == A.FLUX_GODUNOV:
            c.guess, c.riemann_tol = A.GUESS_MLP, 1e-8
        cfgs.append(c)
    assert any(c.guess == A.GUESS_MLP for c in cfgs) and any(c.flux == A.FLUX_HLLC for c in cfgs)
    init = [solver.problem_fill(p) for p in probs]
    out = []
    for mode in (1, 2, 0):
        with solver.Batch(cfgs) as B:
            B.set_mlp(params)
            if mode:
                B.set_mixed(mode)
            else:
                for k in range(B.lib.ast_batch_num_classes(B.h)):
                    B.set_schedule(k, 0)
            for i, (s0, u0) in enumerate(init):
                B.set_state(i, s0, u0)
            B.step(18)
            out.append([(B.get_state(i), B.clock(i), B.stats(i)) for i in range(len(cfgs))])
    for run in out[:2]:
        for i in range(len(cfgs)):
            (s, u), clk, st = run[i]
            (rs, ru), rclk, rst = out[2][i]
            assert np.array_equal(s, rs) and np.array_equal(u, ru) and clk == rclk and st == rst, i


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["persistent", "one_launch"])
def test_persistent_batch_single_and_tiny_problems(mode):
    """The persistent batch kernel on edge cases of its work list: a batch of
    one problem, and a problem of a single tile beside a larger one (more
    CTAs claim than there are tiles; the last CTA to leave shifts every
    clock and rewinds the counter), stepped over several graph blocks."""
    probs = small_set(A.PREC_FP32, n=2)
    probs[1].cfg.N, probs[1].cfg.M = 20, 10        # one 32x16 tile
    for cfgs_idx in ([0], [0, 1], [1]):
        cfgs = [probs[i].cfg for i in cfgs_idx]
        init = [solver.problem_fill(probs[i]) for i in cfgs_idx]
        with solver.Batch(cfgs) as B:
            if mode == "persistent":
                for k in range(B.info()["launches_per_step"]):
                    B.set_schedule(k, solver.PERSISTENT)
            else:
                B.set_mixed(2)
            for i, (s0, u0) in enumerate(init):
                B.set_state(i, s0, u0)
            B.step(37)
            for i, c in enumerate(cfgs):
                rs, ru, rclock = single_run(c, *init[i], 37)
                assert_agree(A.PREC_FP32, B.get_state(i), (rs, ru), B.clock(i), rclock, (mode, cfgs_idx, i))
