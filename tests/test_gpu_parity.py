"""Parity of the CUDA step with the oracle (and through it, the reference).

FP64 bar: relative L-infinity error <= 1e-10 per variable after 100 steps
(max |gpu - oracle| / max |oracle|), shock positions identical to the cell,
and the clock (T_do, TT, step) equal to the oracle's to 1e-12 relative.
"""
import os

import numpy as np
import pytest

import golden_configs as G
import pyoracle as O
from asteriy_2d_gb300 import abi as A
from asteriy_2d_gb300 import problems, solver
from conftest import golden

pytestmark = pytest.mark.gpu
TOL = 1e-10
NT = os.cpu_count() or 1


def rel_linf(a, b):
    return np.max(np.abs(a - b), axis=0) / np.maximum(np.max(np.abs(b), axis=0), 1e-300)


def run_gpu(cfg, s0, u0, nsteps):
    with solver.Solver(cfg) as S:
        S.set_state(s0, u0)
        S.step(nsteps)
        s, u = S.get_state()
        clk = S.clock()
        st = S.stats()
    return s, u, clk, st


def assert_parity(cfg, s0, u0, nsteps, tol=TOL):
    s, u, (tdo, tt, step), _ = run_gpu(cfg, s0, u0, nsteps)
    os_, ou, otdo, ott, ost, _ = O.run(cfg, s0, u0, nsteps, nthreads=NT)
    es, eu = rel_linf(s, os_), rel_linf(u, ou)
    assert np.all(es <= tol) and np.all(eu <= tol), (es, eu)
    assert step == ost
    ctol = max(1e-12, 10 * tol if tol > TOL else 1e-12)
    assert abs(tdo - otdo) <= ctol * otdo and abs(tt - ott) <= ctol * ott, (tdo, otdo, tt, ott)
    return s, u, os_, ou


def jumps(s, cfg):
    rho = s[:, 0].reshape(cfg.M, cfg.N)
    return np.abs(np.diff(rho, axis=1))


def assert_same_shock_cells(s, o, cfg, tie=1e-8, strong=1e-2):
    """Per row of cells (fixed r) and per half of the domain (the blast has
    one shock on either side of z=0): (1) the outermost cell whose density
    departs from the ambient 1 by more than 1e-3 (the leading edge of the
    shock) is the same cell; (2) in rows with a real shock (largest jump
    above `strong`) the face with the largest density jump in the GPU result
    is also the largest jump of the oracle's, up to ties within `tie`
    relative (two adjacent faces with equal jumps)."""
    rg = s[:, 0].reshape(cfg.M, cfg.N)
    ro = o[:, 0].reshape(cfg.M, cfg.N)
    h = cfg.N // 2
    def edges(r):
        dev = np.abs(r - 1.0) > 1e-3
        left = np.where(dev[:, :h].any(1), np.argmax(dev[:, :h], axis=1), -1)
        right = np.where(dev[:, h:].any(1), cfg.N - 1 - np.argmax(dev[:, ::-1][:, :cfg.N - h], axis=1), -1)
        return left, right
    assert all(np.array_equal(a, b) for a, b in zip(edges(rg), edges(ro)))
    jg, jo = jumps(s, cfg), jumps(o, cfg)
    hj = jg.shape[1] // 2
    for lo, hi in ((0, hj), (hj, jg.shape[1])):
        ig = lo + np.argmax(jg[:, lo:hi], axis=1)
        mo = np.max(jo[:, lo:hi], axis=1)
        rows = np.nonzero(mo > strong)[0]
        assert np.all(jo[rows, ig[rows]] >= mo[rows] * (1 - tie)), rows[jo[rows, ig[rows]] < mo[rows] * (1 - tie)]


def test_blast_hll_minmod_fp64_256x128_100_steps():
    cfg = problems.blast_config(256, 128)
    s0, u0 = solver.fill_blast(cfg)
    s, u, os_, ou = assert_parity(cfg, s0, u0, 100)
    assert_same_shock_cells(s, os_, cfg)


def test_blast_hllc():
    cfg = problems.blast_config(128, 64, flux=A.FLUX_HLLC)
    s0, u0 = solver.fill_blast(cfg)
    s, u, os_, ou = assert_parity(cfg, s0, u0, 100)
    assert_same_shock_cells(s, os_, cfg)


@pytest.mark.parametrize("flux", [A.FLUX_HLLC, A.FLUX_GODUNOV])
def test_fp64_32x16_tile_path_matches_oracle(flux):
    # grids with at least two 32x16 tiles per SM step with 32x16 tiles;
    # smaller FP64 grids (every other parity case here) use 16x16 tiles
    cfg = problems.blast_config(640, 320, flux=flux)
    cfg.riemann_tol = 1e-13
    s0, u0 = solver.fill_blast(cfg)
    s, u, os_, ou = assert_parity(cfg, s0, u0, 30)
    assert_same_shock_cells(s, os_, cfg)


# The exact solver's shock-rarefaction bisection stops on an absolute
# residual of 10e-10 (devtwo, kernel.cu:685): which bisection iterate first
# meets it depends on the last bits of pow(), which differ between CUDA and
# glibc, so p* itself agrees only to about 1e-9 relative.  With the
# reference's tolerance the step agrees to TOL_GODUNOV; with a tight
# tolerance the same comparison meets the 1e-10 bar.
TOL_GODUNOV = 1e-9


@pytest.mark.parametrize("riemann_tol,tol", [(10e-10, TOL_GODUNOV), (1e-13, TOL)])
def test_blast_godunov(riemann_tol, tol):
    cfg = problems.blast_config(128, 64, flux=A.FLUX_GODUNOV)
    cfg.riemann_tol = riemann_tol
    s0, u0 = solver.fill_blast(cfg)
    s, u, os_, ou = assert_parity(cfg, s0, u0, 100, tol=tol)
    assert_same_shock_cells(s, os_, cfg)


def test_wind_counterflow_hllc_fixed_sphere():
    cfg = problems.wind_config(128, 64)
    s0, u0 = solver.fill_wind(cfg)
    assert_parity(cfg, s0, u0, 60)


@pytest.mark.parametrize("fname,cfg", [
    ("step_tvd.npz", G.tvd_config()),
    ("step_mk_hll.npz", G.add_mk_config(0)),
    ("step_mk_god.npz", G.add_mk_config(2)),
    ("step_mk_hllca.npz", G.add_mk_config(1)),
])
def test_reference_kernel_fixtures(fname, cfg):
    """Kernel_TVD and add_MK outputs recorded from the reference itself."""
    d = golden(fname)
    s, u, (tdo, tt, step), _ = run_gpu(cfg, d["s0"], d["u0"], int(d["nsteps"]))
    assert np.all(rel_linf(s, d["s"]) <= TOL) and np.all(rel_linf(u, d["u"]) <= TOL)
    assert step == int(d["steps"]) and abs(tdo - float(d["T_do"])) <= 1e-12 * float(d["T_do"])


@pytest.mark.parametrize("N,M", [(37, 21), (4, 4), (33, 17), (65, 5)])
def test_ragged_and_minimal_grids(N, M):
    cfg = problems.blast_config(N, M, flux=A.FLUX_HLLC)
    rng = np.random.default_rng(N * 100 + M)
    s0, u0 = G.random_state(N * M, rng)
    assert_parity(cfg, s0, u0, 20)


@pytest.mark.parametrize("geom", [A.GEOM_PLANAR, A.GEOM_AXISYM])
@pytest.mark.parametrize("kinds", [(A.BC_REFLECT,) * 4, (A.BC_SUCTION, A.BC_FIXED, A.BC_REFLECT, A.BC_OUTFLOW)])
def test_boundary_kinds(geom, kinds):
    cfg = problems.blast_config(48, 24, flux=A.FLUX_GODUNOV)
    cfg.riemann_tol = 1e-13
    cfg.geom = geom
    for side, kind in enumerate(kinds):
        A.set_bc(cfg, side, kind, 1.2, 3.0, -0.7, 0.1)
    rng = np.random.default_rng(7)
    s0, u0 = G.random_state(48 * 24, rng)
    assert_parity(cfg, s0, u0, 20)


def test_raw_drop_in_matches_oracle_over_steps():
    """ast_step_raw + ast_funk_time replace Kernel_TVD + funk_time in the
    reference's host loop (kernel.cu:3868-3947)."""
    import torch
    cfg = G.tvd_config()
    d = golden("step_tvd.npz")
    dev = torch.device("cuda:0")
    bufs = [torch.tensor(d["s0"], device=dev), torch.tensor(d["u0"], device=dev)]
    bufs2 = [torch.empty_like(bufs[0]), torch.empty_like(bufs[1])]
    T = torch.tensor([1e7], dtype=torch.float64, device=dev)
    T_do = torch.tensor([cfg.dt_first], dtype=torch.float64, device=dev)
    TT = torch.zeros(1, dtype=torch.float64, device=dev)
    i = torch.zeros(1, dtype=torch.int32, device=dev)
    for _ in range(int(d["nsteps"])):
        solver.step_raw(bufs[0].data_ptr(), bufs[1].data_ptr(), bufs2[0].data_ptr(), bufs2[1].data_ptr(),
                        T.data_ptr(), T_do.data_ptr(), TT.data_ptr(), cfg)
        solver.funk_time(T.data_ptr(), T_do.data_ptr(), TT.data_ptr(), i.data_ptr())
        bufs, bufs2 = bufs2, bufs
    torch.cuda.synchronize()
    s, u = bufs[0].cpu().numpy(), bufs[1].cpu().numpy()
    assert np.all(rel_linf(s, d["s"]) <= TOL) and np.all(rel_linf(u, d["u"]) <= TOL)
    assert int(i.item()) == int(d["steps"]) and T.item() == 1e7
    assert abs(T_do.item() - float(d["T_do"])) <= 1e-12 * float(d["T_do"])


def test_deterministic_bitwise():
    cfg = problems.blast_config(96, 48, flux=A.FLUX_GODUNOV)
    s0, u0 = solver.fill_blast(cfg)
    a = run_gpu(cfg, s0, u0, 30)
    b = run_gpu(cfg, s0, u0, 30)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[2] == b[2]


def test_mass_conserved_in_closed_planar_box():
    cfg = problems.blast_config(64, 64, flux=A.FLUX_HLLC)
    cfg.geom = A.GEOM_PLANAR
    for side in range(4):
        A.set_bc(cfg, side, A.BC_REFLECT)
    s0, u0 = solver.fill_blast(cfg)
    s, u, _, _ = run_gpu(cfg, s0, u0, 200)
    assert abs(s[:, 0].sum() - s0[:, 0].sum()) <= 1e-12 * s0[:, 0].sum()


@pytest.mark.parametrize("flux", [A.FLUX_HLL, A.FLUX_HLLC, A.FLUX_GODUNOV])
def test_energy_and_mass_conserved_in_closed_planar_box(flux):
    # reflecting walls on all sides: no mass or energy crosses the boundary
    # (the walls' pressure changes the momentum, not the energy)
    cfg = problems.blast_config(96, 64, flux=flux)
    cfg.geom = A.GEOM_PLANAR
    for side in range(4):
        A.set_bc(cfg, side, A.BC_REFLECT)
    s0, u0 = solver.fill_blast(cfg)
    s, u, _, st = run_gpu(cfg, s0, u0, 150)
    assert st["rho_floor"] == 0 and st["p_floor"] == 0

    def totals(s, u):
        e = s[:, 1] / (cfg.gamma - 1.0) + 0.5 * s[:, 0] * (u[:, 0] ** 2 + u[:, 1] ** 2)
        return s[:, 0].sum(), e.sum()

    (m0, e0), (m1, e1) = totals(s0, u0), totals(s, u)
    assert abs(m1 - m0) <= 1e-12 * m0 and abs(e1 - e0) <= 1e-11 * e0, (m1 - m0, e1 - e0)


@pytest.mark.parametrize("precision,tol", [(A.PREC_FP64, 1e-11), (A.PREC_FP32, 1e-5)])
@pytest.mark.parametrize("flux", [A.FLUX_HLL, A.FLUX_HLLC, A.FLUX_GODUNOV])
def test_blast_mirror_symmetric_about_z0(flux, precision, tol):
    # the blast sits at z = 0 of z in [-1, 1]: the solution is even in z
    # (rho, p, v_r) and odd (v_z); every face is evaluated once in the +z
    # frame, so this checks the fluxes under reversal of the normal.  The
    # exact solver's FP64 iteration stops at the reference's absolute
    # tolerance, so mirrored faces agree to its parity bar (1e-9)
    if flux == A.FLUX_GODUNOV and precision == A.PREC_FP64:
        tol = TOL_GODUNOV
    cfg = problems.blast_config(128, 64, flux=flux, precision=precision)
    s0, u0 = solver.fill_blast(cfg)
    s, u, _, _ = run_gpu(cfg, s0, u0, 100)
    sg, ug = s.reshape(cfg.M, cfg.N, 2), u.reshape(cfg.M, cfg.N, 2)
    sm, um = sg[:, ::-1, :], ug[:, ::-1, :]
    scale = np.max(np.abs(sg), axis=(0, 1))
    assert np.all(np.max(np.abs(sg - sm), axis=(0, 1)) <= tol * scale)
    vscale = np.max(np.abs(ug), axis=(0, 1))
    assert np.max(np.abs(ug[..., 0] + um[..., 0])) <= tol * vscale[0]
    assert np.max(np.abs(ug[..., 1] - um[..., 1])) <= tol * vscale[1]


def test_graph_block_and_single_steps_agree():
    cfg = problems.blast_config(64, 32)
    s0, u0 = solver.fill_blast(cfg)
    with solver.Solver(cfg) as S:
        S.set_state(s0, u0)
        S.step(37)
        a = S.get_state()
    with solver.Solver(cfg) as S:
        S.set_state(s0, u0)
        for _ in range(37):
            S.step(1)
        b = S.get_state()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_stats_count_riemann_work():
    cfg = problems.blast_config(64, 32, flux=A.FLUX_GODUNOV)
    cfg.collect_stats = 1
    s0, u0 = solver.fill_blast(cfg)
    _, _, _, st = run_gpu(cfg, s0, u0, 20)
    assert st["newton_calls"] + st["bisect_calls"] > 0 and st["newton_max_iters"] >= 1
    assert st["status"] & A.AST_ST_NONFINITE == 0


def test_fp64_safeguarded_newton_matches_oracle():
    """The Newton iteration used by the learned form, in FP64, converges to
    the reference's p*: with tight tolerances the step agrees to 1e-10."""
    cfg = problems.blast_config(128, 64, flux=A.FLUX_GODUNOV)
    cfg.riemann_tol = 1e-13
    gpu = cfg.copy()
    gpu.riemann_newton = 1
    s0, u0 = solver.fill_blast(cfg)
    s, u, _, _ = run_gpu(gpu, s0, u0, 100)
    os_, ou, *_ = O.run(cfg, s0, u0, 100, nthreads=NT)
    assert np.all(rel_linf(s, os_) <= TOL) and np.all(rel_linf(u, ou) <= TOL)


@pytest.mark.parametrize("flux", [A.FLUX_HLL, A.FLUX_GODUNOV])
def test_fp32_form_error_against_fp64_oracle(flux):
    """Precision form: FP32 state and fluxes, FP64 in the near-axis update,
    in high-Mach pressure recovery and in the dt reduction.  Density L1
    error relative to the FP64 oracle stays below 1e-4 after 100 steps."""
    cfg = problems.blast_config(256, 128, flux=flux, precision=A.PREC_FP32)
    s0, u0 = solver.fill_blast(cfg)
    s, u, (tdo, tt, step), _ = run_gpu(cfg, s0, u0, 100)
    ref = problems.blast_config(256, 128, flux=flux)
    os_, ou, otdo, ott, ost, _ = O.run(ref, s0, u0, 100, nthreads=NT)
    l1_rho = np.sum(np.abs(s[:, 0] - os_[:, 0])) / np.sum(np.abs(os_[:, 0]))
    l1_p = np.sum(np.abs(s[:, 1] - os_[:, 1])) / np.sum(np.abs(os_[:, 1]))
    assert l1_rho < 1e-4 and l1_p < 1e-4, (l1_rho, l1_p)
    assert step == ost and abs(tt - ott) < 1e-4 * ott


@pytest.mark.parametrize("precision", [A.PREC_FP64, A.PREC_FP32])
def test_probe_matches_state(precision):
    cfg = problems.blast_config(64, 32, precision=precision)
    s0, u0 = solver.fill_blast(cfg)
    with solver.Solver(cfg) as S:
        S.set_state(s0, u0)
        S.step(30)
        cells = [0, 5, 64 * 10 + 7, 64 * 32 - 1]
        rho, tt = S.probe(cells)
        s, _ = S.get_state()
        assert np.array_equal(rho, s[cells, 0])
        assert tt == S.clock()[1]
        with pytest.raises(solver.AstError):
            S.probe([64 * 32])


def test_characteristic_inflow_matches_oracle():
    """Kernel_TVD's problem with add2_bound after every step (p_H = 7,
    inflow speed 1): the solver against the oracle's step + inflow."""
    d = golden("step_tvd.npz")
    cfg = G.tvd_config()
    cfg.inflow_p, cfg.inflow_v = 7.0, 1.0
    s, u, os_, ou = assert_parity(cfg, d["s0"], d["u0"], 40)
    assert np.all(os_[0::cfg.N, 1] == 7.0) and np.all(s[0::cfg.N, 1] == 7.0)
    c32 = cfg.copy()
    c32.precision = A.PREC_FP32
    s32, *_ = run_gpu(c32, d["s0"], d["u0"], 40)
    assert np.max(np.abs(s32 - os_)) / np.max(np.abs(os_)) < 1e-4


def test_inflow_raw_drop_in_matches_oracle():
    import torch
    z = golden("inflow.npz")
    cfg = G.inflow_config()
    dev = torch.device("cuda:0")
    t = {k: torch.tensor(z[k], device=dev) for k in ("s", "u", "s2", "u2")}
    solver.inflow_raw(t["s"].data_ptr(), t["u"].data_ptr(), t["s2"].data_ptr(), t["u2"].data_ptr(), cfg)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(t["s2"].cpu().numpy(), z["s2_out"])
    np.testing.assert_array_equal(t["u2"].cpu().numpy(), z["u2_out"])


@pytest.mark.parametrize("flux", [A.FLUX_HLL, A.FLUX_GODUNOV])
def test_nonreflecting_sides_match_oracle(flux):
    cfg = problems.blast_config(128, 64, flux=flux)
    A.set_bc(cfg, A.Z_LO, A.BC_NONREFLECT)
    A.set_bc(cfg, A.Z_HI, A.BC_NONREFLECT)
    A.set_bc(cfg, A.R_HI, A.BC_NONREFLECT)
    s0, u0 = solver.fill_blast(cfg, radius=0.7)
    tol = TOL_GODUNOV if flux == A.FLUX_GODUNOV else TOL
    assert_parity(cfg, s0, u0, 100, tol=tol)
    c32 = cfg.copy()
    c32.precision = A.PREC_FP32
    for persistent in (0, 1):
        c32.persistent = persistent
        s32, *_ = run_gpu(c32, s0, u0, 100)
        assert np.all(np.isfinite(s32))


@pytest.mark.parametrize("precision", [A.PREC_FP64, A.PREC_FP32])
def test_hllc_aleksashov_blast(precision):
    """The second HLLC with minmod on the small blast: FP64 at the parity
    bar, FP32 (persistent and per-tile kernels) within the FP32 form's
    error of the oracle."""
    cfg = problems.blast_config(256, 128, flux=A.FLUX_HLLC_A, precision=precision)
    s0, u0 = solver.fill_blast(cfg)
    if precision == A.PREC_FP64:
        s, u, os_, ou = assert_parity(cfg, s0, u0, 100)
        assert_same_shock_cells(s, os_, cfg)
        return
    os_, *_ = O.run(cfg, s0, u0, 100, nthreads=NT)
    for persistent in (1, 0):
        cfg.persistent = persistent
        s, *_ = run_gpu(cfg, s0, u0, 100)
        l1 = np.sum(np.abs(s[:, 0] - os_[:, 0])) / np.sum(np.abs(os_[:, 0]))
        assert l1 < 1e-5, (persistent, l1)
