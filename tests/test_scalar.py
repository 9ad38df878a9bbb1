"""The passive scalar and the HLLCQ flux.

The reference's HLLC solvers compute a passive scalar's face flux beside the
gas flux: the Q channel of HLLC_2d_Korolkov_b_s (Gas_Dinamic.cu:1604-1811,
metod 2) and HLLCQ_Korolkov_2D (Gas_Dinamic.cu:249-353); its steps never
carry one.  Pinned here:
  - the oracle's restatement of both face functions against the reference's
    own functions compiled for the host (tests/golden/faces_scalar.npz), bit
    for bit;
  - the oracle's scalar step against the same step loop with every face by
    the reference's functions (step_scalar_*.npz), bit for bit;
  - the CUDA path (the FP64 solver with ast_set_scalar; the HLLCQ gas flux)
    against the oracle at 1e-10, and two properties of a passive scalar: a
    scalar proportional to the density stays so, and its total is conserved
    in a closed box.
"""
import ctypes as C
import os

import numpy as np
import pytest

import golden_configs as G
import pyoracle as O
from asteriy_2d_gb300 import abi as A
from asteriy_2d_gb300 import problems, solver
from conftest import golden

TOL = 1e-10
NT = os.cpu_count() or 1


def rel_linf(a, b):
    return np.max(np.abs(a - b), axis=0) / np.maximum(np.max(np.abs(b), axis=0), 1e-300)


@pytest.mark.parametrize("name,flux", [("hllc", A.FLUX_HLLC), ("hllcq", A.FLUX_HLLCQ)])
def test_oracle_scalar_faces_bitwise(name, flux):
    d = golden("faces_scalar.npz")
    X, Q, n, rad = d["states"], d["scalars"], d["normals"], d["rad"]
    F = np.zeros((len(X), 5))
    T = np.zeros(len(X))
    for i, row in enumerate(X):
        T[i], F[i] = O.face_q(flux, row[0:2], row[2:4], row[4:6], row[6:8], Q[i, 0], Q[i, 1], n[i, 0], n[i, 1],
                              rad[i], float(d["gamma"]), float(d["cfl"]))
    np.testing.assert_array_equal(F, d[name + "_flux"])
    np.testing.assert_array_equal(T, d[name + "_dt"])


def test_oracle_hllcq_gas_flux_bitwise():
    # the gas part of HLLCQ (the step's flux AST_FLUX_HLLCQ) does not depend on Q
    d = golden("faces_scalar.npz")
    X, n, rad = d["states"], d["normals"], d["rad"]
    for i, row in enumerate(X):
        t, F, _ = O.face(A.FLUX_HLLCQ, row[0:2], row[2:4], row[4:6], row[6:8], n[i, 0], n[i, 1], rad[i],
                         float(d["gamma"]), float(d["cfl"]))
        np.testing.assert_array_equal(F, d["hllcq_flux"][i, :4])
        assert t == d["hllcq_dt"][i]


@pytest.mark.parametrize("name,flux", [("hllc", A.FLUX_HLLC), ("hllcq", A.FLUX_HLLCQ)])
def test_oracle_scalar_step_bitwise(name, flux):
    d = golden(f"step_scalar_{name}.npz")
    cfg = G.scalar_config(flux)
    s, u, q, tdo, tt, st = O.run_scalar(cfg, d["s0"], d["u0"], d["q0"], int(d["nsteps"]), nthreads=2)
    np.testing.assert_array_equal(s, d["s"])
    np.testing.assert_array_equal(u, d["u"])
    np.testing.assert_array_equal(q, d["q"])
    assert tdo == d["T_do"] and tt == d["TT"] and st == d["steps"]


def test_hllcq_needs_fp64():
    c = G.scalar_config(A.FLUX_HLLCQ)
    assert solver.load().ast_config_check(C.byref(c)) == A.AST_OK
    c.precision = A.PREC_FP32
    assert solver.load().ast_config_check(C.byref(c)) == A.AST_ERR_INVALID


@pytest.mark.gpu
@pytest.mark.parametrize("name,flux", [("hllc", A.FLUX_HLLC), ("hllcq", A.FLUX_HLLCQ)])
def test_scalar_step_matches_reference_fixture(name, flux):
    d = golden(f"step_scalar_{name}.npz")
    cfg = G.scalar_config(flux)
    with solver.Solver(cfg) as S:
        S.set_state(d["s0"], d["u0"])
        S.set_scalar(d["q0"])
        S.step(int(d["nsteps"]))
        s, u = S.get_state()
        q = S.get_scalar()
        tdo, tt, st = S.clock()
    assert np.all(rel_linf(s, d["s"]) <= TOL) and np.all(rel_linf(u, d["u"]) <= TOL)
    assert rel_linf(q, d["q"]) <= TOL, rel_linf(q, d["q"])
    assert st == d["steps"] and abs(tdo - d["T_do"]) <= 1e-12 * d["T_do"] and abs(tt - d["TT"]) <= 1e-12 * d["TT"]


@pytest.mark.gpu
@pytest.mark.parametrize("recon", [A.RECON_NONE, A.RECON_MINMOD])
def test_hllcq_gas_step_matches_oracle(recon):
    cfg = problems.blast_config(64, 32, flux=A.FLUX_HLLCQ)
    cfg.recon = recon
    s0, u0 = solver.fill_blast(cfg)
    with solver.Solver(cfg) as S:
        S.set_state(s0, u0)
        S.step(40)
        s, u = S.get_state()
        tdo, tt, st = S.clock()
    os_, ou, otdo, ott, ost, _ = O.run(cfg, s0, u0, 40, nthreads=NT)
    assert np.all(rel_linf(s, os_) <= TOL) and np.all(rel_linf(u, ou) <= TOL)
    assert st == ost and abs(tdo - otdo) <= 1e-12 * otdo


@pytest.mark.gpu
@pytest.mark.parametrize("flux", [A.FLUX_HLLC, A.FLUX_HLLCQ])
@pytest.mark.parametrize("geom", [A.GEOM_PLANAR, A.GEOM_AXISYM])
def test_scalar_blast_matches_oracle(flux, geom):
    cfg = problems.blast_config(64, 32, flux=flux)
    cfg.recon, cfg.geom = A.RECON_MINMOD, geom
    s0, u0 = solver.fill_blast(cfg)
    rng = np.random.default_rng(5)
    q0 = rng.uniform(0.0, 1.0, cfg.N * cfg.M) * s0[:, 0]
    with solver.Solver(cfg) as S:
        S.set_state(s0, u0)
        S.set_scalar(q0)
        S.step(37)
        s, u = S.get_state()
        q = S.get_scalar()
    os_, ou, oq, *_ = O.run_scalar(cfg, s0, u0, q0, 37, nthreads=NT)
    assert np.all(rel_linf(s, os_) <= TOL) and np.all(rel_linf(u, ou) <= TOL)
    assert rel_linf(q, oq) <= TOL, rel_linf(q, oq)


@pytest.mark.gpu
@pytest.mark.parametrize("flux", [A.FLUX_HLLC, A.FLUX_HLLCQ])
def test_scalar_proportional_to_density_stays_so(flux):
    # Q = c rho: both the solvers' scalar flux and the update are the
    # density's times c, so Q / rho stays c (to rounding) on a blast with
    # reflecting and outflow sides
    cfg = problems.blast_config(96, 48, flux=flux)
    cfg.recon = A.RECON_MINMOD
    s0, u0 = solver.fill_blast(cfg)
    c = 0.7
    with solver.Solver(cfg) as S:
        S.set_state(s0, u0)
        S.set_scalar(c * s0[:, 0])
        S.step(60)
        s, _ = S.get_state()
        q = S.get_scalar()
    assert np.max(np.abs(q / s[:, 0] - c)) <= 1e-12 * 2 * c


@pytest.mark.gpu
def test_scalar_total_conserved_in_closed_box():
    cfg = problems.blast_config(64, 32, flux=A.FLUX_HLLCQ)
    cfg.recon, cfg.geom = A.RECON_MINMOD, A.GEOM_PLANAR
    for side in (A.Z_LO, A.Z_HI, A.R_LO, A.R_HI):
        A.set_bc(cfg, side, A.BC_REFLECT)
    s0, u0 = solver.fill_blast(cfg)
    q0 = np.random.default_rng(9).uniform(0.0, 2.0, cfg.N * cfg.M)
    with solver.Solver(cfg) as S:
        S.set_state(s0, u0)
        S.set_scalar(q0)
        S.step(50)
        q = S.get_scalar()
    assert abs(q.sum() - q0.sum()) <= 1e-12 * q0.sum()


@pytest.mark.gpu
def test_scalar_rejections():
    cfg = problems.blast_config(32, 16, flux=A.FLUX_HLL)
    q = np.ones(cfg.N * cfg.M)
    with solver.Solver(cfg) as S:
        with pytest.raises(solver.AstError) as e:
            S.set_scalar(q)
        assert e.value.code == A.AST_ERR_UNSUPPORTED
        with pytest.raises(solver.AstError):
            S.get_scalar()
    c32 = problems.blast_config(32, 16, flux=A.FLUX_HLLC, precision=A.PREC_FP32)
    with solver.Solver(c32) as S:
        with pytest.raises(solver.AstError) as e:
            S.set_scalar(q)
        assert e.value.code == A.AST_ERR_UNSUPPORTED
    creg = problems.blast_config(32, 16, flux=A.FLUX_HLLC)
    creg.region_select, creg.region_lo, creg.region_hi = 1, 0.2, 0.8
    with solver.Solver(creg) as S:
        with pytest.raises(solver.AstError):
            S.set_scalar(q)
    ch = problems.blast_config(32, 16, flux=A.FLUX_HLLCQ)
    s0, u0 = solver.fill_blast(ch)
    s1, u1 = np.empty_like(s0), np.empty_like(u0)
    args = (s0.ctypes.data, u0.ctypes.data, s1.ctypes.data, u1.ctypes.data)
    with solver.Solver(ch) as S:
        S.set_state(s0, u0)
        S.set_scalar(q)
        with pytest.raises(solver.AstError) as e:
            S.step_host(*args)
        assert e.value.code == A.AST_ERR_UNSUPPORTED
        S.set_scalar(None)
        S.step_host(*args)

