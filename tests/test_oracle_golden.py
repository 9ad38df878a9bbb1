"""The oracle against the golden vectors recorded from the reference's own
functions (tests/golden/make_golden.py).  Bit-for-bit: the oracle restates
the reference's arithmetic in the same order and both are compiled with
-ffp-contract=off."""
import numpy as np
import pytest

import golden_configs as G
import pyoracle as O
from conftest import golden


@pytest.mark.parametrize("name,flux", [("hll", O.FACE_HLL), ("hllc", O.FACE_HLLC),
                                       ("godunov", O.FACE_GODUNOV), ("hllca", O.FACE_HLLC_A)])
def test_face_functions_bitwise(name, flux):
    d = golden("faces.npz")
    X, n, rad = d["states"], d["normals"], d["rad"]
    F = np.zeros((len(X), 4))
    T = np.zeros(len(X))
    for i, row in enumerate(X):
        T[i], F[i], _ = O.face(flux, row[0:2], row[2:4], row[4:6], row[6:8], n[i, 0], n[i, 1], rad[i],
                               float(d["gamma"]), float(d["cfl"]))
    np.testing.assert_array_equal(F, d[name + "_flux"])
    np.testing.assert_array_equal(T, d[name + "_dt"])


def test_godunov_reaches_every_wave_pattern():
    d = golden("faces.npz")
    X = d["states"][-8:]
    seen = {"newton": 0, "bisect": 0, "vacuum": 0}
    for row in X:
        _, _, c = O.face(O.FACE_GODUNOV, row[0:2], row[2:4], row[4:6], row[6:8], 1.0, 0.0, 0.01)
        seen["newton"] += c[0]
        seen["bisect"] += c[3]
        seen["vacuum"] += c[6]
    assert seen["newton"] >= 2 and seen["bisect"] >= 1 and seen["vacuum"] >= 1


def test_uniform_state_flux_is_physical_flux():
    # the idea of the reference's `test` kernel (kernel.cu:3095-3107):
    # identical states give the exact Euler flux for every solver
    s, u = [1.0, 0.0666666], [-1.0, 0.0]
    g = 5.0 / 3.0
    E = s[1] / (g - 1) + 0.5 * s[0] * (u[0] ** 2 + u[1] ** 2)
    exact = np.array([s[0] * u[0], s[0] * u[0] ** 2 + s[1], s[0] * u[0] * u[1], (E + s[1]) * u[0]])
    for flux in (O.FACE_HLL, O.FACE_HLLC, O.FACE_GODUNOV):
        _, F, _ = O.face(flux, s, u, s, u, 1.0, 0.0, 0.01)
        np.testing.assert_allclose(F, exact, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("fname,cfg", [
    ("step_tvd.npz", G.tvd_config()),
    ("step_mk_hll.npz", G.add_mk_config(0)),
    ("step_mk_god.npz", G.add_mk_config(2)),
    ("step_mk_hllca.npz", G.add_mk_config(1)),
])
def test_steps_bitwise_against_reference_kernels(fname, cfg):
    d = golden(fname)
    s, u, tdo, tt, st, _ = O.run(cfg, d["s0"], d["u0"], int(d["nsteps"]), nthreads=2)
    np.testing.assert_array_equal(s, d["s"])
    np.testing.assert_array_equal(u, d["u"])
    assert tdo == float(d["T_do"]) and tt == float(d["TT"]) and st == int(d["steps"])


def test_neutral_source_bitwise_against_reference_add_mk():
    # add_MK with a random nn2 (its momentum source, kernel.cu:2495-2496)
    d = golden("step_mk_neutral.npz")
    s, u, tdo, tt, st, _ = O.run(G.add_mk_config(0), d["s0"], d["u0"], int(d["nsteps"]), nthreads=2, nn2=d["nn2"])
    np.testing.assert_array_equal(s, d["s"])
    np.testing.assert_array_equal(u, d["u"])
    assert tdo == float(d["T_do"]) and tt == float(d["TT"]) and st == int(d["steps"])


def test_step_is_deterministic_across_thread_counts():
    cfg = G.tvd_config()
    rng = np.random.default_rng(3)
    s, u = G.random_state(cfg.N * cfg.M, rng)
    a = O.run(cfg, s, u, 5, nthreads=1)
    b = O.run(cfg, s, u, 5, nthreads=4)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    assert a[2] == b[2]


@pytest.mark.skipif(not O.have_ref(), reason="reference functions not built here")
def test_oracle_matches_live_reference_on_fresh_inputs():
    cfg = G.add_mk_config(2, N=40, M=20)
    rng = np.random.default_rng(11)
    s, u = G.random_state(cfg.N * cfg.M, rng)
    r = O.ref_run(O.REF_ADD_MK, cfg, s, u, 8, method=2)
    o = O.run(cfg, s, u, 8)
    np.testing.assert_array_equal(r[0], o[0])
    np.testing.assert_array_equal(r[1], o[1])


@pytest.mark.skipif(not O.have_ref(), reason="reference functions not built here")
@pytest.mark.parametrize("flux", [O.FACE_HLL, O.FACE_HLLC, O.FACE_GODUNOV])
def test_composed_step_with_reference_faces_is_bitwise(flux):
    """Blast problem (axisymmetric, minmod) stepped with the reference's own
    face functions equals the oracle bit for bit."""
    from asteriy_2d_gb300 import problems
    cfg = problems.blast_config(64, 32, flux=flux)
    s0 = np.stack([np.ones(64 * 32), np.where(np.arange(64 * 32) % 7 == 0, 10.0, 0.1)], 1)
    u0 = np.zeros((64 * 32, 2))
    a = O.run(cfg, s0, u0, 15)
    b = O.ref_run_composed(cfg, s0, u0, 15)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    assert a[2] == b[2]


def test_inflow_bitwise_against_reference_add2_bound():
    """The oracle's characteristic inflow equals the reference's add2_bound
    (kernel.cu:1895-1925) on the recorded random old/new states."""
    z = golden("inflow.npz")
    cfg = G.inflow_config()
    s2, u2 = O.inflow(cfg, z["s"], z["u"], z["s2"], z["u2"])
    assert np.array_equal(s2, z["s2_out"]) and np.array_equal(u2, z["u2_out"])
    # only column 0 changes
    changed = np.any(z["s2_out"] != z["s2"], axis=1).reshape(cfg.M, cfg.N)
    assert changed[:, 0].all() and not changed[:, 1:].any()
    if O.have_ref():
        b2, c2 = O.ref_bound(cfg, z["s"], z["u"], z["s2"], z["u2"])
        assert np.array_equal(b2, s2) and np.array_equal(c2, u2)
