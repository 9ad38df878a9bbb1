"""Parity of the FP64 CUDA path with the oracle at the stated configurations
of the benchmark problems, at their full sizes.

  C1  blast 256x128, HLL + minmod, CFL 0.4, 500 steps (the whole run);
  C2  wind-counterflow 2048x1024, HLLC + minmod, seeded density noise, the
      wind sphere held fixed (add_MK, kernel.cu:2317-2324; set-up of
      kernel.cu:3355-3373), 100 steps;
  C4's problem in FP64: blast 4096x2048, exact Godunov + minmod at the
      reference's tolerance (10e-10, Header.h:62), 10 steps from t = 0.

Bar: relative L-infinity error <= 1e-10 per variable (max |gpu - oracle| /
max |oracle|), the clock equal to 1e-12, and the shock cells identical.
The oracle runs on all host cores.
"""
import os

import numpy as np
import pytest

import pyoracle as O
from asteriy_2d_gb300 import abi as A
from asteriy_2d_gb300 import problems, solver
from test_gpu_parity import TOL, assert_parity, assert_same_shock_cells

pytestmark = pytest.mark.gpu


def assert_same_front_faces(s, o, cfg, tie=1e-8, strong=5e-2):
    """Per row of cells (fixed r): in rows whose largest density jump along
    z exceeds `strong`, the face with the largest jump in the GPU result is
    also a largest jump of the oracle's (up to ties within `tie`)."""
    jg = np.abs(np.diff(s[:, 0].reshape(cfg.M, cfg.N), axis=1))
    jo = np.abs(np.diff(o[:, 0].reshape(cfg.M, cfg.N), axis=1))
    ig = np.argmax(jg, axis=1)
    mo = jo.max(axis=1)
    rows = np.nonzero(mo > strong)[0]
    assert len(rows) > 0
    bad = rows[jo[rows, ig[rows]] < mo[rows] * (1 - tie)]
    assert len(bad) == 0, bad


def test_c1_blast_hll_fp64_256x128_500_steps():
    cfg = problems.blast_config(256, 128)
    assert cfg.flux == A.FLUX_HLL and cfg.cfl == 0.4 and cfg.precision == A.PREC_FP64
    s0, u0 = solver.fill_blast(cfg)
    s, u, os_, ou = assert_parity(cfg, s0, u0, 500)
    assert_same_shock_cells(s, os_, cfg)


def test_c2_wind_hllc_fp64_2048x1024_100_steps():
    cfg = problems.wind_config(2048, 1024)
    assert cfg.flux == A.FLUX_HLLC and cfg.fixed_region == 1
    s0, u0 = solver.fill_wind(cfg)
    s, u, os_, ou = assert_parity(cfg, s0, u0, 100)
    assert_same_front_faces(s, os_, cfg)


def test_blast_godunov_fp64_4096x2048_10_steps():
    cfg = problems.blast_config(4096, 2048, flux=A.FLUX_GODUNOV)
    assert cfg.riemann_tol == 10e-10
    s0, u0 = solver.fill_blast(cfg)
    s, u, os_, ou = assert_parity(cfg, s0, u0, 10)
    assert_same_shock_cells(s, os_, cfg)


def test_exact_solver_excess_at_reference_tolerance_is_explained():
    """At the reference's tolerance (10e-10) the FP64 exact-solver step
    agrees with the oracle to 1e-9, not 1e-10, after 100 steps of the
    128x64 blast.  Cell by cell, this is where the excess comes from:
      (1) one step from identical inputs agrees to 1e-14 at every step of
          the oracle's trajectory: rounding only;
      (2) along the two runs' own trajectories every jump (a cell whose
          difference grows more than 100-fold in one step, to above 1e-12,
          over its stencil's input difference) sits at a cell one of whose
          faces' bisection stopping tests (devtwo, kernel.cu:682-749) came
          within 1% of the tolerance, |res| within 1e-11 of 10e-10, or whose
          Udf lies within 1e-9 (relative) of a wave-pattern threshold: the
          inputs' accumulated 1e-13-level difference moves the absolute
          stopping test by one bisection iterate (about tol in the residual)
          or the face into the neighbouring pattern."""
    from scipy.ndimage import maximum_filter
    cfg = problems.blast_config(128, 64, flux=A.FLUX_GODUNOV)
    N, M = cfg.N, cfg.M
    foot = np.zeros((5, 5), bool)
    foot[2, :] = True
    foot[:, 2] = True
    nt = os.cpu_count() or 1

    def dcell(sg, ug, so, uo):
        return np.maximum(np.abs(sg - so) / np.max(np.abs(so), axis=0),
                          np.abs(ug - uo) / np.maximum(np.max(np.abs(uo), axis=0), 1e-300)).max(axis=1)

    s, u = solver.fill_blast(cfg)
    so, uo = s.copy(), u.copy()
    tdo = cfg.dt_first
    prev = np.zeros(N * M)
    jumps = 0
    with solver.Solver(cfg) as S, solver.Solver(cfg) as S1:
        S.set_state(s, u)
        for k in range(100):
            so2, uo2, T, bm, pm = O.step_margin(cfg, so, uo, tdo, nthreads=nt)
            S1.set_state(so, uo)
            S1.set_clock(tdo, 0.0, k)
            S1.step(1)
            assert dcell(*S1.get_state(), so2, uo2).max() <= 1e-14, k
            S.step(1)
            d = dcell(*S.get_state(), so2, uo2)
            pnb = maximum_filter(prev.reshape(M, N), footprint=foot, mode="nearest").reshape(-1)
            jump = (d > 1e-12) & (d > 100 * pnb)
            explained = (bm < 1e-2) | (pm < 1e-9)
            assert np.all(explained[jump]), (k, np.nonzero(jump & ~explained)[0][:5])
            jumps += int(jump.sum())
            prev = d
            so, uo, tdo = so2, uo2, T
    assert jumps > 0                     # the mechanism shows up in this run
    assert prev.max() <= 1e-9
