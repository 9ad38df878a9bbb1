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
