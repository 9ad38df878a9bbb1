"""Host-side pieces of bench.py's reference arm (CPU only): the blast's
initial state by numpy equals ast_fill_blast, and the start state it
advances on the part of the grid the blast can reach (z >= 0 mirrored)
equals the oracle's full-grid run; and each form the bench times is the
configuration its name states."""
import ctypes

import numpy as np
import pytest

import bench
import pyoracle as O
from asteriy_2d_gb300 import abi as A
from asteriy_2d_gb300 import problems, solver


@pytest.mark.parametrize("N,M", [(256, 128), (130, 64)])
def test_blast_host_equals_library_fill(N, M):
    cfg = problems.blast_config(N, M, flux=A.FLUX_GODUNOV)
    s, u = bench.blast_host(cfg)
    s2, u2 = solver.fill_blast(cfg)
    assert np.array_equal(s, s2) and np.array_equal(u, u2)


@pytest.mark.parametrize("flux", [A.FLUX_HLL, A.FLUX_GODUNOV])
def test_advanced_start_state_matches_full_grid(flux):
    cfg = problems.blast_config(256, 128, flux=flux)
    nsteps = 40

    def run(c, s, u, n, clock=None):
        return O.run(c, s, u, n, nthreads=O.max_threads())

    s, u, (T_do, TT, step) = bench.blast_host_advanced(cfg, nsteps, run, margin=8)
    s0, u0 = solver.fill_blast(cfg)
    fs, fu, fT, fTT, fstep, _ = O.run(cfg, s0, u0, nsteps, nthreads=O.max_threads())
    assert step == fstep == nsteps
    assert abs(T_do - fT) <= 1e-12 * fT and abs(TT - fTT) <= 1e-12 * fTT
    es = np.max(np.abs(s - fs), axis=0) / np.max(np.abs(fs), axis=0)
    eu = np.max(np.abs(u - fu), axis=0) / np.max(np.abs(fu), axis=0)
    # the mirrored half and the sub-grid's cell size agree with the full
    # grid to rounding (the full-grid run is symmetric to rounding)
    assert np.all(es < 1e-11) and np.all(eu < 1e-11), (es, eu)


@pytest.mark.parametrize("form", bench.FORMS)
def test_bench_forms_map_to_their_configurations(form):
    # each form's name states its precision, flux, start value and skip flag
    cfg = bench.make_config(form)
    assert (cfg.N, cfg.M) == (bench.N_Z, bench.M_R)
    assert cfg.precision == (A.PREC_FP64 if form.startswith("fp64") else A.PREC_FP32)
    assert cfg.flux == (A.FLUX_HLL if "_hll" in form else A.FLUX_GODUNOV)
    assert cfg.recon == A.RECON_MINMOD
    if cfg.precision == A.PREC_FP32:
        assert cfg.skip_uniform == (1 if form.endswith("_skip") else 0)
        assert cfg.guess == (A.GUESS_MLP if form.startswith("fp32_learned") else A.GUESS_PVRS)
    assert solver.load().ast_config_check(ctypes.byref(cfg)) == A.AST_OK
