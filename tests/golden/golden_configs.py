"""Runtime configurations that reproduce the reference's hard-coded kernels.

Shared by tests/golden/make_golden.py (which records the reference's outputs)
and by the tests (which replay the same configurations on the oracle and on
the CUDA path).
"""
import numpy as np

from asteriy_2d_gb300 import abi as A

V_INF = -2.54186  # Velosity_inf, Header.h:86


def face_config():
    return A.default_config()


def tvd_config(N=96, M=12):
    """Kernel_TVD (kernel.cu:2513-3093) with Header.h's domain [0,80]x[0,1]:
    HLLC + minmod faces for 10.000001 < z_face < 40.000001, first-order HLL
    elsewhere; inflow (1, p_H) (1, 0) at n=0, outflow at n=N-1, reflecting
    r=0 and r=y_max; body force +-4 rho for 20.000001 < z < 30.000001."""
    c = A.default_config()
    c.N, c.M = N, M
    c.flux, c.recon, c.geom = A.FLUX_HLLC, A.RECON_MINMOD, A.GEOM_PLANAR
    c.region_select, c.region_lo, c.region_hi = 1, 10.000001, 40.000001
    A.set_bc(c, A.Z_LO, A.BC_FIXED, 1.0, 7.0, 1.0, 0.0)
    A.set_bc(c, A.Z_HI, A.BC_OUTFLOW)
    A.set_bc(c, A.R_LO, A.BC_REFLECT)
    A.set_bc(c, A.R_HI, A.BC_REFLECT)
    c.body_force, c.body_lo, c.body_hi, c.body_rsplit, c.body_amp = 1, 20.000001, 30.000001, 0.5, 4.0
    return c


def add_mk_config(method, N=48, M=24):
    """add_MK (kernel.cu:2293-2511) on z in [-1,1], r in [0,1]: first order,
    method 0 = HLL, 1 = HLLC_Aleksashov, 2 = exact Godunov (hx, hy of
    Header.h:29-30 select no HLL
    face), axisymmetric source, free stream (1, 1) (V_inf, 0) at n=N-1,
    suction clamp v_z <= V_inf/2 at n=0, zero gradient at r=y_max, axis
    reflection, cells inside z^2/0.04 + r^2/0.04 < 1 held fixed."""
    c = A.default_config()
    c.N, c.M = N, M
    c.x_min, c.x_max, c.y_max = -1.0, 1.0, 1.0
    c.flux = {0: A.FLUX_HLL, 1: A.FLUX_HLLC_A, 2: A.FLUX_GODUNOV}[method]
    c.recon, c.geom = A.RECON_NONE, A.GEOM_AXISYM
    A.set_bc(c, A.Z_HI, A.BC_FIXED, 1.0, 1.0, V_INF, 0.0)
    A.set_bc(c, A.Z_LO, A.BC_SUCTION, 0.0, 0.0, 0.5 * V_INF, 0.0)
    A.set_bc(c, A.R_HI, A.BC_OUTFLOW)
    A.set_bc(c, A.R_LO, A.BC_REFLECT)
    c.fixed_region, c.fixed_zc, c.fixed_az, c.fixed_ar = 1, 0.0, 0.2, 0.2
    return c


def random_state(K, rng):
    s = np.stack([rng.uniform(0.5, 2.0, K), rng.uniform(2.0, 10.0, K)], 1)
    u = np.stack([rng.uniform(-1.0, 2.0, K), rng.uniform(-0.5, 0.5, K)], 1)
    return s, u


def inflow_config(N=24, M=8):
    """add2_bound (kernel.cu:1895-1925): p_H = 7 (Header.h:6), inflow speed 1."""
    c = A.default_config()
    c.N, c.M = N, M
    c.inflow_p, c.inflow_v = 7.0, 1.0
    return c


def writer_config(N=24, M=12):
    """The grid of the writer fixtures: z in [-1, 1], r in [0, 1], gamma 5/3."""
    c = A.default_config()
    c.N, c.M = N, M
    c.x_min, c.x_max, c.y_max = -1.0, 1.0, 1.0
    return c


def add2_config(N=96, M=12):
    """add2 (kernel.cu:1928-2291) with Header.h's domain [0,80]x[0,1]: the
    region 10.000001 < x < 40.000001 of its flux rule, inflow (1, p_H)
    (1, 0) at n=0 (p_H = 7), outflow at n=N-1, reflecting r sides, body
    force +-2.5 rho for 20.000001 < x < 30.000001 (split at r = 0.5),
    first order, planar."""
    c = A.default_config()
    c.N, c.M = N, M
    c.flux, c.recon, c.geom = A.FLUX_HLLC, A.RECON_NONE, A.GEOM_PLANAR
    c.region_select, c.region_lo, c.region_hi = 1, 10.000001, 40.000001
    A.set_bc(c, A.Z_LO, A.BC_FIXED, 1.0, 7.0, 1.0, 0.0)
    A.set_bc(c, A.Z_HI, A.BC_OUTFLOW)
    A.set_bc(c, A.R_LO, A.BC_REFLECT)
    A.set_bc(c, A.R_HI, A.BC_REFLECT)
    c.body_force, c.body_lo, c.body_hi, c.body_rsplit, c.body_amp = 1, 20.000001, 30.000001, 0.5, 2.5
    return c


def scalar_config(flux, N=48, M=24):
    """A passive scalar carried by the HLLC (flux 1) or HLLCQ (flux 4) solver
    on an axisymmetric 48x24 grid, z in [-1, 1], r in [0, 1], minmod: fixed
    inflow (1, 1) (V_inf, 0) with scalar 2 at n = N-1, outflow at n = 0 and
    r = y_max, axis reflection, cells inside z^2/0.04 + r^2/0.04 < 1 held
    fixed; FP64."""
    c = A.default_config()
    c.N, c.M = N, M
    c.x_min, c.x_max, c.y_max = -1.0, 1.0, 1.0
    c.flux, c.recon, c.geom = flux, A.RECON_MINMOD, A.GEOM_AXISYM
    A.set_bc(c, A.Z_HI, A.BC_FIXED, 1.0, 1.0, V_INF, 0.0)
    A.set_bc(c, A.Z_LO, A.BC_OUTFLOW)
    A.set_bc(c, A.R_HI, A.BC_OUTFLOW)
    A.set_bc(c, A.R_LO, A.BC_REFLECT)
    c.fixed_region, c.fixed_zc, c.fixed_az, c.fixed_ar = 1, 0.0, 0.2, 0.2
    c.scalar_in = 2.0
    return c
