"""The benchmark problems as runtime configurations.

blast    axisymmetric blast on z in [-1,1], r in [0,1]: rho=1, v=0, p=10
         inside a sphere of radius 0.2 at the origin, p=0.1 outside;
         reflecting axis, outflow elsewhere; gamma 5/3, CFL 0.4.  At 256x128
         with HLL + minmod in FP64 it is the small CPU-runnable case; at
         4096x2048 it is the precision (FP32) and learned-guess (exact
         Godunov) workload.
wind     wind-counterflow: a supersonic radial wind (rho ~ 1/R^2, |v|=10,
         Mach 10 at the wind sphere R=0.05 at the origin, held fixed as in
         add_MK, kernel.cu:2317-2324) against a Mach-2 counterflow along -z
         (rho=1, p=1/gamma, v_z=-2) entering at z=1, +-1% seeded density
         noise; axis reflecting, outflow at z=-1 and r=1; HLLC + minmod.
"""
from . import abi as A


def blast_config(N=256, M=128, flux=A.FLUX_HLL, precision=A.PREC_FP64, cfl=0.4):
    c = A.default_config()
    c.N, c.M = N, M
    c.x_min, c.x_max, c.y_max = -1.0, 1.0, 1.0
    c.gamma, c.cfl = 5.0 / 3.0, cfl
    c.flux, c.recon, c.geom, c.precision = flux, A.RECON_MINMOD, A.GEOM_AXISYM, precision
    A.set_bc(c, A.Z_LO, A.BC_OUTFLOW)
    A.set_bc(c, A.Z_HI, A.BC_OUTFLOW)
    A.set_bc(c, A.R_LO, A.BC_REFLECT)
    A.set_bc(c, A.R_HI, A.BC_OUTFLOW)
    return c


def wind_config(N=2048, M=1024, flux=A.FLUX_HLLC, precision=A.PREC_FP64, cfl=0.4, gamma=5.0 / 3.0,
                v_inf=-2.0):
    c = A.default_config()
    c.N, c.M = N, M
    c.x_min, c.x_max, c.y_max = -1.0, 1.0, 1.0
    c.gamma, c.cfl = gamma, cfl
    c.flux, c.recon, c.geom, c.precision = flux, A.RECON_MINMOD, A.GEOM_AXISYM, precision
    A.set_bc(c, A.Z_HI, A.BC_FIXED, 1.0, 1.0 / gamma, v_inf, 0.0)
    A.set_bc(c, A.Z_LO, A.BC_OUTFLOW)
    A.set_bc(c, A.R_LO, A.BC_REFLECT)
    A.set_bc(c, A.R_HI, A.BC_OUTFLOW)
    c.fixed_region, c.fixed_zc, c.fixed_az, c.fixed_ar = 1, 0.0, 0.05, 0.05
    return c
