"""ctypes mirror of include/asteriy_gb300.h.

The structures here must match the C layout byte for byte;
tests/test_abi.py checks ctypes.sizeof against the library's own sizeof.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libasteriy_gb300.so")

AST_OK = 0
AST_ERR_INVALID = -1
AST_ERR_CUDA = -2
AST_ERR_NOMEM = -3
AST_ERR_IO = -4
AST_ERR_UNSUPPORTED = -5
AST_ERR_NUMERIC = -6

AST_ST_RHO_FLOOR = 0x01
AST_ST_P_FLOOR = 0x02
AST_ST_NEWTON_CAP = 0x04
AST_ST_BISECT_CAP = 0x08
AST_ST_NONFINITE = 0x10
AST_ST_VACUUM = 0x20
AST_ST_MLP_FALLBACK = 0x40
AST_ST_TIMEOUT = 0x80
AST_MLP_NPARAM = 1325
AST_RECORD_FLOATS = 10

FLUX_HLL, FLUX_HLLC, FLUX_GODUNOV, FLUX_HLLC_A, FLUX_HLLCQ = 0, 1, 2, 3, 4
RECON_NONE, RECON_MINMOD = 0, 1
GEOM_PLANAR, GEOM_AXISYM = 0, 1
PREC_FP64, PREC_FP32 = 0, 1
GUESS_PVRS, GUESS_MLP = 0, 1
Z_LO, Z_HI, R_LO, R_HI = 0, 1, 2, 3
BC_REFLECT, BC_OUTFLOW, BC_FIXED, BC_SUCTION, BC_NONREFLECT = 0, 1, 2, 3, 4
SETUP_BLAST, SETUP_WIND = 0, 1
AST_BATCH_MAX = 4096


class ast_bc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("pad_", C.c_int32),
                ("rho", C.c_double), ("p", C.c_double), ("vz", C.c_double), ("vr", C.c_double)]


class ast_config(C.Structure):
    _fields_ = [
        ("N", C.c_int32), ("M", C.c_int32),
        ("x_min", C.c_double), ("x_max", C.c_double), ("y_max", C.c_double),
        ("gamma", C.c_double), ("cfl", C.c_double),
        ("flux", C.c_int32), ("recon", C.c_int32), ("geom", C.c_int32),
        ("precision", C.c_int32), ("grad_p", C.c_int32), ("guess", C.c_int32),
        ("bc", ast_bc * 4),
        ("fixed_region", C.c_int32), ("region_select", C.c_int32),
        ("fixed_zc", C.c_double), ("fixed_az", C.c_double), ("fixed_ar", C.c_double),
        ("region_lo", C.c_double), ("region_hi", C.c_double),
        ("body_force", C.c_int32), ("riemann_max_iter", C.c_int32),
        ("body_lo", C.c_double), ("body_hi", C.c_double),
        ("body_rsplit", C.c_double), ("body_amp", C.c_double),
        ("dt_first", C.c_double), ("dt_cap", C.c_double), ("p_floor", C.c_double),
        ("riemann_tol", C.c_double),
        ("collect_stats", C.c_int32), ("riemann_newton", C.c_int32), ("persistent", C.c_int32),
        ("skip_uniform", C.c_int32), ("copy_wait_polls", C.c_int32), ("reserved_i", C.c_int32 * 3),
        ("mlp_gate", C.c_double), ("inflow_p", C.c_double), ("inflow_v", C.c_double),
        ("neutral_nh", C.c_double), ("neutral_kn", C.c_double), ("scalar_in", C.c_double),
        ("reserved_d", C.c_double * 2),
    ]

    def copy(self):
        c = ast_config()
        C.pointer(c)[0] = self
        return c

    def describe(self):
        out = {}
        for name, _ in self._fields_:
            if name in ("bc", "reserved_i", "reserved_d", "pad_"):
                continue
            out[name] = getattr(self, name)
        out["bc"] = [(b.kind, b.rho, b.p, b.vz, b.vr) for b in self.bc]
        return out


class ast_stats(C.Structure):
    _fields_ = [
        ("status", C.c_uint32), ("newton_max_iters", C.c_uint32),
        ("rho_floor", C.c_uint64), ("p_floor", C.c_uint64),
        ("newton_calls", C.c_uint64), ("newton_iters", C.c_uint64),
        ("bisect_calls", C.c_uint64), ("bisect_iters", C.c_uint64),
        ("mlp_fallback", C.c_uint64), ("strong_calls", C.c_uint64), ("strong_iters", C.c_uint64),
        ("reserved", C.c_uint64 * 2),
    ]


class ast_problem(C.Structure):
    _fields_ = [
        ("cfg", ast_config), ("setup", C.c_int32), ("reserved_i", C.c_int32),
        ("mach", C.c_double), ("seed", C.c_uint64), ("reserved_d", C.c_double * 5),
    ]


def default_config():
    """The reference's Header.h values (see ast_config_default in C)."""
    c = ast_config()
    c.N, c.M = 32000, 400
    c.x_min, c.x_max, c.y_max = 0.0, 80.0, 1.0
    c.gamma, c.cfl = 5.0 / 3.0, 0.05
    c.flux, c.recon, c.geom, c.precision = FLUX_HLL, RECON_MINMOD, GEOM_PLANAR, PREC_FP64
    c.grad_p, c.guess = 1, GUESS_PVRS
    for side in range(4):
        c.bc[side].kind = BC_OUTFLOW
    c.bc[R_LO].kind = BC_REFLECT
    c.bc[R_HI].kind = BC_REFLECT
    c.fixed_region = 0
    c.fixed_zc, c.fixed_az, c.fixed_ar = 0.0, 1.0, 1.0
    c.region_select, c.region_lo, c.region_hi = 0, 0.0, 0.0
    c.body_force, c.body_lo, c.body_hi, c.body_rsplit, c.body_amp = 0, 0.0, 0.0, 0.0, 0.0
    c.riemann_max_iter = 200
    c.dt_first, c.dt_cap, c.p_floor, c.riemann_tol = 1e-9, 1000.0, 1e-6, 10e-10
    c.collect_stats = 0
    c.persistent = 1
    c.mlp_gate = 0.2
    c.inflow_p, c.inflow_v = 0.0, 1.0
    c.neutral_nh, c.neutral_kn = 3.0, 0.419231
    return c


def set_bc(cfg, side, kind, rho=0.0, p=0.0, vz=0.0, vr=0.0):
    b = cfg.bc[side]
    b.kind, b.rho, b.p, b.vz, b.vr = kind, rho, p, vz, vr
