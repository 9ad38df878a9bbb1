"""ctypes wrapper of the CPU oracle (oracle/ast_oracle.c) and of the host-
compiled reference functions (oracle/_ref/libastref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
the cpu_baseline / reference legs of bench.py, never by the package.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libastoracle.so")
REF_SO = os.path.join(HERE, "_ref", "libastref.so")

_dp = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_int64)


def build_oracle(cc="gcc"):
    """Compile the C restatement (a few seconds)."""
    cmd = [cc, "-O2", "-std=c99", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
           os.path.join(HERE, "ast_oracle.c"), "-lm", "-o", ORACLE_SO]
    subprocess.run(cmd, check=True)
    return ORACLE_SO


def _ptr(a):
    return a.ctypes.data_as(_dp)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build_oracle()
        L = C.CDLL(ORACLE_SO)
        L.ora_minmod.restype = C.c_double
        L.ora_minmod.argtypes = [C.c_double, C.c_double]
        L.ora_linear.restype = C.c_double
        L.ora_linear.argtypes = [C.c_double] * 7
        L.ora_linear2.restype = None
        L.ora_linear2.argtypes = [C.c_double] * 8 + [_dp, _dp]
        L.ora_face.restype = C.c_double
        L.ora_face.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_int,
                               _dp, _dp, _dp, _dp, C.c_double, C.c_double, C.c_double, _dp, _i64p]
        L.ora_set_neutral.restype = None
        L.ora_set_neutral.argtypes = [C.c_void_p]
        L.ora_step.restype = C.c_double
        L.ora_step.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, C.c_double, C.c_int, _i64p]
        L.ora_run.restype = C.c_int
        L.ora_run.argtypes = [C.c_void_p, _dp, _dp, C.c_int, _dp, _dp, _i64p, C.c_int, _i64p]
        L.ora_max_threads.restype = C.c_int
        L.ora_set_margin.restype = None
        L.ora_set_margin.argtypes = [C.c_void_p, C.c_void_p]
        L.ora_inflow.restype = None
        L.ora_inflow.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
        _scalar_api(L)
        L.ora_face_q.restype = C.c_double
        L.ora_face_q.argtypes = [C.c_int, C.c_double, C.c_double, _dp, _dp, _dp, _dp] + [C.c_double] * 5 + [_dp]
        _lib = L
    return _lib


def have_ref():
    return os.path.exists(REF_SO)


def ref():
    global _ref
    if _ref is None:
        R = C.CDLL(REF_SO)
        R.ref_set_params.restype = None
        R.ref_set_params.argtypes = [C.c_int, C.c_int] + [C.c_double] * 5
        R.ref_face.restype = C.c_double
        R.ref_face.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.c_double, C.c_double, C.c_double, _dp]
        R.ref_minmod.restype = C.c_double
        R.ref_minmod.argtypes = [C.c_double, C.c_double]
        R.ref_linear.restype = C.c_double
        R.ref_linear.argtypes = [C.c_double] * 7
        R.ref_linear2.restype = None
        R.ref_linear2.argtypes = [C.c_double] * 8 + [_dp, _dp]
        R.ref_kernel_step.restype = C.c_double
        R.ref_kernel_step.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.c_double, C.c_double, C.c_int, C.c_int]
        R.ref_kernel_run.restype = C.c_int
        R.ref_kernel_run.argtypes = [C.c_int, _dp, _dp, C.c_int, C.c_int, _dp, _dp,
                                     C.POINTER(C.c_longlong), C.c_int]
        R.ora_run.restype = C.c_int
        R.ora_run.argtypes = [C.c_void_p, _dp, _dp, C.c_int, _dp, _dp, _i64p, C.c_int, _i64p]
        R.ref_set_neutral.restype = None
        R.ref_set_neutral.argtypes = [C.c_void_p]
        R.ref_bound.restype = None
        R.ref_bound.argtypes = [_dp, _dp, _dp, _dp]
        R.ref_diag_count.restype = C.c_longlong
        if hasattr(R, "ref_print_file_mini"):
            R.ref_print_file_mini.restype = None
            R.ref_print_file_mini.argtypes = [_dp, _dp, C.c_int, C.c_double, C.c_char_p]
            R.ref_end_of_run.restype = None
            R.ref_end_of_run.argtypes = [_dp, _dp, C.c_double, C.c_int, C.c_double, C.c_double, C.c_char_p]
        R.ref_max_threads.restype = C.c_int
        _scalar_api(R)
        R.ref_face_q.restype = C.c_double
        R.ref_face_q.argtypes = [C.c_int, _dp, _dp, _dp, _dp] + [C.c_double] * 5 + [_dp]
        _ref = R
    return _ref


def _scalar_api(L):
    """The step loop's entry points (in both libraries: libastref.so carries
    the oracle's loop with the reference's face functions)."""
    L.ora_step.restype = C.c_double
    L.ora_step.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, C.c_double, C.c_int, _i64p]
    L.ora_set_scalar.restype = None
    L.ora_set_scalar.argtypes = [C.c_void_p, C.c_void_p, C.c_double]
    L.ora_inflow.restype = None
    L.ora_inflow.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]


# ---------------------------------------------------------------- oracle

FACE_HLL, FACE_HLLC, FACE_GODUNOV, FACE_HLLC_A = 0, 1, 2, 3


def face(flux, sL, uL, sR, uR, n1, n2, rad, gamma=5.0 / 3.0, cfl=0.05, tol=10e-10, max_iter=200):
    """One face flux.  Returns (dt, out[4] = mass, mom_z, mom_r, energy, counters[7])."""
    a = [np.ascontiguousarray(v, dtype=np.float64) for v in (sL, uL, sR, uR)]
    out = np.zeros(4)
    cnt = np.zeros(7, dtype=np.int64)
    t = lib().ora_face(flux, gamma, cfl, tol, max_iter, _ptr(a[0]), _ptr(a[1]), _ptr(a[2]), _ptr(a[3]),
                       n1, n2, rad, _ptr(out), cnt.ctypes.data_as(_i64p))
    return t, out, cnt


def face_q(flux, sL, uL, sR, uR, QL, QR, n1, n2, rad, gamma=5.0 / 3.0, cfl=0.05):
    """One face of a passive-scalar solver (flux 1: HLLC, 4: HLLCQ).
    Returns (dt, out[5] = mass, mom_z, mom_r, energy, scalar)."""
    a = [np.ascontiguousarray(v, dtype=np.float64) for v in (sL, uL, sR, uR)]
    out = np.zeros(5)
    t = lib().ora_face_q(flux, gamma, cfl, _ptr(a[0]), _ptr(a[1]), _ptr(a[2]), _ptr(a[3]), QL, QR, n1, n2, rad,
                         _ptr(out))
    return t, out


def run_scalar(cfg, s, u, q, nsteps, nthreads=1, T_do=None, TT=0.0, step_no=0, use_ref=False):
    """nsteps steps carrying the passive scalar q (K values, index m*N + n),
    with the lagged-dt protocol (and the characteristic inflow after each
    step when cfg.inflow_p > 0).  use_ref: the faces evaluated by the
    reference's own functions (libastref.so).  Returns (s, u, q, T_do, TT,
    step)."""
    L = ref() if use_ref else lib()
    if use_ref:
        ref_set(cfg)
    s = np.array(s, dtype=np.float64, order="C")
    u = np.array(u, dtype=np.float64, order="C")
    q = np.array(q, dtype=np.float64, order="C").reshape(-1)
    s2, u2, q2 = np.empty_like(s), np.empty_like(u), np.empty_like(q)
    tdo = cfg.dt_first if T_do is None else T_do
    cnt = np.zeros(10, dtype=np.int64)
    for _ in range(nsteps):
        L.ora_set_scalar(q.ctypes.data, q2.ctypes.data, cfg.scalar_in)
        try:
            T = L.ora_step(C.byref(cfg), _ptr(s), _ptr(u), _ptr(s2), _ptr(u2), tdo, nthreads,
                           cnt.ctypes.data_as(_i64p))
        finally:
            L.ora_set_scalar(None, None, 0.0)
        if cfg.inflow_p > 0.0:
            L.ora_inflow(C.byref(cfg), _ptr(s), _ptr(u), _ptr(s2), _ptr(u2))
        tdo = T
        TT = TT + tdo
        step_no += 1
        s, s2 = s2, s
        u, u2 = u2, u
        q, q2 = q2, q
    return s, u, q, tdo, TT, step_no


def step(cfg, s, u, T_do, nthreads=1):
    """One step; s, u: (K, 2) float64.  Returns (s2, u2, new_dt, counters[10])."""
    s = np.ascontiguousarray(s, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    s2 = np.empty_like(s)
    u2 = np.empty_like(u)
    cnt = np.zeros(10, dtype=np.int64)
    T = lib().ora_step(C.byref(cfg), _ptr(s), _ptr(u), _ptr(s2), _ptr(u2), T_do, nthreads,
                       cnt.ctypes.data_as(_i64p))
    return s2, u2, T, cnt


def run(cfg, s, u, nsteps, T_do=None, TT=0.0, step_no=0, nthreads=1, nn2=None):
    """nsteps steps with the lagged-dt protocol.  Returns (s, u, T_do, TT, step, counters).
    nn2: the neutral-coupling source, K (x, y, z) triples (add_MK's nn2), or None."""
    s = np.array(s, dtype=np.float64, order="C")
    u = np.array(u, dtype=np.float64, order="C")
    tdo = C.c_double(cfg.dt_first if T_do is None else T_do)
    tt = C.c_double(TT)
    st = C.c_int64(step_no)
    cnt = np.zeros(10, dtype=np.int64)
    src = None if nn2 is None else np.ascontiguousarray(nn2, dtype=np.float64).reshape(-1, 3)
    lib().ora_set_neutral(None if src is None else src.ctypes.data)
    try:
        rc = lib().ora_run(C.byref(cfg), _ptr(s), _ptr(u), nsteps, C.byref(tdo), C.byref(tt),
                           C.byref(st), nthreads, cnt.ctypes.data_as(_i64p))
    finally:
        lib().ora_set_neutral(None)
    if rc != 0:
        raise RuntimeError(f"ora_run failed: {rc}")
    return s, u, tdo.value, tt.value, st.value, cnt


def step_margin(cfg, s, u, T_do, nthreads=1):
    """One step like step(), plus two per-cell diagnostics of the exact
    solver's faces: the bisection margin, the smallest | |res| - tol | / tol
    over the bisection stopping tests (devtwo), and the pattern margin, the
    smallest distance of Udf to a wave-pattern threshold relative to
    cI + cII, over faces with unequal states (1e300 where none applies).
    Returns (s2, u2, new_dt, bisect_margin[K], pattern_margin[K])."""
    margin = np.empty(cfg.N * cfg.M)
    pmargin = np.empty(cfg.N * cfg.M)
    lib().ora_set_margin(margin.ctypes.data, pmargin.ctypes.data)
    try:
        s2, u2, T, _ = step(cfg, s, u, T_do, nthreads)
    finally:
        lib().ora_set_margin(None, None)
    return s2, u2, T, margin, pmargin


def max_threads():
    return lib().ora_max_threads()


# ---------------------------------------------------------------- reference

REF_KERNEL_TVD, REF_ADD_MK, REF_ADD2 = 0, 1, 2


def ref_set(cfg):
    ref().ref_set_params(cfg.N, cfg.M, cfg.x_min, cfg.x_max, cfg.y_max, cfg.gamma, cfg.cfl)


def ref_face(which, sL, uL, sR, uR, n1, n2, rad):
    a = [np.ascontiguousarray(v, dtype=np.float64) for v in (sL, uL, sR, uR)]
    out = np.zeros(4)
    t = ref().ref_face(which, _ptr(a[0]), _ptr(a[1]), _ptr(a[2]), _ptr(a[3]), n1, n2, rad, _ptr(out))
    return t, out


def ref_face_q(which, sL, uL, sR, uR, QL, QR, n1, n2, rad):
    """The reference's face with a passive scalar: which 1 HLLC_2d_Korolkov_b_s
    (metod 2, its PQ), 5 HLLCQ_Korolkov_2D.  Returns (dt, out[5])."""
    a = [np.ascontiguousarray(v, dtype=np.float64) for v in (sL, uL, sR, uR)]
    out = np.zeros(5)
    t = ref().ref_face_q(which, _ptr(a[0]), _ptr(a[1]), _ptr(a[2]), _ptr(a[3]), QL, QR, n1, n2, rad, _ptr(out))
    return t, out


def ref_run(kernel, cfg, s, u, nsteps, method=0, nthreads=1, nn2=None):
    """nsteps launches of the reference's own kernel (REF_KERNEL_TVD, REF_ADD_MK,
    ...) + funk_time; nn2: add_MK's neutral source (K x, y, z triples) or None
    for the zeros of the reference's main."""
    ref_set(cfg)
    s = np.array(s, dtype=np.float64, order="C")
    u = np.array(u, dtype=np.float64, order="C")
    tdo = C.c_double(cfg.dt_first)
    tt = C.c_double(0.0)
    st = C.c_longlong(0)
    src = None if nn2 is None else np.ascontiguousarray(nn2, dtype=np.float64).reshape(-1, 3)
    ref().ref_set_neutral(None if src is None else src.ctypes.data)
    try:
        ref().ref_kernel_run(kernel, _ptr(s), _ptr(u), nsteps, method, C.byref(tdo), C.byref(tt),
                             C.byref(st), nthreads)
    finally:
        ref().ref_set_neutral(None)
    return s, u, tdo.value, tt.value, st.value


def inflow(cfg, s, u, s2, u2):
    """The oracle's characteristic inflow (add2_bound restated): column 0 of
    copies of (s2, u2) from the old (s, u) and the new column 1."""
    s2 = np.array(s2, dtype=np.float64, order="C")
    u2 = np.array(u2, dtype=np.float64, order="C")
    lib().ora_inflow(C.byref(cfg), _ptr(np.ascontiguousarray(s, dtype=np.float64)),
                     _ptr(np.ascontiguousarray(u, dtype=np.float64)), _ptr(s2), _ptr(u2))
    return s2, u2


def ref_bound(cfg, s, u, s2, u2):
    """The reference's own add2_bound (p_H = 7, inflow speed 1) on copies of
    (s2, u2)."""
    ref_set(cfg)
    s2 = np.array(s2, dtype=np.float64, order="C")
    u2 = np.array(u2, dtype=np.float64, order="C")
    ref().ref_bound(_ptr(np.ascontiguousarray(s, dtype=np.float64)), _ptr(np.ascontiguousarray(u, dtype=np.float64)),
                    _ptr(s2), _ptr(u2))
    return s2, u2


def have_ref_writers():
    return have_ref() and hasattr(ref(), "ref_print_file_mini")


def ref_print_file_mini(cfg, s, u, stride, soltime, path):
    """The reference's print_file_mini (kernel.cu:3109-3173) of (s, u) to path."""
    ref_set(cfg)
    ref().ref_print_file_mini(_ptr(np.ascontiguousarray(s, dtype=np.float64)),
                              _ptr(np.ascontiguousarray(u, dtype=np.float64)), stride, soltime, path.encode())


def ref_end_of_run(cfg, s, u, TT, stride, mach_inf, chi, name):
    """The end-of-run files of the reference's main (kernel.cu:4109-4221):
    name.bin, name_param_for_texplot.txt, name_param_for_texplot_mini.txt,
    name_param_y=0.txt, name_inform.txt."""
    ref_set(cfg)
    ref().ref_end_of_run(_ptr(np.ascontiguousarray(s, dtype=np.float64)),
                         _ptr(np.ascontiguousarray(u, dtype=np.float64)), TT, stride, mach_inf, chi, name.encode())


def ref_run_composed(cfg, s, u, nsteps, nthreads=1, T_do=None, TT=0.0, step_no=0):
    """The oracle's step loop with every face evaluated by the reference's own
    HLL / HLLC / Godunov functions (any configuration), from the clock
    (T_do, TT, step_no) (T_do None: cfg.dt_first).  Returns like run()."""
    ref_set(cfg)
    s = np.array(s, dtype=np.float64, order="C")
    u = np.array(u, dtype=np.float64, order="C")
    tdo = C.c_double(cfg.dt_first if T_do is None else T_do)
    tt = C.c_double(TT)
    st = C.c_int64(step_no)
    cnt = np.zeros(10, dtype=np.int64)
    rc = ref().ora_run(C.byref(cfg), _ptr(s), _ptr(u), nsteps, C.byref(tdo), C.byref(tt), C.byref(st),
                       nthreads, cnt.ctypes.data_as(_i64p))
    if rc != 0:
        raise RuntimeError(f"ora_run failed: {rc}")
    return s, u, tdo.value, tt.value, st.value, cnt
