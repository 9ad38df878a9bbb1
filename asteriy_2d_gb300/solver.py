"""Python binding of libasteriy_gb300.so (the C ABI in include/asteriy_gb300.h).

The library is the product: every step runs in its CUDA kernels.  There is
no CPU path; loading fails loudly when the library has not been built.
"""
import ctypes as C
import os

import numpy as np

from . import abi as A

_lib = None
_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)

# every entry point of include/asteriy_gb300.h with (restype, argtypes)
SIGNATURES = {
    "ast_abi_version": (C.c_int, []),
    "ast_strerror": (C.c_char_p, [C.c_int]),
    "ast_last_error": (C.c_char_p, []),
    "ast_sizeof_config": (C.c_size_t, []),
    "ast_sizeof_stats": (C.c_size_t, []),
    "ast_config_default": (None, [C.POINTER(A.ast_config)]),
    "ast_config_check": (C.c_int, [C.POINTER(A.ast_config)]),
    "ast_create": (C.c_int, [C.POINTER(A.ast_config), C.POINTER(C.c_void_p)]),
    "ast_destroy": (C.c_int, [C.c_void_p]),
    "ast_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ast_set_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "ast_get_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "ast_set_clock": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_int64]),
    "ast_get_clock": (C.c_int, [C.c_void_p, _dp, _dp, C.POINTER(C.c_int64)]),
    "ast_step": (C.c_int, [C.c_void_p, C.c_int]),
    "ast_step_host": (C.c_int, [C.c_void_p] * 5),
    "ast_step_host_n": (C.c_int, [C.c_void_p, C.c_int] + [C.c_void_p] * 4),
    "ast_set_neutral": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "ast_add_mk_raw": (C.c_int, [C.c_void_p] * 9 + [C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    "ast_synchronize": (C.c_int, [C.c_void_p]),
    "ast_get_stats": (C.c_int, [C.c_void_p, C.POINTER(A.ast_stats), C.c_int]),
    "ast_get_phase_clocks": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.c_int]),
    "ast_set_scalar": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "ast_get_scalar": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "ast_device_state": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_int64), C.POINTER(C.c_int)]),
    "ast_step_raw": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.c_void_p, C.c_int, C.POINTER(A.ast_config), C.c_void_p]),
    "ast_funk_time": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ast_add2_raw": (C.c_int, [C.c_void_p] * 7 + [C.c_int, C.c_int, C.POINTER(A.ast_config), C.c_void_p]),
    "ast_inflow_raw": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(A.ast_config),
                                 C.c_void_p]),
    "ast_step_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.POINTER(A.ast_config), C.c_void_p]),
    "ast_fill_blast": (C.c_int, [C.POINTER(A.ast_config), C.c_double, C.c_double, C.c_double, _dp, _dp]),
    "ast_fill_wind": (C.c_int, [C.POINTER(A.ast_config), C.c_double, C.c_double, C.c_double, C.c_double,
                                C.c_double, C.c_double, C.c_double, C.c_double, C.c_uint64, _dp, _dp]),
    "ast_write_bin": (C.c_int, [C.POINTER(A.ast_config), _dp, _dp, C.c_char_p]),
    "ast_read_bin": (C.c_int, [C.POINTER(A.ast_config), _dp, _dp, C.c_char_p]),
    "ast_write_tecplot": (C.c_int, [C.POINTER(A.ast_config), _dp, _dp, C.c_int, C.c_double, C.c_char_p]),
    "ast_write_tecplot_final": (C.c_int, [C.POINTER(A.ast_config), _dp, _dp, C.c_int, C.c_char_p]),
    "ast_write_axis": (C.c_int, [C.POINTER(A.ast_config), _dp, _dp, C.c_char_p]),
    "ast_write_inform": (C.c_int, [C.POINTER(A.ast_config), C.c_double, C.c_double, C.c_double, C.c_char_p]),
    "ast_probe": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.c_int, _dp, _dp]),
    "ast_set_mlp": (C.c_int, [C.c_void_p, _fp]),
    "ast_batch_create": (C.c_int, [C.POINTER(A.ast_config), C.c_int, C.POINTER(C.c_void_p)]),
    "ast_batch_destroy": (C.c_int, [C.c_void_p]),
    "ast_batch_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ast_batch_set_state": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int]),
    "ast_batch_get_state": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int]),
    "ast_batch_set_clock": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int64]),
    "ast_batch_get_clock": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, C.POINTER(C.c_int64)]),
    "ast_batch_step": (C.c_int, [C.c_void_p, C.c_int]),
    "ast_batch_synchronize": (C.c_int, [C.c_void_p]),
    "ast_batch_get_stats": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(A.ast_stats), C.c_int]),
    "ast_batch_set_mlp": (C.c_int, [C.c_void_p, _fp]),
    "ast_batch_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int)]),
    "ast_batch_autotune": (C.c_int, [C.c_void_p, C.c_int]),
    "ast_batch_num_classes": (C.c_int, [C.c_void_p]),
    "ast_batch_set_mixed": (C.c_int, [C.c_void_p, C.c_int]),
    "ast_batch_get_mixed": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), _fp, _fp]),
    "ast_batch_class": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                  C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), _fp]),
    "ast_batch_set_schedule": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "ast_batch_set_tiles": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "ast_problem_set": (C.c_int, [C.c_uint64, C.c_int, C.c_int, C.POINTER(A.ast_problem)]),
    "ast_problem_fill": (C.c_int, [C.POINTER(A.ast_problem), _dp, _dp]),
    "ast_record_start": (C.c_int, [C.c_void_p, C.c_int64, C.c_int, C.c_double]),
    "ast_record_stop": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "ast_record_read": (C.c_int, [C.c_void_p, _fp, C.c_int64]),
    "ast_mlp_init": (C.c_int, [_fp, C.c_int64, C.c_uint64, _fp]),
    "ast_mlp_grad": (C.c_int, [_fp, _fp, C.c_int64, _fp, _fp]),
    "ast_mlp_forward": (C.c_int, [_fp, _fp, C.c_int64, C.c_int, _fp]),
    "ast_mlp_forward_tc": (C.c_int, [_fp, _fp, C.c_int64, C.c_int, _fp]),
    "ast_mlp_train": (C.c_int, [_fp, C.c_int64, C.c_int, C.c_int, C.c_float, C.c_uint64, _fp, _fp]),
}


class AstError(RuntimeError):
    def __init__(self, code, where):
        lib = load()
        msg = lib.ast_strerror(code).decode()
        detail = lib.ast_last_error().decode()
        super().__init__(f"{where}: {msg} ({code}) {detail}")
        self.code = code


def load(path=None):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or A.LIB_PATH
    if not os.path.exists(path):
        raise FileNotFoundError(
            f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc, where):
    if rc != A.AST_OK:
        raise AstError(rc, where)


def _dptr(a):
    return a.ctypes.data_as(_dp)


def _fptr(a):
    return a.ctypes.data_as(_fp)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


# ---------------------------------------------------------------- learned start value

def mlp_init(samples, seed=7):
    samples = _f32(samples)
    params = np.zeros(A.AST_MLP_NPARAM, dtype=np.float32)
    check(load().ast_mlp_init(_fptr(samples), len(samples), seed, _fptr(params)), "ast_mlp_init")
    return params


def mlp_grad(params, samples):
    params, samples = _f32(params), _f32(samples)
    grad = np.zeros(A.AST_MLP_NPARAM, dtype=np.float32)
    loss = C.c_float()
    check(load().ast_mlp_grad(_fptr(params), _fptr(samples), len(samples), _fptr(grad), C.byref(loss)),
          "ast_mlp_grad")
    return grad, loss.value


def mlp_forward(params, x):
    params = _f32(params)
    x = _f32(x)
    y = np.zeros(len(x), dtype=np.float32)
    check(load().ast_mlp_forward(_fptr(params), _fptr(x), len(x), x.shape[1], _fptr(y)), "ast_mlp_forward")
    return y


def mlp_forward_tc(params, x):
    """The step kernel's tensor-core inference on given feature rows."""
    params = _f32(params)
    x = _f32(x)
    y = np.zeros(len(x), dtype=np.float32)
    check(load().ast_mlp_forward_tc(_fptr(params), _fptr(x), len(x), x.shape[1], _fptr(y)), "ast_mlp_forward_tc")
    return y


def mlp_train(samples, params, epochs=10, batch=8192, lr=3e-3, seed=7):
    samples = _f32(samples)
    params = _f32(params).copy()
    losses = np.zeros(epochs, dtype=np.float32)
    check(load().ast_mlp_train(_fptr(samples), len(samples), epochs, batch, lr, seed, _fptr(params),
                               _fptr(losses)), "ast_mlp_train")
    return params, losses


def fill_blast(cfg, p_in=10.0, p_out=0.1, radius=0.2):
    K = cfg.N * cfg.M
    s = np.empty((K, 2))
    u = np.empty((K, 2))
    check(load().ast_fill_blast(C.byref(cfg), p_in, p_out, radius, _dptr(s), _dptr(u)), "ast_fill_blast")
    return s, u


def fill_wind(cfg, r_w=0.05, rho_w=1.0, v_w=10.0, mach_w=10.0, rho_inf=1.0, p_inf=None, v_inf=-2.0,
              noise=0.01, seed=20261203):
    K = cfg.N * cfg.M
    s = np.empty((K, 2))
    u = np.empty((K, 2))
    if p_inf is None:
        p_inf = 1.0 / cfg.gamma
    check(load().ast_fill_wind(C.byref(cfg), r_w, rho_w, v_w, mach_w, rho_inf, p_inf, v_inf, noise, seed,
                               _dptr(s), _dptr(u)), "ast_fill_wind")
    return s, u


def write_bin(cfg, s, u, path):
    check(load().ast_write_bin(C.byref(cfg), _dptr(np.ascontiguousarray(s)), _dptr(np.ascontiguousarray(u)),
                               os.fsencode(path)), "ast_write_bin")


def read_bin(cfg, path):
    K = cfg.N * cfg.M
    s = np.empty((K, 2))
    u = np.empty((K, 2))
    check(load().ast_read_bin(C.byref(cfg), _dptr(s), _dptr(u), os.fsencode(path)), "ast_read_bin")
    return s, u


def write_tecplot(cfg, s, u, path, stride=2, soltime=0.0):
    check(load().ast_write_tecplot(C.byref(cfg), _dptr(np.ascontiguousarray(s)), _dptr(np.ascontiguousarray(u)),
                                   stride, soltime, os.fsencode(path)), "ast_write_tecplot")


def write_tecplot_final(cfg, s, u, path, stride=2):
    check(load().ast_write_tecplot_final(C.byref(cfg), _dptr(np.ascontiguousarray(s)),
                                         _dptr(np.ascontiguousarray(u)), stride, os.fsencode(path)),
          "ast_write_tecplot_final")


def write_axis(cfg, s, u, path):
    check(load().ast_write_axis(C.byref(cfg), _dptr(np.ascontiguousarray(s)), _dptr(np.ascontiguousarray(u)),
                                os.fsencode(path)), "ast_write_axis")


def write_inform(cfg, TT, path, mach_inf=0.0, chi=0.0):
    check(load().ast_write_inform(C.byref(cfg), TT, mach_inf, chi, os.fsencode(path)), "ast_write_inform")


def write_probe_series(path, series):
    """One watch cell's samples as the reference's "TT rho" lines."""
    with open(path, "w") as f:
        for tt, rho in series:
            f.write("%g %g\n" % (tt, rho))


class Solver:
    """One r-z problem resident on the GPU (the ast_solver object)."""

    def __init__(self, cfg, stream=None):
        self.lib = load()
        self.cfg = cfg.copy()
        h = C.c_void_p()
        check(self.lib.ast_create(C.byref(self.cfg), C.byref(h)), "ast_create")
        self.h = h
        if stream is not None:
            check(self.lib.ast_set_stream(self.h, C.c_void_p(stream)), "ast_set_stream")

    def close(self):
        if getattr(self, "h", None):
            self.lib.ast_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def K(self):
        return self.cfg.N * self.cfg.M

    def set_state(self, s, u):
        s = np.ascontiguousarray(s, dtype=np.float64)
        u = np.ascontiguousarray(u, dtype=np.float64)
        assert s.shape == (self.K, 2) and u.shape == (self.K, 2)
        check(self.lib.ast_set_state(self.h, s.ctypes.data, u.ctypes.data, 0), "ast_set_state")

    def set_state_device(self, s_ptr, u_ptr):
        check(self.lib.ast_set_state(self.h, C.c_void_p(s_ptr), C.c_void_p(u_ptr), 1), "ast_set_state")

    def get_state(self):
        s = np.empty((self.K, 2))
        u = np.empty((self.K, 2))
        check(self.lib.ast_get_state(self.h, s.ctypes.data, u.ctypes.data, 0), "ast_get_state")
        return s, u

    def get_state_device(self, s_ptr, u_ptr):
        check(self.lib.ast_get_state(self.h, C.c_void_p(s_ptr), C.c_void_p(u_ptr), 1), "ast_get_state")

    def set_clock(self, T_do, TT=0.0, step=0):
        check(self.lib.ast_set_clock(self.h, T_do, TT, step), "ast_set_clock")

    def clock(self):
        a, b, c = C.c_double(), C.c_double(), C.c_int64()
        check(self.lib.ast_get_clock(self.h, C.byref(a), C.byref(b), C.byref(c)), "ast_get_clock")
        return a.value, b.value, c.value

    def set_neutral(self, nn2):
        """The neutral-coupling momentum source (add_MK's nn2): K (x, y, z)
        triples, or None to remove it."""
        if nn2 is None:
            check(self.lib.ast_set_neutral(self.h, None, 0), "ast_set_neutral")
            return
        a = np.ascontiguousarray(nn2, dtype=np.float64).reshape(self.K, 3)
        check(self.lib.ast_set_neutral(self.h, a.ctypes.data, 0), "ast_set_neutral")

    def set_neutral_device(self, ptr):
        check(self.lib.ast_set_neutral(self.h, C.c_void_p(ptr), 1), "ast_set_neutral")

    def step_host_n(self, n, s_a, u_a, s_b, u_b):
        """n host-array steps ping-ponging between two pairs of (K, 2)
        float64 arrays given by address (ast_step_host_n)."""
        check(self.lib.ast_step_host_n(self.h, n, C.c_void_p(s_a), C.c_void_p(u_a), C.c_void_p(s_b),
                                       C.c_void_p(u_b)), "ast_step_host_n")

    def step_host(self, s_in, u_in, s_out, u_out):
        """One step from host arrays to host arrays (ast_step_host): the
        addresses of four (K, 2) float64 arrays; page-locked arrays are
        pipelined by bands, others are copied in, stepped and copied out."""
        check(self.lib.ast_step_host(self.h, C.c_void_p(s_in), C.c_void_p(u_in), C.c_void_p(s_out),
                                     C.c_void_p(u_out)), "ast_step_host")

    def step(self, n=1, sync=True):
        check(self.lib.ast_step(self.h, n), "ast_step")
        if sync:
            self.synchronize()

    def synchronize(self):
        check(self.lib.ast_synchronize(self.h), "ast_synchronize")

    def stats(self, reset=False):
        st = A.ast_stats()
        check(self.lib.ast_get_stats(self.h, C.byref(st), int(reset)), "ast_get_stats")
        return {name: getattr(st, name) for name, _ in st._fields_ if name != "reserved"}

    def set_scalar(self, q):
        """The passive scalar (K = N*M FP64 values, index m*N + n), or None
        to remove it (ast_set_scalar)."""
        if q is None:
            check(self.lib.ast_set_scalar(self.h, None, 0), "ast_set_scalar")
            return
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1)
        assert q.size == self.cfg.N * self.cfg.M
        check(self.lib.ast_set_scalar(self.h, q.ctypes.data, 0), "ast_set_scalar")

    def get_scalar(self):
        q = np.empty(self.cfg.N * self.cfg.M, dtype=np.float64)
        check(self.lib.ast_get_scalar(self.h, q.ctypes.data, 0), "ast_get_scalar")
        return q

    def phase_clocks(self, reset=False):
        """Profiling builds (AST_PHASE_CLOCKS=1 at build time): SM cycles per
        phase of the persistent FP32 kernel, summed over CTAs, with the CTA
        and tile counts (ast_get_phase_clocks)."""
        out = (C.c_uint64 * 8)()
        check(self.lib.ast_get_phase_clocks(self.h, out, int(reset)), "ast_get_phase_clocks")
        names = ("arrival", "ghost", "faces", "queue", "update", "report", "ctas", "tiles")
        return dict(zip(names, (int(v) for v in out)))

    def set_mlp(self, params):
        params = _f32(params)
        assert params.shape == (A.AST_MLP_NPARAM,)
        check(self.lib.ast_set_mlp(self.h, _fptr(params)), "ast_set_mlp")

    def probe(self, cells):
        """Density at the watch cells (k = m*N + n) and the time TT."""
        cells = np.ascontiguousarray(cells, dtype=np.int64)
        rho = np.zeros(len(cells))
        tt = C.c_double()
        check(self.lib.ast_probe(self.h, cells.ctypes.data_as(C.POINTER(C.c_int64)), len(cells), _dptr(rho),
                                 C.byref(tt)), "ast_probe")
        return rho, tt.value

    def record_start(self, capacity, every=1, min_strength=0.0):
        check(self.lib.ast_record_start(self.h, capacity, every, min_strength), "ast_record_start")
        self._rec_cap = capacity

    def record_stop(self):
        n = C.c_int64()
        check(self.lib.ast_record_stop(self.h, C.byref(n)), "ast_record_stop")
        stored = min(n.value, self._rec_cap)
        out = np.zeros((stored, A.AST_RECORD_FLOATS), dtype=np.float32)
        if stored:
            check(self.lib.ast_record_read(self.h, _fptr(out), stored), "ast_record_read")
        return out, n.value

    def device_state(self):
        p, ld, el = C.c_void_p(), C.c_int64(), C.c_int()
        check(self.lib.ast_device_state(self.h, C.byref(p), C.byref(ld), C.byref(el)), "ast_device_state")
        return p.value, ld.value, el.value


def step_raw(s, u, s2, u2, T, T_do, TT, cfg, method=1, stream=None):
    """ast_step_raw on device pointers (ints), the Kernel_TVD drop-in."""
    check(load().ast_step_raw(C.c_void_p(s), C.c_void_p(u), C.c_void_p(s2), C.c_void_p(u2), C.c_void_p(T),
                              C.c_void_p(T_do), C.c_void_p(TT), method, C.byref(cfg),
                              C.c_void_p(stream) if stream else None), "ast_step_raw")


def add_mk_raw(s, u, s2, u2, nn2, T, T_do, cfg, stream=None):
    """ast_add_mk_raw on device pointers (ints; nn2 may be 0 for none), the
    add_MK drop-in with its neutral-coupling source."""
    check(load().ast_add_mk_raw(C.c_void_p(s), C.c_void_p(u), C.c_void_p(s2), C.c_void_p(u2), None,
                                C.c_void_p(nn2) if nn2 else None, None, C.c_void_p(T), C.c_void_p(T_do), 0, 0,
                                C.byref(cfg), C.c_void_p(stream) if stream else None), "ast_add_mk_raw")


def add2_raw(s, u, s2, u2, T, T_do, TT, cfg, method=1, stream=None):
    """ast_add2_raw on device pointers (ints), the add2 drop-in."""
    check(load().ast_add2_raw(C.c_void_p(s), C.c_void_p(u), C.c_void_p(s2), C.c_void_p(u2), C.c_void_p(T),
                              C.c_void_p(T_do), C.c_void_p(TT), method, 0, C.byref(cfg),
                              C.c_void_p(stream) if stream else None), "ast_add2_raw")


def inflow_raw(s, u, s2, u2, cfg, stream=None):
    """ast_inflow_raw on device pointers (ints), the add2_bound drop-in."""
    check(load().ast_inflow_raw(C.c_void_p(s), C.c_void_p(u), C.c_void_p(s2), C.c_void_p(u2), C.byref(cfg),
                                C.c_void_p(stream) if stream else None), "ast_inflow_raw")


def funk_time(T, T_do, TT, i, stream=None):
    check(load().ast_funk_time(C.c_void_p(T), C.c_void_p(T_do), C.c_void_p(TT), C.c_void_p(i),
                               C.c_void_p(stream) if stream else None), "ast_funk_time")


def step_noalloc(s, u, s2, u2, T_do, TT, step, cfg, status=None, stream=None):
    """ast_step_noalloc on device pointers (ints): one step plus the dt shift
    in one launch, with no device allocation (static scratch)."""
    check(load().ast_step_noalloc(C.c_void_p(s), C.c_void_p(u), C.c_void_p(s2), C.c_void_p(u2), C.c_void_p(T_do),
                                  C.c_void_p(TT), C.c_void_p(step), C.c_void_p(status) if status else None,
                                  C.byref(cfg), C.c_void_p(stream) if stream else None), "ast_step_noalloc")


def problem_set(seed=64, n=64, precision=A.PREC_FP32):
    """The seeded benchmark problem set (ast_problem_set): a list of
    ast_problem structures (config, setup, Mach number, noise seed)."""
    arr = (A.ast_problem * n)()
    check(load().ast_problem_set(seed, n, precision, arr), "ast_problem_set")
    return [arr[i] for i in range(n)]


def problem_fill(prob):
    """Initial state (s, u) of one drawn problem."""
    K = prob.cfg.N * prob.cfg.M
    s = np.empty((K, 2))
    u = np.empty((K, 2))
    check(load().ast_problem_fill(C.byref(prob), _dptr(s), _dptr(u)), "ast_problem_fill")
    return s, u


TILE_SHAPES = ((32, 16), (16, 16), (64, 8))
# batch schedules: one CTA per tile with each tile shape, then the
# persistent batch kernel and one persistent kernel per problem (FP32)
SCHEDULES = ("32x16", "16x16", "64x8", "persistent", "per-problem")
PERSISTENT, PER_PROBLEM = 3, 4


class Batch:
    """Many independent r-z problems advanced together (the ast_batch object)."""

    def __init__(self, cfgs, stream=None):
        self.lib = load()
        n = len(cfgs)
        self.cfgs = [c.copy() for c in cfgs]
        arr = (A.ast_config * n)(*self.cfgs)
        h = C.c_void_p()
        check(self.lib.ast_batch_create(arr, n, C.byref(h)), "ast_batch_create")
        self.h = h
        if stream is not None:
            check(self.lib.ast_batch_set_stream(self.h, C.c_void_p(stream)), "ast_batch_set_stream")

    def close(self):
        if getattr(self, "h", None):
            self.lib.ast_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __len__(self):
        return len(self.cfgs)

    def set_state(self, i, s, u):
        K = self.cfgs[i].N * self.cfgs[i].M
        s = np.ascontiguousarray(s, dtype=np.float64)
        u = np.ascontiguousarray(u, dtype=np.float64)
        assert s.shape == (K, 2) and u.shape == (K, 2)
        check(self.lib.ast_batch_set_state(self.h, i, s.ctypes.data, u.ctypes.data, 0), "ast_batch_set_state")

    def set_state_device(self, i, s_ptr, u_ptr):
        check(self.lib.ast_batch_set_state(self.h, i, C.c_void_p(s_ptr), C.c_void_p(u_ptr), 1),
              "ast_batch_set_state")

    def get_state(self, i):
        K = self.cfgs[i].N * self.cfgs[i].M
        s = np.empty((K, 2))
        u = np.empty((K, 2))
        check(self.lib.ast_batch_get_state(self.h, i, s.ctypes.data, u.ctypes.data, 0), "ast_batch_get_state")
        return s, u

    def get_state_device(self, i, s_ptr, u_ptr):
        check(self.lib.ast_batch_get_state(self.h, i, C.c_void_p(s_ptr), C.c_void_p(u_ptr), 1),
              "ast_batch_get_state")

    def set_clock(self, i, T_do, TT=0.0, step=0):
        check(self.lib.ast_batch_set_clock(self.h, i, T_do, TT, step), "ast_batch_set_clock")

    def clock(self, i):
        a, b, c = C.c_double(), C.c_double(), C.c_int64()
        check(self.lib.ast_batch_get_clock(self.h, i, C.byref(a), C.byref(b), C.byref(c)), "ast_batch_get_clock")
        return a.value, b.value, c.value

    def step(self, n=1, sync=True):
        check(self.lib.ast_batch_step(self.h, n), "ast_batch_step")
        if sync:
            self.synchronize()

    def synchronize(self):
        check(self.lib.ast_batch_synchronize(self.h), "ast_batch_synchronize")

    def stats(self, i, reset=False):
        st = A.ast_stats()
        check(self.lib.ast_batch_get_stats(self.h, i, C.byref(st), int(reset)), "ast_batch_get_stats")
        return {name: getattr(st, name) for name, _ in st._fields_ if name != "reserved"}

    def set_mlp(self, params):
        params = _f32(params)
        assert params.shape == (A.AST_MLP_NPARAM,)
        check(self.lib.ast_batch_set_mlp(self.h, _fptr(params)), "ast_batch_set_mlp")

    def info(self):
        cells, tiles, launches = C.c_int64(), C.c_int64(), C.c_int()
        check(self.lib.ast_batch_info(self.h, C.byref(cells), C.byref(tiles), C.byref(launches)), "ast_batch_info")
        return {"cells": cells.value, "tiles": tiles.value, "launches_per_step": launches.value}

    def classes(self):
        """Per (flux, recon) class: problems, tile shape in use, and the
        autotuner's ms per step of each built shape."""
        out = []
        for k in range(self.lib.ast_batch_num_classes(self.h)):
            v = [C.c_int() for _ in range(6)]
            ms = np.zeros(len(SCHEDULES), dtype=np.float32)
            check(self.lib.ast_batch_class(self.h, k, *[C.byref(x) for x in v], _fptr(ms)), "ast_batch_class")
            out.append({"flux": v[0].value, "recon": v[1].value, "problems": v[2].value,
                        "schedule": v[3].value, "tile": (v[4].value, v[5].value),
                        "ms_per_schedule": [float(x) for x in ms]})
        return out

    def autotune(self, trials=3):
        check(self.lib.ast_batch_autotune(self.h, trials), "ast_batch_autotune")
        return self.classes()

    def set_mixed(self, mode):
        """One launch per step for the whole batch (ast_batch_set_mixed):
        0 one launch per class, 1 (or True) a CTA per tile, 2 the persistent
        kernel."""
        check(self.lib.ast_batch_set_mixed(self.h, int(mode)), "ast_batch_set_mixed")

    def mixed(self):
        """(one-launch mode: 0 off, 1 CTA per tile, 2 persistent; tuner ms per
        step of the faster one-launch mode; of the per-class launches)."""
        on = C.c_int()
        a = np.zeros(1, dtype=np.float32)
        b = np.zeros(1, dtype=np.float32)
        check(self.lib.ast_batch_get_mixed(self.h, C.byref(on), _fptr(a), _fptr(b)), "ast_batch_get_mixed")
        return int(on.value), float(a[0]), float(b[0])

    def set_tiles(self, cls, tile_z, tile_r):
        check(self.lib.ast_batch_set_tiles(self.h, cls, tile_z, tile_r), "ast_batch_set_tiles")

    def set_schedule(self, cls, schedule):
        check(self.lib.ast_batch_set_schedule(self.h, cls, schedule), "ast_batch_set_schedule")
