"""C-ABI library: it loads without a GPU, exports every declared entry point,
its structures match the ctypes mirror, and its host-only functions
(configuration, initial conditions, file formats) behave as specified."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from asteriy_2d_gb300 import abi as A
from asteriy_2d_gb300 import problems, solver
from conftest import ROOT


def header_functions():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"\b(ast_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    lib = solver.load()
    names = header_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) <= set(solver.SIGNATURES), set(names) - set(solver.SIGNATURES)


def test_struct_layouts_match():
    lib = solver.load()
    assert lib.ast_sizeof_config() == C.sizeof(A.ast_config)
    assert lib.ast_sizeof_stats() == C.sizeof(A.ast_stats)
    assert lib.ast_abi_version() == 1


def test_config_default_matches_reference_macros():
    c = A.ast_config()
    solver.load().ast_config_default(C.byref(c))
    d = A.default_config()
    assert c.describe() == d.describe()
    assert (c.gamma, c.cfl, c.dt_first, c.dt_cap, c.p_floor) == (5.0 / 3.0, 0.05, 1e-9, 1000.0, 1e-6)
    assert c.riemann_tol == 10e-10


@pytest.mark.parametrize("field,value", [("N", 2), ("M", 0), ("gamma", 1.0), ("cfl", 0.0), ("flux", 7),
                                         ("riemann_max_iter", 0), ("x_max", -5.0),
                                         ("persistent", 3), ("copy_wait_polls", -1), ("skip_uniform", 2), ("skip_uniform", -1),
                                         ("neutral_nh", float("nan")), ("neutral_kn", float("inf"))])
def test_config_check_rejects(field, value):
    c = problems.blast_config(64, 32)
    setattr(c, field, value)
    assert solver.load().ast_config_check(C.byref(c)) == A.AST_ERR_INVALID
    h = C.c_void_p()
    assert solver.load().ast_create(C.byref(c), C.byref(h)) == A.AST_ERR_INVALID


def test_null_solver_is_refused():
    L = solver.load()
    assert L.ast_set_neutral(None, None, 0) == A.AST_ERR_INVALID
    assert L.ast_step_host(None, None, None, None, None) == A.AST_ERR_INVALID
    assert L.ast_step_host_n(None, 1, None, None, None, None) == A.AST_ERR_INVALID
    assert L.ast_batch_set_mixed(None, 1) == A.AST_ERR_INVALID
    assert L.ast_batch_get_mixed(None, None, None, None) == A.AST_ERR_INVALID
    assert L.ast_batch_num_classes(None) == A.AST_ERR_INVALID
    c = problems.blast_config(64, 32)
    assert L.ast_add_mk_raw(None, None, None, None, None, None, None, None, None, 0, 0, C.byref(c), None) == \
        A.AST_ERR_INVALID


def test_fixed_side_needs_positive_state():
    c = problems.blast_config(64, 32)
    A.set_bc(c, A.Z_HI, A.BC_FIXED, 0.0, 1.0, 0.0, 0.0)
    assert solver.load().ast_config_check(C.byref(c)) == A.AST_ERR_INVALID


def test_fill_blast():
    c = problems.blast_config(64, 32)
    s, u = solver.fill_blast(c)
    x = -1.0 + np.arange(64) * (2.0 / 63)
    y = 1.0 / 64 + np.arange(32) * (1.0 / 32)
    X, Y = np.meshgrid(x, y)
    inside = np.sqrt(X * X + Y * Y).ravel() < 0.2
    assert np.all(s[inside, 1] == 10.0) and np.all(s[~inside, 1] == 0.1)
    assert np.all(s[:, 0] == 1.0) and np.all(u == 0.0)


def test_fill_wind_is_seeded_and_bounded():
    c = problems.wind_config(128, 64)
    s1, u1 = solver.fill_wind(c, seed=5)
    s2, _ = solver.fill_wind(c, seed=5)
    s3, _ = solver.fill_wind(c, seed=6)
    assert np.array_equal(s1, s2) and not np.array_equal(s1, s3)
    outside = u1[:, 0] == -2.0
    assert np.all(np.abs(s1[outside, 0] - 1.0) <= 0.01 + 1e-15)
    inside = ~outside
    assert inside.sum() > 0
    speed = np.hypot(u1[inside, 0], u1[inside, 1])
    assert np.allclose(speed, 10.0)


def test_bin_round_trip_and_format(tmp_path):
    c = problems.blast_config(16, 8)
    rng = np.random.default_rng(0)
    s = rng.random((128, 2))
    u = rng.random((128, 2))
    p = str(tmp_path / "state.bin")
    solver.write_bin(c, s, u, p)
    raw = np.fromfile(p, dtype=np.float64).reshape(-1, 6)
    assert raw.shape == (128, 6)
    assert np.array_equal(raw[:, 2:4], s) and np.array_equal(raw[:, 4:6], u)
    assert raw[1, 0] == -1.0 + 1 * (2.0 / 15) and raw[16, 1] == 1.0 / 16 + 1 * 1.0 / 8
    s2, u2 = solver.read_bin(c, p)
    assert np.array_equal(s, s2) and np.array_equal(u, u2)


def test_truncated_bin_is_an_io_error(tmp_path):
    c = problems.blast_config(16, 8)
    p = tmp_path / "short.bin"
    np.zeros(6 * 100).tofile(p)
    with pytest.raises(solver.AstError) as e:
        solver.read_bin(c, str(p))
    assert e.value.code == A.AST_ERR_IO


def test_tecplot_writer(tmp_path):
    c = problems.blast_config(16, 8)
    s, u = solver.fill_blast(c)
    p = str(tmp_path / "t.dat")
    solver.write_tecplot(c, s, u, p, stride=2, soltime=0.5)
    lines = open(p).read().splitlines()
    assert lines[0].startswith('TITLE = "HP"  VARIABLES = "X", "Y", "Ro", "P", "Vx", "Vy", "Mach", "omega"')
    assert "SOLUTIONTIME = 0.5, N = 32 , E = 21, F = FEPOINT, ET = quadrilateral" in lines[0]
    assert len(lines) == 1 + 32 + 21
    assert lines[-1] == "23 24 32 31"


def test_tecplot_final_writer(tmp_path):
    c = problems.blast_config(16, 8)
    rng = np.random.default_rng(3)
    s = 0.5 + rng.random((128, 2))
    u = rng.random((128, 2)) - 0.5
    p = str(tmp_path / "final.dat")
    solver.write_tecplot_final(c, s, u, p, stride=2)
    lines = open(p).read().splitlines()
    assert lines[0] == ('TITLE = "HP"  VARIABLES = "X", "Y", "Ro", "P", "Vx", "Vy", "Mach", "T", "Zav", '
                        'ZONE T = "HP", N = 32 , E = 21, F = FEPOINT, ET = quadrilateral')
    assert len(lines) == 1 + 32 + 21
    rows = np.array([[float(v) for v in ln.split()] for ln in lines[1:33]])
    # cell (n, m) = (2, 2): the sixth sampled cell of the second sampled row
    n, m, N = 2, 2, 16
    k = m * N + n
    dx, dy = 2.0 / 15, 1.0 / 8
    zav = (u[k + 1, 1] - u[k - 1, 1]) / (2 * dx) - (u[k + N, 0] - u[k - N, 0]) / (2 * dy)
    mach = np.sqrt((u[k, 0] ** 2 + u[k, 1] ** 2) / (c.gamma * s[k, 1] / s[k, 0]))
    r = rows[1 * 8 + 1]
    expect = [-1.0 + n * dx, 1.0 / 16 + m * dy, s[k, 0], s[k, 1], u[k, 0], u[k, 1], mach, s[k, 1] / s[k, 0], zav]
    assert np.allclose(r, expect, rtol=1e-5, atol=1e-6), (r, expect)
    assert rows[0, 8] == 0.0      # outer cell: no vorticity


def test_axis_and_inform_writers(tmp_path):
    c = problems.blast_config(16, 8)
    s, u = solver.fill_blast(c)
    p = str(tmp_path / "axis.txt")
    solver.write_axis(c, s, u, p)
    rows = np.loadtxt(p)
    assert rows.shape == (16, 7)
    assert np.allclose(rows[:, 0], -1.0 + np.arange(16) * 2.0 / 15, atol=1e-6)
    assert np.allclose(rows[:, 1], 1.0 / 16)
    assert np.allclose(rows[:, 6], 1.0 / np.sqrt(c.gamma * s[:16, 1] / s[:16, 0]), rtol=1e-5)
    q = str(tmp_path / "inform.txt")
    solver.write_inform(c, 0.25, q, mach_inf=2.0, chi=0.5)
    lines = open(q).read().splitlines()
    assert lines == ["TT = 0.25    N = 16   M = 8   K = 128",
                     "x_min = -1 x_max = 1 y_min = 0.0625 y_max = 1",
                     "M_inf = 2 chi_ = 0.5"]


def test_probe_series_file(tmp_path):
    p = str(tmp_path / "1_inStable.txt")
    solver.write_probe_series(p, [(0.125, 1.5), (0.25, 2.0)])
    assert open(p).read() == "0.125 1.5\n0.25 2\n"
