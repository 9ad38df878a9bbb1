"""The library's file writers against the reference's own writers, byte for
byte (CPU only).  tests/golden/writers.npz holds the bytes the reference's
print_file_mini (kernel.cu:3109-3173) and the end-of-run block of its main
(kernel.cu:4109-4221: the .bin dump, the mini Tecplot file with T and Zav,
the axis line and the run summary) write for a random 24x12 state, recorded
from the reference compiled for the host (tests/golden/make_golden.py).
Where that build is present the files are also written by it now and
compared on a second state."""
import os

import numpy as np
import pytest

import golden_configs as G
import pyoracle as O
from asteriy_2d_gb300 import solver
from conftest import golden


def ours(cfg, s, u, d, TT, mach_inf, chi, soltime):
    """The files of the library's writers: name -> bytes."""
    out = {}
    for stride in (2, 3):
        p = os.path.join(d, f"pfm{stride}.txt")
        solver.write_tecplot(cfg, s, u, p, stride=stride, soltime=soltime)
        out[f"pfm{stride}"] = open(p, "rb").read()
        p = os.path.join(d, f"final{stride}.txt")
        solver.write_tecplot_final(cfg, s, u, p, stride=stride)
        out[f"final{stride}"] = open(p, "rb").read()
    for name, fn in (("bin", lambda p: solver.write_bin(cfg, s, u, p)),
                     ("axis", lambda p: solver.write_axis(cfg, s, u, p)),
                     ("inform", lambda p: solver.write_inform(cfg, TT, p, mach_inf=mach_inf, chi=chi))):
        p = os.path.join(d, name)
        fn(p)
        out[name] = open(p, "rb").read()
    return out


KEYS = ["pfm2", "pfm3", "final2", "final3", "bin", "axis", "inform"]


@pytest.mark.parametrize("key", KEYS)
def test_writers_equal_reference_fixture(key, tmp_path):
    z = golden("writers.npz")
    cfg = G.writer_config()
    got = ours(cfg, z["s"], z["u"], str(tmp_path), float(z["TT"]), float(z["mach_inf"]), float(z["chi"]),
               float(z["soltime"]))
    assert got[key] == z[key].tobytes()


def test_bin_round_trip_of_reference_dump(tmp_path):
    z = golden("writers.npz")
    cfg = G.writer_config()
    p = str(tmp_path / "ref.bin")
    with open(p, "wb") as f:
        f.write(z["bin"].tobytes())
    s, u = solver.read_bin(cfg, p)
    assert np.array_equal(s, z["s"]) and np.array_equal(u, z["u"])


@pytest.mark.skipif(not O.have_ref_writers(), reason="the reference's writers are not built here")
def test_writers_equal_reference_live(tmp_path):
    cfg = G.writer_config(37, 19)
    s, u = G.random_state(37 * 19, np.random.default_rng(4111))
    u[:, 1] -= 0.2
    TT, mach_inf, chi, soltime = 1.5e-3, 2.0, 36.0, 3.0
    got = ours(cfg, s, u, str(tmp_path), TT, mach_inf, chi, soltime)
    ref = {}
    for stride in (2, 3):
        p = str(tmp_path / f"ref_pfm{stride}.txt")
        O.ref_print_file_mini(cfg, s, u, stride, soltime, p)
        ref[f"pfm{stride}"] = open(p, "rb").read()
        name = str(tmp_path / f"ref{stride}")
        O.ref_end_of_run(cfg, s, u, TT, stride, mach_inf, chi, name)
        ref[f"final{stride}"] = open(name + "_param_for_texplot_mini.txt", "rb").read()
        if stride == 2:
            ref["bin"] = open(name + ".bin", "rb").read()
            ref["axis"] = open(name + "_param_y=0.txt", "rb").read()
            ref["inform"] = open(name + "_inform.txt", "rb").read()
    for k in KEYS:
        assert got[k] == ref[k], k
