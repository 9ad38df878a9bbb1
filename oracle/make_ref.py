"""Build oracle/_ref/libastref.so from the reference's own sources.

TEST INFRASTRUCTURE ONLY.  Recipe:
  1. copy the listed line ranges of the reference, byte for byte, into
     oracle/_ref/ref_extract.inc (each range preceded by a #line directive
     naming its origin, and checked against the function it must start with),
     and the reference's file writers into oracle/_ref/ref_pfm.inc and
     ref_endrun.inc (compiled by oracle/ref_writers.cpp);
  2. compile oracle/ref_driver.cpp, which includes oracle/ref_shim.h and that
     file, with g++ -fopenmp -ffp-contract=off into oracle/_ref/libastref.so,
     together with the oracle's step loop (oracle/ast_oracle.c built with
     -DORA_WITH_REF) so that any configuration can be stepped with the
     reference's own face functions (the CPU baseline of the benchmark).

oracle/_ref/ is git-ignored.  The reference cannot be built as a binary
unmodified (kernel.cu:20 declares an add2 overload that is never defined and
is called at kernel.cu:3652, 3676), and it needs nvcc -rdc plus a GPU; only
its functions are compiled here, for the host.

Usage:  python oracle/make_ref.py [--src /path/to/reference] [--extract-only]
(or ASTERIY_REF_SRC=/path/to/reference in the environment)
With --extract-only the .inc is written but not compiled; build() on a
machine without the reference sources compiles an existing .inc.
"""
import argparse
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# the reference checkout: $ASTERIY_REF_SRC, else --src, else the checkout
# location of the machine this recipe was written on
DEFAULT_SRC = os.environ.get("ASTERIY_REF_SRC") or "/root/reference"

# (file, first line, last line, text the first line must contain)
RANGES = [
    ("Gas_Dinamic.cu", 249, 353, "double HLLCQ_Korolkov_2D("),
    ("Gas_Dinamic.cu", 858, 872, "int sign(double& x)"),
    ("kernel.cu", 22, 75, "double minmod(double x, double y)"),
    ("kernel.cu", 77, 86, "void lev("),
    ("kernel.cu", 128, 570, "double Godunov_Solver_Alexashov("),
    ("kernel.cu", 635, 765, "void newton("),
    ("kernel.cu", 767, 1079, "double HLLC_Aleksashov("),
    ("kernel.cu", 1399, 1523, "double HLL("),
    ("Gas_Dinamic.cu", 1604, 1826, "double HLLC_2d_Korolkov_b_s("),
    ("kernel.cu", 1525, 1536, "void funk_time("),
    ("kernel.cu", 1895, 1925, "void add2_bound("),
    ("kernel.cu", 1928, 2291, "void add2("),
    ("kernel.cu", 2293, 2511, "void add_MK("),
    ("kernel.cu", 2513, 3093, "void Kernel_TVD("),
]


# the reference's writers (host C++), for pinning the library's file writers:
# print_file_mini (the snapshot with Mach and vorticity) and the end-of-run
# block of main that writes the .bin dump, the mini Tecplot file with T and
# Zav, the axis line and the run summary; written to their own files
WRITER_RANGES = {
    "ref_pfm.inc": [("kernel.cu", 3109, 3173, "void print_file_mini(")],
    "ref_endrun.inc": [("kernel.cu", 4109, 4221, "ofstream fout;")],
}


def _copy_ranges(src, ranges, dst):
    chunks = []
    for fname, a, b, must in ranges:
        path = os.path.join(src, fname)
        with open(path, "rb") as f:
            lines = f.read().decode("latin-1").splitlines()
        first = lines[a - 1]
        if must not in first:
            raise RuntimeError(f"{fname}:{a} does not start {must!r}: {first!r}")
        chunks.append(f'#line {a} "{fname}"')
        chunks.extend(lines[a - 1:b])
    with open(dst, "wb") as f:
        f.write(("\n".join(chunks) + "\n").encode("latin-1"))
    return dst


def extract(src):
    os.makedirs(OUT, exist_ok=True)
    for name, ranges in WRITER_RANGES.items():
        _copy_ranges(src, ranges, os.path.join(OUT, name))
    chunks = []
    for fname, a, b, must in RANGES:
        path = os.path.join(src, fname)
        with open(path, "rb") as f:
            lines = f.read().decode("latin-1").splitlines()
        first = lines[a - 1]
        if must not in first:
            raise RuntimeError(f"{fname}:{a} does not start {must!r}: {first!r}")
        chunks.append(f'#line {a} "{fname}"')
        chunks.extend(lines[a - 1:b])
    text = "\n".join(chunks) + "\n"
    dst = os.path.join(OUT, "ref_extract.inc")
    with open(dst, "wb") as f:
        f.write(text.encode("latin-1"))
    return dst


def compile_ref(cxx="g++"):
    inc = os.path.join(OUT, "ref_extract.inc")
    if not os.path.exists(inc):
        raise FileNotFoundError(inc)
    so = os.path.join(OUT, "libastref.so")
    obj = os.path.join(OUT, "ast_oracle_ref.o")
    # the oracle's step loop, with every face evaluated by the reference's functions
    subprocess.run(["gcc", "-O2", "-std=c99", "-fopenmp", "-ffp-contract=off", "-fPIC", "-DORA_WITH_REF", "-c",
                    os.path.join(HERE, "ast_oracle.c"), "-o", obj], check=True)
    srcs = [os.path.join(HERE, "ref_driver.cpp")]
    if all(os.path.exists(os.path.join(OUT, n)) for n in WRITER_RANGES):
        srcs.append(os.path.join(HERE, "ref_writers.cpp"))
    cmd = [cxx, "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-w",
           "-I", HERE] + srcs + [obj, "-o", so]
    subprocess.run(cmd, check=True)
    return so


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", default=DEFAULT_SRC)
    ap.add_argument("--extract-only", action="store_true")
    args = ap.parse_args(argv)
    if os.path.isdir(args.src):
        extract(args.src)
    if not args.extract_only:
        print(compile_ref())
    return 0


if __name__ == "__main__":
    sys.exit(main())
