"""Build libasteriy_gb300.so in-tree with nvcc for sm_103a.

Every translation unit is compiled in parallel with
  nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo
and linked into asteriy_2d_gb300/libasteriy_gb300.so (git-ignored).
Usage: python -m asteriy_2d_gb300.build [--ptxas-verbose]
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libasteriy_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["api.cu", "step_f64.cu", "step_f32.cu", "step_raw.cu", "batch.cu",
           "batch_f64_s0.cu", "batch_f64_s1.cu", "batch_f64_s2.cu", "batch_f32_s0.cu", "batch_f32_s1.cu",
           "batch_f32_s2.cu", "batch_mixed.cu", "mlp_train.cu", "noalloc.cu", "add2.cu", "scalar.cu", "host_io.cpp"]
# per-file extra flags: the FP32 form uses the fast single-precision
# intrinsics (division, sqrt, pow); double-precision code is not affected
EXTRA = {"step_f32.cu": ["--use_fast_math"], "batch_f32_s0.cu": ["--use_fast_math"],
         "batch_f32_s1.cu": ["--use_fast_math"], "batch_f32_s2.cu": ["--use_fast_math"],
         "batch_mixed.cu": ["--use_fast_math"]}


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise FileNotFoundError("nvcc not found")


def _flags(ptxas_verbose=False):
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                "-I", os.path.join(ROOT, "include"), "-I", CSRC]
    if ptxas_verbose:
        f += ["-Xptxas", "-v"]
    # profiling build: per-phase SM cycle counters in the persistent
    # kernels (ast_get_phase_clocks); off in the product build
    if os.environ.get("AST_PHASE_CLOCKS", "0") == "1":
        f += ["-DAST_PHASE_CLOCKS"]
    return f


def _compile(src, ptxas_verbose):
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + _flags(ptxas_verbose) + EXTRA.get(src, []) + ["-c", path, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-x", "c++", "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-I",
               os.path.join(ROOT, "include"), "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(ptxas_verbose=False, quiet=True):
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, ptxas_verbose), SOURCES))
    objs = [o for o, _ in results]
    log = "".join(e for _, e in results)
    cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if not quiet or ptxas_verbose:
        sys.stderr.write(log)
    return LIB


if __name__ == "__main__":
    print(build(ptxas_verbose="--ptxas-verbose" in sys.argv, quiet=False))
