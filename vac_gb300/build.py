"""In-tree build of the native parts: ``vac_gb300/lib/libvacgpu.so`` (the
CUDA engine behind include/vacgpu.h, sm_103a) and the host driver.

Every translation unit is compiled for sm_103a only.  The FP64 path and the
time-loop control are built with ``-fmad=false`` and host code with
``-ffp-contract=off`` so no multiply-add is contracted where the reference's
FP64 operation order is reproduced.  The FP32-state (mixed) units are built
with ``--use_fast_math``: FP32 subnormals flush to zero and FP32 division
and square root are the approximate forms; the double arithmetic they
contain keeps IEEE division and square root (and, as in any default build,
may contract multiply-adds).
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(HERE, "lib", "obj")
LIB = os.path.join(LIBDIR, "libvacgpu.so")
BINDIR = os.path.join(HERE, "bin")
VACGB = os.path.join(BINDIR, "vacgb")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

# (source, extra flags)
UNITS = [
    ("sweep_fp64.cu", ["-fmad=false"]),
    ("roe_fp64.cu", ["-fmad=false"]),
    ("control.cu", ["-fmad=false"]),
    ("roe_mixed.cu", ["--use_fast_math"]),
    ("sweep_mixed.cu", ["--use_fast_math"]),
    ("vacgpu.cu", []),
    ("noalloc.cu", []),
    ("sweep_fused.cu", ["--use_fast_math"]),
    ("sweep_pair.cu", ["--use_fast_math"]),
    ("sweep_line2.cu", ["--use_fast_math"]),
    ("batch.cu", ["--use_fast_math"]),
    ("server.cu", []),
    ("diag.cu", []),
]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(src, extra, verbose):
    obj = os.path.join(OBJDIR, src.replace(".cu", ".o"))
    srcp = os.path.join(CSRC, src)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(HERE, "..", "include", "vacgpu.h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc(), ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler",
           "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr", "-c", srcp,
           "-o", obj] + extra
    if verbose:
        cmd.append("-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr))
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose=False):
    os.makedirs(OBJDIR, exist_ok=True)
    with ThreadPoolExecutor(len(UNITS)) as ex:
        objs = list(ex.map(lambda u: _compile(u[0], u[1], verbose), UNITS))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc(), ARCH, "-shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr)
    # the host program (a drop-in for VAC's `vac` on this path)
    src = os.path.join(HERE, "host", "vacgb.cpp")
    os.makedirs(BINDIR, exist_ok=True)
    if not os.path.exists(VACGB) or os.path.getmtime(VACGB) < max(
            os.path.getmtime(src), os.path.getmtime(LIB)):
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-pthread", src, "-o", VACGB,
               "-L" + LIBDIR, "-lvacgpu", "-ldl", "-Wl,-rpath,$ORIGIN/../lib"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("host program build failed:\n" + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
