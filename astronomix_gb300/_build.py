"""Build recipe of the CUDA library ``libamx.so`` (sm_103a only).

Each translation unit under ``csrc/`` is compiled by nvcc in parallel into
``_build/`` and linked into ``_lib/libamx.so`` next to this file.  A unit is
rebuilt when it, or any header of the library, is newer than its object.
"""

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libamx.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2", "--expt-relaxed-constexpr"]

# the slowest units first, so that the parallel build finishes early
SOURCES = ["fv_f32_schemes.cu", "fv_f64_schemes.cu", "fv_batch_f32.cu", "fv_batch_f32_alt.cu", "adjoint_f32.cu",
           "fv_f32_split_am.cu", "fv_f64_split_am.cu",
           "adjoint_f64.cu", "amx_api.cu", "fv_f32.cu", "fv_f64.cu", "fd.cu", "fd_f32.cu", "fd_f64.cu",
           "fv_batch_f64.cu", "batch.cu", "adjoint.cu", "gravity.cu", "gravity_f32.cu", "forcing.cu", "diag.cu"]

# FP32 FV kernels use approximate division and square root: the FP32 path is
# held to an L1 tolerance against FP64, while the FP64 units keep IEEE
# operations for round-off parity with the reference.
_FAST = ["-prec-div=false", "-prec-sqrt=false"]
EXTRA_FLAGS = {"fv_f32.cu": _FAST, "fv_f32_schemes.cu": _FAST, "fd_f32.cu": _FAST, "fv_batch_f32.cu": _FAST,
               "fv_batch_f32_alt.cu": _FAST, "adjoint_f32.cu": _FAST, "gravity_f32.cu": _FAST,
               "fv_f32_split_am.cu": _FAST}


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libamx.so")


def _headers():
    out = []
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".cuh", ".h")):
                out.append(os.path.join(d, f))
    return out


def _mtime(p):
    try:
        return os.path.getmtime(p)
    except OSError:
        return -1.0


def sources():
    srcs = [f for f in SOURCES if os.path.exists(os.path.join(CSRC, f))]
    extra = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu") and f not in srcs)
    return srcs + extra


def build(verbose: bool = False, jobs: int = 0) -> str:
    """Compile (incrementally) and link libamx.so; returns its path."""
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    hdr_time = max([_mtime(h) for h in _headers()] + [_mtime(__file__)])
    objs, todo = [], []
    for src in sources():
        sp = os.path.join(CSRC, src)
        op = os.path.join(BUILD, src[:-3] + ".o")
        objs.append(op)
        if _mtime(op) < max(_mtime(sp), hdr_time):
            todo.append((sp, op))

    def compile_one(job):
        sp, op = job
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *EXTRA_FLAGS.get(os.path.basename(sp), []), "-I", INCLUDE, "-c", sp,
               "-o", op]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (sp, r.stdout, r.stderr))
        if verbose:
            print("built", os.path.basename(op))
        return op

    if todo:
        n = jobs or min(len(todo), os.cpu_count() or 4)
        with ThreadPoolExecutor(max_workers=n) as ex:
            list(ex.map(compile_one, todo))
    if todo or _mtime(LIB) < max(_mtime(o) for o in objs):
        tmp = LIB + ".tmp"
        cudalib = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "lib64")
        cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-L" + cudalib, "-lcufft", "-Xlinker", "-rpath=" + cudalib]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
