"""Build ``libevx.so`` (the sm_103a CUDA library behind the C ABI in ``include/evx.h``).

Each ``csrc/*.cu`` is compiled by nvcc in parallel for ``sm_103a`` only, then
linked into one shared library in this package folder, against the shared CUDA
runtime and cuFFT (the same sonames torch loads, so one runtime serves both).

Usage: ``python -m evoxels_gb300.build`` or ``evoxels_gb300.build.build()``.
"""

from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libevx.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-Xptxas", "-v", "-I", INCLUDE]
# Forward kernels mirror the reference's float32 rounding op by op: no FMA
# contraction.  The adjoint has no bitwise-parity requirement and contracts.
FMAD_ON = {"evx_adjoint.cu", "evx_ch_fast_adj.cu", "evx_fftx.cu", "evx_fftyz.cu", "evx_fftz.cu"}


def _fmad(src):
    return ["--fmad=true"] if os.path.basename(src) in FMAD_ON else ["--fmad=false"]


def _extra():
    """Developer hook: extra nvcc flags (e.g. -D tuning macros) from EVX_EXTRA_NVCC_FLAGS."""
    return os.environ.get("EVX_EXTRA_NVCC_FLAGS", "").split()


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; the CUDA 13 toolkit is required to build libevx.so")


def _cuda_lib_dir(nvcc):
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "lib64")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _fingerprint(srcs):
    h = hashlib.sha256()
    h.update(" ".join(ARCH + NVCC_FLAGS + sorted(FMAD_ON) + _extra()).encode())
    deps = srcs + sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h")))
    deps.append(os.path.join(INCLUDE, "evx.h"))
    for p in deps:
        with open(p, "rb") as f:
            h.update(p.encode())
            h.update(f.read())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    """Compile and link ``libevx.so``; returns its path.  Skips work when up to date."""
    srcs = sources()
    fp = _fingerprint(srcs)
    stamp = os.path.join(BUILD, "libevx.fingerprint")
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == fp:
                return LIB
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    objs = []

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc] + ARCH + NVCC_FLAGS + _fmad(src) + _extra() + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, len(srcs))) as ex:
        for obj, log in ex.map(compile_one, srcs):
            objs.append(obj)
            if verbose:
                sys.stderr.write(log)
            with open(obj + ".ptxas.txt", "w") as f:
                f.write(log)
    libdir = _cuda_lib_dir(nvcc)
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs + [
        "-L" + libdir, "-lcufft", "-Xlinker", "-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(fp)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
