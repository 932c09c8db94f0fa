"""Builds libtomoj_gb300.so (the C-ABI engine) in-tree with nvcc for sm_103a.

Device code is compiled with -fmad=false (every fused multiply-add in the
kernels is an explicit fmaf) and host code with -ffp-contract=off, so that the
double-precision geometry rounds like the Java reference.  Translation units are
compiled in parallel and linked into tomoj_gb300/_lib/libtomoj_gb300.so.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libtomoj_gb300.so")
SOURCES = ["tomo_abi.cu", "kernels_fp.cu", "fp_kernel_q1.cu", "fp_kernel_q2.cu", "fp_kernel_q2w.cu", "fp_kernel_q4.cu", "fp_kernel_q8.cu", "fp_persist_t256.cu", "fp_persist_t512.cu", "kernels_bp.cu", "kernels_misc.cu", "kernels_vol.cu", "kernels_generic.cu", "geometry.cpp", "noalloc.cu", "batch.cu",
           "kernels_wavelet.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(extra_ptxas: bool) -> list[str]:
    f = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
         "--expt-relaxed-constexpr"] + ARCH
    if extra_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "tomoj_gb300.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False, out: str | None = None, defines=()) -> str:
    """Compile (if stale) and return the path of the shared library.
    `out` and `defines` (e.g. ["TOMO_BP_MIN_BLOCKS=2"]) build a tuning variant elsewhere."""
    lib = out or LIB
    if not force and out is None and not _stale():
        return LIB
    os.makedirs(os.path.dirname(lib), exist_ok=True)
    obj_dir = os.path.join(os.path.dirname(lib), "obj_" + os.path.basename(lib))
    os.makedirs(obj_dir, exist_ok=True)
    cc = nvcc()

    def compile_one(src: str) -> str:
        obj = os.path.join(obj_dir, src + ".o")
        cmd = [cc, "-c", os.path.join(CSRC, src), "-o", obj] + _flags(verbose) + [f"-D{d}" for d in defines]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = lib + ".tmp"
    # --no-undefined: a declared but undefined symbol fails here, not at load time
    cmd = [cc, "-shared", "-o", tmp] + objs + ARCH + ["--cudart", "static", "-Xlinker", "--no-undefined"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
