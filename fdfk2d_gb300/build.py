"""Build the CUDA extension in-tree: fdfk2d_gb300/_build/libfdfk_gb300.so (sm_103a only).

The library is a plain C-ABI shared object (include/fdfk_gb300.h); Python
loads it with ctypes.  Translation units compile in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libfdfk_gb300.so")
SOURCES = ("fdfk_sweep.cu", "fdfk_capi.cu", "fdfk_fk.cu", "fdfk_noalloc.cu", "fdfk_batch.cu", "fdfk_server.cu", "fdfk_io.cpp",
           "fdfk_rf.cu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                   "-I" + os.path.join(ROOT, "include"), "-I" + CSRC] + list(extra)


def build(verbose: bool = False, extra=()) -> str:
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hdrs.append(os.path.join(ROOT, "include", "fdfk_gb300.h"))
    newest_in = max(os.path.getmtime(p) for p in srcs + hdrs + [__file__])
    if os.path.exists(LIB) and os.path.getmtime(LIB) > newest_in and not extra:
        return LIB
    cc = nvcc()
    objs = [os.path.join(OUT, os.path.splitext(os.path.basename(s))[0] + ".o") for s in srcs]

    def compile_one(pair):
        src, obj = pair
        cmd = [cc, "-c", src, "-o", obj] + _flags(extra)
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        for msg in ex.map(compile_one, zip(srcs, objs)):
            if verbose and msg:
                print(msg, file=sys.stderr)
    cmd = [cc, "-shared", "-o", LIB + ".tmp"] + objs + ARCH + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, extra=sys.argv[1:]))
