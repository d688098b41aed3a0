"""In-tree build of the CUDA library (nvcc, sm_103a) and of the CPU oracle.

The library is compiled from csrc/ with one -gencode (compute_103a/sm_103a)
into temporalspecklescode_gb300/_lib/libsstmc_gb300.so; the translation units
compile in parallel.  Host code is compiled with -ffp-contract=off: the
scene tables must be bit-identical to the oracle's restatement.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
OBJDIR = os.path.join(PKG, "_build")
LIBNAME = "libsstmc_gb300.so"
SOURCES = ["scene.cpp", "api.cpp", "errors.cpp", "pathwalk.cu", "trace.cu", "viewsum.cu", "contract.cu", "static_render.cu", "gemm_tc.cu", "serve.cpp", "plugins.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the library")


def lib_path() -> str:
    return os.path.join(LIBDIR, LIBNAME)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(ROOT, "include", "sstmc.h"))
    return hs


def build_library(verbose: bool = False, force: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    hdr_mtime = max(os.path.getmtime(h) for h in _headers())
    common = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I", os.path.join(ROOT, "include")] + ARCH

    def compile_one(src: str) -> str:
        path = os.path.join(CSRC, src)
        obj = os.path.join(OBJDIR, src + ".o")
        if not force and os.path.exists(obj) and os.path.getmtime(obj) > max(os.path.getmtime(path), hdr_mtime):
            return obj
        cmd = [nvcc] + common + ["-c", path, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    out = lib_path()
    if force or not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc, "-shared", "-o", out] + objs + ARCH
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return out


def build_oracle(verbose: bool = False) -> str:
    """Compile the CPU oracle (test infrastructure) with its Makefile."""
    odir = os.path.join(ROOT, "oracle")
    r = subprocess.run(["make", "-C", odir], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(r.stdout)
    return os.path.join(odir, "_build", "libsstmc_oracle.so")
