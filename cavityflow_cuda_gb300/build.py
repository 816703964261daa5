"""In-tree build of the solver's shared library for sm_103a.

``python -m cavityflow_cuda_gb300.build`` (or ``build()``) compiles every
``csrc/*.cu`` translation unit in parallel with nvcc and links
``cavityflow_cuda_gb300/liblbm_gb300.so`` and the ``lbm_gb300`` command
beside it (host/lbm_main.cpp).  Object files go to
``cavityflow_cuda_gb300/_build/`` (git-ignored).

The library is compiled with ``-fmad=false``: the FP64/FP32 collision must
not be contracted into fused multiply-adds, so that it performs the same IEEE
operations as the reference kernels.  The one exception is ``*_fma.cu``
(``fast_fma.cu``): the opt-in FP64 and FP32 kernels whose multiply-adds are
fused on purpose (lbm_params.fused_multiply_add), built like the reference's
own nvcc build (-fmad=true -ftz=true).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "liblbm_gb300.so")
HOST = os.path.join(PKG, "host")
CLI = os.path.join(PKG, "lbm_gb300")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-fmad=false", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblbm_gb300.so")


def sources() -> list[str]:
    """Library translation units: CUDA (.cu) and host C++ (.cpp), both through nvcc."""
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile the library if any source or header is newer than it; return its path."""
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(PKG), "include", "lbm_gb300.h"))
    srcs = sources()
    objs = [os.path.join(BUILD, os.path.basename(s).replace(".", "_") + ".o") for s in srcs]

    def compile_one(src_obj):
        src, obj = src_obj
        if not force and not _stale(obj, [src] + headers):
            return None
        # .cpp units include the kernel headers, so they are compiled as CUDA too
        lang = ["-x", "cu"] if src.endswith(".cpp") else []
        flags = NVCC_FLAGS
        if src.endswith("_fma.cu"):  # kernels that fuse multiply-adds on purpose (fast_fma.cu), as
            # the reference's -use_fast_math build does (which also flushes FP32 subnormals)
            flags = [("-fmad=true" if f == "-fmad=false" else f) for f in NVCC_FLAGS] + ["-ftz=true"]
        cmd = [nvcc, *ARCH, *flags, *lang, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=max(1, len(srcs))) as ex:
        list(ex.map(compile_one, zip(srcs, objs)))
    if force or _stale(LIB, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    build_cli(verbose, force)
    return LIB


def build_cli(verbose: bool = False, force: bool = False) -> str:
    """Link the lbm_gb300 command (host C++ over the C ABI) beside the library."""
    src = os.path.join(HOST, "lbm_main.cpp")
    header = os.path.join(os.path.dirname(PKG), "include", "lbm_gb300.h")
    if force or _stale(CLI, [src, header, LIB]):
        cxx = shutil.which("g++") or "g++"
        cmd = [cxx, "-O2", "-std=c++17", "-Wall", src, "-o", CLI + ".tmp", f"-L{PKG}", "-llbm_gb300",
               "-Wl,-rpath,$ORIGIN"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"building lbm_gb300 failed:\n{r.stdout}\n{r.stderr}")
        os.replace(CLI + ".tmp", CLI)
    return CLI


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
