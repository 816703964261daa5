"""Test infrastructure, not part of the product: the reference's own CUDA
kernels on the GPU.

``oracle/_ref/lbm_ref_kernels.cubin`` is src/gpukernels/lbm_{init,alpha,beta}.cu
of the reference compiled with its own nvcc flags into a device-only sm_103a
image (``make -C oracle refgpu``; built where the reference checkout exists,
then carried as a prebuilt file).  This module loads it through the CUDA
driver API (ctypes on libcuda) into the context PyTorch uses and launches the
kernels the way CLbmSolverGPU does: one thread per stored cell over the whole
domain with its halo, blocks of 32 x 8 x 1 threads (the alpha/beta grid
configuration of configurations/default.xml), alpha on even steps and beta on
odd ones (src/CLbmSolverGPU.cu:173-227, :339-394; src/CController.cpp:
1278-1287), densities and velocities not stored.

Used by the GPU parity tests (the contract's max |du| after 1000 steps
against the reference kernels themselves) and by the reference arm of
bench.py (the reference kernels' MLUPS on the same GPU).  Populations and
flags are in the reference layout: 19 slots of (nz+2)(ny+2)(nx+2) cells, x
fastest; flags are the reference's 4-byte Flag values.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "lbm_ref_kernels.cubin")
NAMES = os.path.join(HERE, "_ref", "lbm_ref_kernels.names")
BLOCK = (32, 8, 1)


def available() -> bool:
    return os.path.exists(CUBIN) and os.path.exists(NAMES)


class _Driver:
    _inst = None

    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")
        self.cu.cuModuleLoad.argtypes = [C.POINTER(C.c_void_p), C.c_char_p]
        self.cu.cuModuleGetFunction.argtypes = [C.POINTER(C.c_void_p), C.c_void_p, C.c_char_p]
        self.cu.cuLaunchKernel.argtypes = [C.c_void_p] + [C.c_uint] * 7 + [C.c_void_p, C.POINTER(C.c_void_p),
                                                                           C.c_void_p]
        self.cu.cuCtxGetCurrent.argtypes = [C.POINTER(C.c_void_p)]

    @classmethod
    def get(cls):
        if cls._inst is None:
            cls._inst = _Driver()
        return cls._inst

    def check(self, r, what):
        if r != 0:
            raise RuntimeError(f"{what}: CUDA driver error {r}")


class RefGpuCavity:
    """A lid-driven cavity advanced by the reference's CUDA kernels.

    ``dd`` (19, nz+2, ny+2, nx+2) and ``flags`` (nz+2, ny+2, nx+2) give the
    initial state (for instance a solver's get_all() / flags_all() right after
    creation); ``dtype`` float32 or float64 selects the kernel instantiation.
    """

    def __init__(self, dd: np.ndarray, flags: np.ndarray, inv_tau: float, lid: float):
        import torch

        if not available():
            raise FileNotFoundError(CUBIN)
        self.torch = torch
        self.dtype = np.dtype(dd.dtype)
        if self.dtype not in (np.dtype(np.float32), np.dtype(np.float64)):
            raise ValueError("float32 or float64 populations")
        nzh, nyh, nxh = flags.shape
        if dd.shape != (19, nzh, nyh, nxh):
            raise ValueError("dd must be (19,) + flags.shape")
        self.size_halo = (nxh, nyh, nzh)
        self.cells = nxh * nyh * nzh
        tdt = torch.float64 if self.dtype == np.float64 else torch.float32
        self.dd = torch.from_numpy(np.ascontiguousarray(dd)).to("cuda")
        self.flags = torch.from_numpy(np.ascontiguousarray(flags).astype(np.int32)).to("cuda")
        self.scratch = torch.zeros(4, dtype=tdt, device="cuda")  # velocity/density (not stored)
        self.T = C.c_double if self.dtype == np.float64 else C.c_float
        self.inv_tau = float(inv_tau)
        self.lid = float(lid)
        self.counter = 0
        torch.cuda.synchronize()
        drv = _Driver.get()
        ctx = C.c_void_p()
        drv.check(drv.cu.cuCtxGetCurrent(C.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context (PyTorch should have made one)")
        self.module = C.c_void_p()
        drv.cu.cuModuleUnload.argtypes = [C.c_void_p]
        drv.check(drv.cu.cuModuleLoad(C.byref(self.module), CUBIN.encode()), "cuModuleLoad")
        names = open(NAMES).read().split()
        sfx = "d" if self.dtype == np.float64 else "f"
        self.fn = {}
        for kind, stem in (("alpha", "16lbm_kernel_alphaI"), ("beta", "15lbm_kernel_betaI")):
            name = next(n for n in names if f"{stem}{sfx}E" in n)
            f = C.c_void_p()
            drv.check(drv.cu.cuModuleGetFunction(C.byref(f), self.module, name.encode()), "cuModuleGetFunction")
            self.fn[kind] = f

    def _launch(self, kind: str, stream: int) -> None:
        drv = _Driver.get()
        nx, ny, nz = self.size_halo
        T = self.T
        args = [C.c_void_p(self.dd.data_ptr()), C.c_void_p(self.flags.data_ptr()),
                C.c_void_p(self.scratch.data_ptr()), C.c_void_p(self.scratch.data_ptr()),
                T(self.inv_tau), T(0.0), T(0.0), T(0.0), T(self.lid),
                C.c_int(0), C.c_int(0), C.c_int(0), C.c_int(nx), C.c_int(ny), C.c_int(nz),
                C.c_int(nx), C.c_int(ny), C.c_int(nz)]
        if kind == "beta":
            local = BLOCK[0] * BLOCK[1] * BLOCK[2]
            pow2 = lambda v: v > 0 and (v & (v - 1)) == 0  # noqa: E731
            args += [C.c_size_t(local), C.c_bool(pow2(self.cells)), C.c_bool(pow2(local))]
        args += [C.c_bool(False), C.c_bool(False)]
        params = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        grid = [(s - 1) // b + 1 for s, b in zip(self.size_halo, BLOCK)]
        drv.check(drv.cu.cuLaunchKernel(self.fn[kind], grid[0], grid[1], grid[2], BLOCK[0], BLOCK[1], BLOCK[2], 0,
                                        C.c_void_p(stream), params, None), f"cuLaunchKernel {kind}")

    def step(self, stream: int = 0) -> None:
        """One time step: alpha on an even counter, beta on an odd one."""
        self._launch("alpha" if self.counter % 2 == 0 else "beta", stream)
        self.counter += 1

    def run(self, steps: int, stream: int = 0) -> None:
        for _ in range(steps):
            self.step(stream)

    def get_all(self) -> np.ndarray:
        self.torch.cuda.synchronize()
        return self.dd.cpu().numpy()

    def close(self) -> None:
        if self.module is not None and self.module.value:
            self.torch.cuda.synchronize()
            _Driver.get().cu.cuModuleUnload(self.module)
            self.module = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def momentum(dd: np.ndarray) -> np.ndarray:
    """(jx, jy, jz) of every cell in float64 from reference-layout populations
    (the incompressible model's velocity is j, not j / rho)."""
    c = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [1, 1, 0], [-1, -1, 0], [1, -1, 0], [-1, 1, 0],
                  [1, 0, 1], [-1, 0, -1], [1, 0, -1], [-1, 0, 1], [0, 1, 1], [0, -1, -1], [0, 1, -1], [0, -1, 1],
                  [0, 0, 1], [0, 0, -1], [0, 0, 0]], dtype=np.float64)
    f = dd.astype(np.float64)
    return np.einsum("kd,kzyx->dzyx", c, f)


_C = ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (1, 1, 0), (-1, -1, 0), (1, -1, 0), (-1, 1, 0), (1, 0, 1),
      (-1, 0, -1), (1, 0, -1), (-1, 0, 1), (0, 1, 1), (0, -1, -1), (0, 1, -1), (0, -1, 1), (0, 0, 1), (0, 0, -1),
      (0, 0, 0))


def interior_momentum_max_diff(a, b) -> float:
    """max over interior cells and components of |j_a - j_b|, j = sum_k c_k f_k
    of the raw slots at each cell, for two reference-layout population tensors
    on the device (19, nz+2, ny+2, nx+2); float64 accumulation one slot at a
    time, so no host copy of the (possibly many-GB) arrays is needed."""
    import torch

    inner = (slice(1, -1),) * 3
    worst = 0.0
    for d in range(3):
        acc = None
        for k in range(19):
            c = _C[k][d]
            if c == 0:
                continue
            t = a[k][inner].double() - b[k][inner].double()
            acc = c * t if acc is None else acc.add_(t, alpha=c)
        worst = max(worst, float(acc.abs().max()))
        del acc
    torch.cuda.synchronize()
    return worst


def interior_momentum_max(a) -> float:
    """max |j| over interior cells of a reference-layout tensor on the device."""
    inner = (slice(1, -1),) * 3
    worst = 0.0
    for d in range(3):
        acc = None
        for k in range(19):
            c = _C[k][d]
            if c == 0:
                continue
            t = a[k][inner].double()
            acc = c * t if acc is None else acc.add_(t, alpha=c)
        worst = max(worst, float(acc.abs().max()))
    return worst


def interior_mass(a) -> float:
    """FP64 sum of every slot over the interior cells of a device tensor."""
    inner = (slice(None),) + (slice(1, -1),) * 3
    return float(a[inner].double().sum())
