"""ctypes access to the CPU oracles.  TEST INFRASTRUCTURE ONLY.

Two libraries, both driven through the same small interface:

* ``liblbm_oracle.so`` -- this repository's C restatement of the reference's
  A-A kernels (oracle/lbm_oracle.c).  Builds on any host.
* ``_ref/libref_cavity.so`` -- the reference's own CPU kernels
  (src/cpukernels/CLbm{Init,Alpha,Beta}CPU.cpp) compiled from the reference
  checkout by ``make -C oracle ref``.  Exists only where that checkout exists.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs may
import this module, and only as the checker.

Arrays use the reference layout: populations ``(19, nz+2, ny+2, nx+2)``,
flags ``(nz+2, ny+2, nx+2)`` int32, x fastest.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liblbm_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref_cavity.so")

OBSTACLE, FLUID, VELOCITY_INJECTION, GHOST_LAYER = 1, 2, 4, 8

_P = C.c_void_p
_I = C.c_int


def reference_checkout() -> str | None:
    """Root of a checkout of the reference (saleemayman/cavityflow_cuda): the
    directory named by the environment variable LBM_REFERENCE_DIR, else a
    directory ``reference`` beside this repository; None when neither exists
    (as on a machine that only runs the prebuilt oracle files)."""
    env = os.environ.get("LBM_REFERENCE_DIR")
    cands = [env] if env else [os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")]
    for c in cands:
        if c and os.path.isdir(os.path.join(c, "src")):
            return os.path.abspath(c)
    return None


def reference_src() -> str | None:
    """The checkout's src/ directory, or None."""
    root = reference_checkout()
    return os.path.join(root, "src") if root else None


def build(ref_src: str | None = None) -> None:
    """Build liblbm_oracle.so (always) and the reference harness when ``ref_src`` exists."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref_src and os.path.isdir(ref_src):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_SRC={ref_src}"], check=True)
        subprocess.run(["make", "-s", "-C", HERE, "refgpu", f"REF_SRC={ref_src}"], check=True)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_P)


def _i3(v):
    return (C.c_int32 * 3)(*[int(t) for t in v])


class _Lib:
    """Shared calling code for both libraries (same argument conventions)."""

    prefix = ""

    def __init__(self, path: str):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        self.path = path

    def _fn(self, name: str, dtype):
        sfx = "d" if np.dtype(dtype) == np.float64 else "f"
        return getattr(self.lib, f"{self.prefix}_{name}_{sfx}")

    @staticmethod
    def _real(dtype):
        return C.c_double if np.dtype(dtype) == np.float64 else C.c_float

    def init(self, nx, ny, nz, dtype, bc=(OBSTACLE,) * 6):
        dd = np.zeros((19, nz + 2, ny + 2, nx + 2), dtype=dtype)
        flags = np.zeros((nz + 2, ny + 2, nx + 2), dtype=np.int32)
        fn = self._fn("init", dtype)
        fn.argtypes = [_P, _P, _I, _I, _I, _P]
        fn(_ptr(dd), _ptr(flags), nx, ny, nz, (C.c_int32 * 6)(*bc))
        return dd, flags


class Oracle(_Lib):
    """The C restatement (oracle/lbm_oracle.c)."""

    prefix = "orc"

    def __init__(self, path: str = ORACLE_SO):
        super().__init__(path)

    def num_threads(self) -> int:
        return int(self.lib.orc_num_threads())

    def set_num_threads(self, n: int) -> None:
        self.lib.orc_set_num_threads(int(n))

    def set_lid(self, flags: np.ndarray) -> None:
        nz, ny, nx = (s - 2 for s in flags.shape)
        self.lib.orc_set_lid.argtypes = [_P, _I, _I, _I]
        self.lib.orc_set_lid(_ptr(flags), nx, ny, nz)

    def alpha(self, dd, flags, inv_tau, lid_u, g=(0.0, 0.0, 0.0), origin=None, size=None, wall=False):
        """wall=True: the moving top wall (lid_u along x) instead of an injection lid."""
        nz, ny, nx = (s - 2 for s in flags.shape)
        origin = (0, 0, 0) if origin is None else origin
        size = (nx + 2, ny + 2, nz + 2) if size is None else size
        R = self._real(dd.dtype)
        fn = self._fn("alpha_wall" if wall else "alpha", dd.dtype)
        fn.argtypes = [_P, _P, _I, _I, _I, R, R, R, R, R, _P, _P]
        fn(_ptr(dd), _ptr(flags), nx, ny, nz, inv_tau, g[0], g[1], g[2], lid_u, _i3(origin), _i3(size))

    def beta(self, dd, flags, inv_tau, lid_u, origin=None, size=None, wall=False):
        nz, ny, nx = (s - 2 for s in flags.shape)
        origin = (0, 0, 0) if origin is None else origin
        size = (nx + 2, ny + 2, nz + 2) if size is None else size
        R = self._real(dd.dtype)
        fn = self._fn("beta_wall" if wall else "beta", dd.dtype)
        fn.argtypes = [_P, _P, _I, _I, _I, R, R, _P, _P]
        fn(_ptr(dd), _ptr(flags), nx, ny, nz, inv_tau, lid_u, _i3(origin), _i3(size))

    def macros(self, dd, flags, last_was_alpha, lid_u):
        nz, ny, nx = (s - 2 for s in flags.shape)
        out = [np.zeros(flags.shape, dtype=dd.dtype) for _ in range(4)]
        R = self._real(dd.dtype)
        fn = self._fn("macros", dd.dtype)
        fn.argtypes = [_P, _P, _I, _I, _I, _I, R, _P, _P, _P, _P]
        fn(_ptr(dd), _ptr(flags), nx, ny, nz, int(bool(last_was_alpha)), lid_u, *[_ptr(o) for o in out])
        return out  # rho, jx, jy, jz

    def reduce(self, dd, flags, last_was_alpha):
        nz, ny, nx = (s - 2 for s in flags.shape)
        out = np.zeros(4, dtype=np.float64)
        fn = self._fn("reduce", dd.dtype)
        fn.argtypes = [_P, _P, _I, _I, _I, _I, _P]
        fn(_ptr(dd), _ptr(flags), nx, ny, nz, int(bool(last_was_alpha)), _ptr(out))
        return out  # mass, px, py, pz

    # -- shifted 16-bit storage (the solver's FP16/BF16 extension) --------------
    # kind 0: FP16, 1: BF16, 2: FP16 of (f - w) * 2^12 with stochastic
    # rounding.  Arrays are uint16 bit patterns.
    def init_s(self, nx, ny, nz, bc=(OBSTACLE,) * 6):
        dd = np.zeros((19, nz + 2, ny + 2, nx + 2), dtype=np.uint16)
        flags = np.zeros((nz + 2, ny + 2, nx + 2), dtype=np.int32)
        fn = self.lib.orc_init_s
        fn.argtypes = [_P, _P, _I, _I, _I, _P]
        fn(_ptr(dd), _ptr(flags), nx, ny, nz, (C.c_int32 * 6)(*bc))
        return dd, flags

    def step_s(self, dd, flags, counter, inv_tau, lid_u, kind, origin=None, size=None, wall=False):
        nz, ny, nx = (s - 2 for s in flags.shape)
        origin = (0, 0, 0) if origin is None else origin
        size = (nx + 2, ny + 2, nz + 2) if size is None else size
        w = "_wall" if wall else ""
        fn = getattr(self.lib, f"orc_beta{w}_s" if counter & 1 else f"orc_alpha{w}_s")
        fn.argtypes = [_P, _P, _I, _I, _I, C.c_float, C.c_float, _I, _P, _P, C.c_uint32]
        fn(_ptr(dd), _ptr(flags), nx, ny, nz, inv_tau, lid_u, int(kind), _i3(origin), _i3(size),
           int(counter) & 0xFFFFFFFF)

    def run_cavity_s(self, nx, ny, nz, kind, inv_tau, lid_u, steps, lid=True):
        """lid: True (the injection lid), "wall" (the moving top wall) or False."""
        dd, flags = self.init_s(nx, ny, nz)
        wall = lid == "wall"
        if lid and not wall:
            self.set_lid(flags)
        for i in range(steps):
            self.step_s(dd, flags, i, inv_tau, lid_u, kind, wall=wall)
        return dd, flags

    def unshift(self, dd, kind):
        """float32 populations f = s + w of a shifted 16-bit array."""
        if kind == 0:
            f = dd.view(np.float16).astype(np.float32)
        elif kind == 2:
            f = dd.view(np.float16).astype(np.float32) * np.float32(1.0 / 4096.0)
        else:
            f = (dd.astype(np.uint32) << 16).view(np.float32)
        w = np.array([np.float32(1) / np.float32(18)] * 4 + [np.float32(1) / np.float32(36)] * 12 +
                     [np.float32(1) / np.float32(18)] * 2 + [np.float32(1) / np.float32(3)], dtype=np.float32)
        return f + w[:, None, None, None]

    def macros_s(self, dd, flags, last_was_alpha, lid_u, kind):
        nz, ny, nx = (s - 2 for s in flags.shape)
        out = [np.zeros(flags.shape, dtype=np.float32) for _ in range(4)]
        fn = self.lib.orc_macros_s
        fn.argtypes = [_P, _P, _I, _I, _I, _I, C.c_float, _I, _P, _P, _P, _P]
        fn(_ptr(dd), _ptr(flags), nx, ny, nz, int(bool(last_was_alpha)), lid_u, int(kind), *[_ptr(o) for o in out])
        return out

    def reduce_s(self, dd, flags, last_was_alpha, kind):
        nz, ny, nx = (s - 2 for s in flags.shape)
        out = np.zeros(4, dtype=np.float64)
        fn = self.lib.orc_reduce_s
        fn.argtypes = [_P, _P, _I, _I, _I, _I, _I, _P]
        fn(_ptr(dd), _ptr(flags), nx, ny, nz, int(bool(last_was_alpha)), int(kind), _ptr(out))
        return out

    def to_half(self, x: np.ndarray, kind: int) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        fn = self.lib.orc_float_to_bf16 if kind else self.lib.orc_float_to_half
        fn.argtypes = [C.c_float]
        fn.restype = C.c_uint16
        return np.array([fn(float(v)) for v in x.ravel()], dtype=np.uint16).reshape(x.shape)

    # -- convenience: the reference's time loop (src/CController.cpp:1278-1287) --
    def config(self, xml_path: str, dtype) -> dict:
        """Every field of the reference's XML reader (src/CConfiguration.cpp:28-172),
        named as in include/lbm_gb300.h's lbm_configuration."""
        r = np.zeros(14, dtype=np.float64)
        n = np.zeros(27, dtype=np.int32)
        dirs = C.create_string_buffer(4 * 256)
        fn = self._fn("config", dtype)
        fn.argtypes = [C.c_char_p, _P, _P, C.c_char_p]
        fn(xml_path.encode(), _ptr(r), _ptr(n), dirs)
        raw = dirs.raw
        names = ["benchmark_dir", "logging_dir", "validation_dir", "visualization_dir"]
        out = dict(velocity=tuple(r[0:3]), acceleration=tuple(r[3:6]), viscosity=r[6], max_velocity=r[7],
                   max_acceleration=r[8], domain_length=tuple(r[9:12]), cpu_subdomain_ratio=r[12],
                   timestep=r[13], domain_size=tuple(int(v) for v in n[0:3]),
                   subdomain_num=tuple(int(v) for v in n[3:6]), loops=int(n[6]), do_benchmark=int(n[7]),
                   do_logging=int(n[8]), do_validation=int(n[9]), do_visualization=int(n[10]),
                   visualization_rate=int(n[11]), cpu_alpha_block=tuple(int(v) for v in n[12:15]),
                   cpu_beta_block=tuple(int(v) for v in n[15:18]), gpu_init_block=tuple(int(v) for v in n[18:21]),
                   gpu_alpha_block=tuple(int(v) for v in n[21:24]), gpu_beta_block=tuple(int(v) for v in n[24:27]))
        for i, name in enumerate(names):
            out[name] = raw[256 * i:256 * (i + 1)].split(b"\0", 1)[0].decode()
        return out

    def step(self, dd, flags, counter, inv_tau, lid_u, g=(0.0, 0.0, 0.0), wall=False):
        if counter & 1:
            self.beta(dd, flags, inv_tau, lid_u, wall=wall)
        else:
            self.alpha(dd, flags, inv_tau, lid_u, g, wall=wall)

    def run_cavity(self, nx, ny, nz, dtype, inv_tau, lid_u, steps, g=(0.0, 0.0, 0.0), lid=True):
        """lid: True (the reference's injection lid), "wall" (the moving top
        wall) or False (closed box at rest)."""
        dd, flags = self.init(nx, ny, nz, dtype)
        wall = lid == "wall"
        if lid and not wall:
            self.set_lid(flags)
        for i in range(steps):
            self.step(dd, flags, i, inv_tau, lid_u, g, wall=wall)
        return dd, flags


class Reference(_Lib):
    """The reference's own CPU kernels (oracle/_ref/libref_cavity.so)."""

    prefix = "ref"

    def __init__(self, path: str = REF_SO):
        super().__init__(path)

    def alpha(self, dd, flags, inv_tau, lid_u, g=(0.0, 0.0, 0.0), origin=None, size=None, block=(32, 32, 32)):
        nz, ny, nx = (s - 2 for s in flags.shape)
        origin = (0, 0, 0) if origin is None else origin
        size = (nx + 2, ny + 2, nz + 2) if size is None else size
        R = self._real(dd.dtype)
        fn = self._fn("alpha", dd.dtype)
        fn.argtypes = [_P, _P, _I, _I, _I, R, R, R, R, R, _P, _P, _P]
        fn(_ptr(dd), _ptr(flags), nx, ny, nz, inv_tau, g[0], g[1], g[2], lid_u,
           _i3(origin), _i3(size), _i3(block))

    def beta(self, dd, flags, inv_tau, lid_u, origin=None, size=None, block=(32, 32, 32)):
        nz, ny, nx = (s - 2 for s in flags.shape)
        origin = (0, 0, 0) if origin is None else origin
        size = (nx + 2, ny + 2, nz + 2) if size is None else size
        R = self._real(dd.dtype)
        fn = self._fn("beta", dd.dtype)
        fn.argtypes = [_P, _P, _I, _I, _I, R, R, _P, _P, _P]
        fn(_ptr(dd), _ptr(flags), nx, ny, nz, inv_tau, lid_u, _i3(origin), _i3(size), _i3(block))

    def params(self, xml_path: str, dtype) -> np.ndarray:
        """(timestep, tau, tauInv, U*x, U*y, U*z, g*x, g*y, g*z, nu*) as the
        reference's CLbmSolver constructor derives them (src/CLbmSolver.cpp:28-327)."""
        out = np.zeros(10, dtype=np.float64)
        fn = self._fn("params", dtype)
        fn.argtypes = [C.c_char_p, _P]
        fn(xml_path.encode(), _ptr(out))
        return out

    def config(self, xml_path: str, dtype) -> dict:
        """Every field of the reference's XML reader (src/CConfiguration.cpp:28-172),
        named as in include/lbm_gb300.h's lbm_configuration."""
        r = np.zeros(14, dtype=np.float64)
        n = np.zeros(27, dtype=np.int32)
        dirs = C.create_string_buffer(4 * 256)
        fn = self._fn("config", dtype)
        fn.argtypes = [C.c_char_p, _P, _P, C.c_char_p]
        fn(xml_path.encode(), _ptr(r), _ptr(n), dirs)
        raw = dirs.raw
        names = ["benchmark_dir", "logging_dir", "validation_dir", "visualization_dir"]
        out = dict(velocity=tuple(r[0:3]), acceleration=tuple(r[3:6]), viscosity=r[6], max_velocity=r[7],
                   max_acceleration=r[8], domain_length=tuple(r[9:12]), cpu_subdomain_ratio=r[12],
                   timestep=r[13], domain_size=tuple(int(v) for v in n[0:3]),
                   subdomain_num=tuple(int(v) for v in n[3:6]), loops=int(n[6]), do_benchmark=int(n[7]),
                   do_logging=int(n[8]), do_validation=int(n[9]), do_visualization=int(n[10]),
                   visualization_rate=int(n[11]), cpu_alpha_block=tuple(int(v) for v in n[12:15]),
                   cpu_beta_block=tuple(int(v) for v in n[15:18]), gpu_init_block=tuple(int(v) for v in n[18:21]),
                   gpu_alpha_block=tuple(int(v) for v in n[21:24]), gpu_beta_block=tuple(int(v) for v in n[24:27]))
        for i, name in enumerate(names):
            out[name] = raw[256 * i:256 * (i + 1)].split(b"\0", 1)[0].decode()
        return out

    def step(self, dd, flags, counter, inv_tau, lid_u, g=(0.0, 0.0, 0.0)):
        if counter & 1:
            self.beta(dd, flags, inv_tau, lid_u)
        else:
            self.alpha(dd, flags, inv_tau, lid_u, g)

    def run_cavity(self, nx, ny, nz, dtype, inv_tau, lid_u, steps, g=(0.0, 0.0, 0.0), lid=True):
        dd, flags = self.init(nx, ny, nz, dtype)
        if lid:
            flags[1:-1, ny, 1:-1] = VELOCITY_INJECTION  # src/CController.cpp:1313-1345
        for i in range(steps):
            self.step(dd, flags, i, inv_tau, lid_u, g)
        return dd, flags


def tau_of(nu, dtype):
    """tau = 0.5*(6 nu + 1) and 1/tau in the working precision, for dx = dt = 1
    (src/CLbmSolver.cpp:227, :281)."""
    T = np.dtype(dtype).type
    tau = T(0.5) * (T(6) * T(nu) + T(1))
    return tau, T(1) / tau
