"""Python binding of the solver's C ABI (include/lbm_gb300.h) via ctypes.

``CLbmSolverGB300`` mirrors the method names and argument meaning of the
reference's ``CLbmSolverGPU<T>`` (src/CLbmSolverGPU.cuh:25-95): alpha/beta
steps over the whole domain or a cuboid, and get/set of populations, flags,
velocities and densities over cuboids in halo coordinates.  Where the
reference asserts or exits, these methods raise ``LbmError``.

The library is the in-tree ``liblbm_gb300.so``; importing this module does
not load it, constructing a solver does, and fails loudly if it is missing.
"""
from __future__ import annotations

import ctypes as C
import os
import re
from typing import Optional, Sequence

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "liblbm_gb300.so")
HEADER = os.path.join(os.path.dirname(PKG), "include", "lbm_gb300.h")

OBSTACLE, FLUID, VELOCITY_INJECTION, GHOST_LAYER = 1, 2, 4, 8
DIRECTION_ALL, LEFT, RIGHT, BOTTOM, TOP, BACK, FRONT = -1, 0, 1, 2, 3, 4, 5
STORAGE = {"f64": 0, "f32": 1, "f16s": 2, "bf16s": 3, "f16sr": 4}
# lbm_params.lid_mode: the reference's injection lid, or the moving top wall
LID_MODES = {"injection": 0, "wall": 1}

_lib: Optional[C.CDLL] = None


class LbmError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


class _Physical(C.Structure):
    _fields_ = [("velocity", C.c_double * 3), ("acceleration", C.c_double * 3), ("viscosity", C.c_double),
                ("max_velocity", C.c_double), ("max_acceleration", C.c_double), ("domain_size", C.c_int32 * 3),
                ("domain_length", C.c_double * 3), ("timestep", C.c_double)]


class _Lattice(C.Structure):
    _fields_ = [("timestep", C.c_double), ("tau", C.c_double), ("inv_tau", C.c_double),
                ("velocity", C.c_double * 3), ("acceleration", C.c_double * 3), ("viscosity", C.c_double)]


class _Configuration(C.Structure):
    _fields_ = [("velocity", C.c_double * 3), ("acceleration", C.c_double * 3), ("viscosity", C.c_double),
                ("max_velocity", C.c_double), ("max_acceleration", C.c_double), ("domain_size", C.c_int32 * 3),
                ("subdomain_num", C.c_int32 * 3), ("domain_length", C.c_double * 3),
                ("cpu_subdomain_ratio", C.c_double), ("timestep", C.c_double), ("loops", C.c_int32),
                ("do_benchmark", C.c_int32), ("do_logging", C.c_int32), ("do_validation", C.c_int32),
                ("do_visualization", C.c_int32), ("visualization_rate", C.c_int32),
                ("cpu_alpha_block", C.c_int32 * 3), ("cpu_beta_block", C.c_int32 * 3),
                ("gpu_init_block", C.c_int32 * 3), ("gpu_alpha_block", C.c_int32 * 3),
                ("gpu_beta_block", C.c_int32 * 3), ("reserved", C.c_int32), ("benchmark_dir", C.c_char * 256),
                ("logging_dir", C.c_char * 256), ("validation_dir", C.c_char * 256),
                ("visualization_dir", C.c_char * 256)]


class _Params(C.Structure):
    _fields_ = [("size", C.c_int32 * 3), ("storage", C.c_int32), ("boundary", C.c_int32 * 6),
                ("inv_tau", C.c_double), ("lid_velocity", C.c_double), ("gravity", C.c_double * 3),
                ("device", C.c_int32), ("fast_variant", C.c_int32), ("fused_multiply_add", C.c_int32),
                ("lid_mode", C.c_int32)]


class _Info(C.Structure):
    _fields_ = [("size", C.c_int32 * 3), ("storage", C.c_int32), ("value_size", C.c_int32),
                ("vector_cells", C.c_int32), ("step_counter", C.c_int64), ("last_step_was_alpha", C.c_int32),
                ("fast_path", C.c_int32), ("fast_variant", C.c_int32), ("cells_per_thread", C.c_int32),
                ("block_threads", C.c_int32), ("beta_cells_per_thread", C.c_int32),
                ("beta_block_threads", C.c_int32), ("beta_block_exchange", C.c_int32),
                ("fused_multiply_add", C.c_int32), ("row_pitch", C.c_int64), ("slot_stride", C.c_int64),
                ("device_bytes", C.c_int64), ("x1_column", C.c_int64), ("lid_mode", C.c_int32),
                ("moving_wall", C.c_int32)]


def declared_functions() -> list[str]:
    """Names of the functions include/lbm_gb300.h declares."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lbm_[a-z0-9_]+)\s*\(", text)))


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Load liblbm_gb300.so; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -m cavityflow_cuda_gb300.build`")
    lib = C.CDLL(path)
    P, I, I64, V = C.c_void_p, C.c_int, C.c_int64, C.c_void_p
    sig = {
        "lbm_derive_lattice": ([P, C.c_int32, P], I),
        "lbm_create": ([P, P], I),
        "lbm_destroy": ([V], I),
        "lbm_get_info": ([V, P], I),
        "lbm_get_domain": ([V, P], I),
        "lbm_value_size": ([V], I),
        "lbm_set_driven_cavity": ([V], I),
        "lbm_step_alpha": ([V, P], I),
        "lbm_step_alpha_cuboid": ([V, P, P, P], I),
        "lbm_step_beta": ([V, P], I),
        "lbm_step_beta_cuboid": ([V, P, P, P], I),
        "lbm_run": ([V, I64, P], I),
        "lbm_synchronize": ([V], I),
        "lbm_selftest_bounded_wait": ([V, C.c_int32], I),
        "lbm_fast_variant_count": ([], I),
        "lbm_register_variant_count": ([], I),
        "lbm_set_fast_variant": ([V, C.c_int32], I),
        "lbm_autotune": ([V, C.c_int32, P, P], I),
        "lbm_get_density_distributions": ([V, P, P, P, P], I),
        "lbm_set_density_distributions": ([V, P, P, C.c_int32, P, P], I),
        "lbm_get_flags": ([V, P, P, P], I),
        "lbm_set_flags": ([V, P, P, P], I),
        "lbm_get_velocities": ([V, P, P, P], I),
        "lbm_set_velocities": ([V, P, P, P], I),
        "lbm_get_densities": ([V, P, P, P], I),
        "lbm_set_densities": ([V, P, P, P], I),
        "lbm_reduce": ([V, P, P], I),
        "lbm_read_configuration": ([C.c_char_p, P], I),
        "lbm_configuration_physical": ([P, P], I),
        "lbm_save_checkpoint": ([V, C.c_char_p], I),
        "lbm_load_checkpoint": ([V, C.c_char_p], I),
        "lbm_create_from_checkpoint": ([C.c_char_p, C.c_int32, P], I),
        "lbm_write_vtk": ([V, C.c_char_p, P, C.c_int32], I),
        "lbm_batch_create": ([P, C.c_int32, C.c_int32, C.c_int32, P], I),
        "lbm_batch_destroy": ([V], I),
        "lbm_batch_get_info": ([V, P], I),
        "lbm_batch_domain": ([V, C.c_int32, P], I),
        "lbm_batch_run": ([V, I64, P], I),
        "lbm_batch_set_fast_variant": ([V, C.c_int32], I),
        "lbm_batch_autotune": ([V, C.c_int32, P, P], I),
        "lbm_server_create": ([P, P], I),
        "lbm_server_destroy": ([V], I),
        "lbm_server_submit": ([V, P, P], I),
        "lbm_server_round": ([V, P], I),
        "lbm_server_poll": ([V, P, C.c_int32, P], I),
        "lbm_server_take_result": ([V, C.c_int64, P, P], I),
        "lbm_server_get_stats": ([V, P], I),
        "lbm_status_string": ([I], C.c_char_p),
        "lbm_last_error": ([], C.c_char_p),
        "lbm_kernel_launches": ([], I64),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def _check(status: int) -> None:
    if status != 0:
        lib = load_library()
        raise LbmError(status, f"{lib.lbm_status_string(status).decode()}: {lib.lbm_last_error().decode()}")


def _stream_ptr(stream) -> Optional[int]:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream or None
    return int(getattr(stream, "cuda_stream"))


def _i3(v: Optional[Sequence[int]]):
    return None if v is None else (C.c_int32 * 3)(*[int(t) for t in v])


def kernel_launches() -> int:
    return int(load_library().lbm_kernel_launches())


def derive_lattice(velocity=(0.05, 0.0, 0.0), acceleration=(0.0, 0.0, 0.0), viscosity=0.032, max_velocity=0.1,
                   max_acceleration=0.1, domain_size=(64, 64, 64), domain_length=None, timestep=1.0,
                   storage: str = "f32") -> dict:
    """Lattice parameters from physical ones, as src/CLbmSolver.cpp:28-327 derives them."""
    lib = load_library()
    ph = _Physical()
    ph.velocity[:] = list(velocity)
    ph.acceleration[:] = list(acceleration)
    ph.viscosity = viscosity
    ph.max_velocity = max_velocity
    ph.max_acceleration = max_acceleration
    ph.domain_size[:] = list(domain_size)
    ph.domain_length[:] = list(domain_length if domain_length is not None else domain_size)
    ph.timestep = timestep
    out = _Lattice()
    _check(lib.lbm_derive_lattice(C.byref(ph), STORAGE[storage], C.byref(out)))
    return dict(timestep=out.timestep, tau=out.tau, inv_tau=out.inv_tau, velocity=tuple(out.velocity),
                acceleration=tuple(out.acceleration), viscosity=out.viscosity)


def read_configuration(path: str) -> dict:
    """An XML configuration of the reference's schema, as
    CConfiguration<T>::CConfiguration (src/CConfiguration.cpp:28-172) reads it."""
    lib = load_library()
    c = _Configuration()
    _check(lib.lbm_read_configuration(os.fsencode(path), C.byref(c)))
    out = {}
    for f, t in _Configuration._fields_:
        v = getattr(c, f)
        if f.endswith("_dir"):
            v = v.decode()
        elif hasattr(t, "_length_"):
            v = tuple(v)
        out[f] = v
    out.pop("reserved")
    return out


def configuration_lattice(path: str, storage: str = "f32") -> dict:
    """Lattice parameters of an XML configuration (reader + derivation)."""
    lib = load_library()
    c = _Configuration()
    _check(lib.lbm_read_configuration(os.fsencode(path), C.byref(c)))
    ph = _Physical()
    _check(lib.lbm_configuration_physical(C.byref(c), C.byref(ph)))
    out = _Lattice()
    _check(lib.lbm_derive_lattice(C.byref(ph), STORAGE[storage], C.byref(out)))
    return dict(timestep=out.timestep, tau=out.tau, inv_tau=out.inv_tau, velocity=tuple(out.velocity),
                acceleration=tuple(out.acceleration), viscosity=out.viscosity)


class _DomainSpec(C.Structure):
    _fields_ = [("size", C.c_int32 * 3), ("reserved", C.c_int32), ("inv_tau", C.c_double),
                ("lid_velocity", C.c_double)]


class _BatchInfo(C.Structure):
    _fields_ = [("count", C.c_int32), ("storage", C.c_int32), ("fast_variant", C.c_int32),
                ("cells_per_thread", C.c_int32), ("block_threads", C.c_int32),
                ("beta_cells_per_thread", C.c_int32), ("beta_block_threads", C.c_int32), ("reserved", C.c_int32),
                ("interior_cells", C.c_int64), ("step_counter", C.c_int64), ("device_bytes", C.c_int64)]


class CLbmSolverGB300:
    """One D3Q19 domain on one GPU, driven through the C ABI."""

    def __init__(self, size: Sequence[int], inv_tau: float, lid_velocity: float, storage: str = "f32",
                 boundary: Sequence[int] = (OBSTACLE,) * 6, gravity: Sequence[float] = (0.0, 0.0, 0.0),
                 device: int = 0, driven_cavity: bool = True, fast_variant: int = -1,
                 fused_multiply_add: bool = False, lid: str = "injection"):
        self._lib = load_library()
        p = _Params()
        p.size[:] = [int(s) for s in size]
        p.storage = STORAGE[storage]
        p.boundary[:] = [int(b) for b in boundary]
        p.inv_tau = float(inv_tau)
        p.lid_velocity = float(lid_velocity)
        p.gravity[:] = [float(g) for g in gravity]
        p.device = int(device)
        p.fast_variant = 0 if fast_variant < 0 else int(fast_variant) + 1
        p.fused_multiply_add = 1 if fused_multiply_add else 0
        p.lid_mode = LID_MODES[lid]
        h = C.c_void_p()
        _check(self._lib.lbm_create(C.byref(p), C.byref(h)))
        self._h = h
        self.storage = storage
        self.size = tuple(int(s) for s in size)
        self.dtype = np.float64 if storage == "f64" else np.float32
        if driven_cavity:
            self.setDrivenCavity()

    @classmethod
    def _view(cls, lib, handle, size, storage, owner):
        """A non-owning wrapper of a batch domain's solver handle."""
        self = cls.__new__(cls)
        self._lib = lib
        self._h = C.c_void_p(handle)
        self._owner = owner
        self.storage = storage
        self.size = tuple(int(s) for s in size)
        self.dtype = np.float64 if storage == "f64" else np.float32
        return self

    @classmethod
    def from_checkpoint(cls, path: str, device: int = 0) -> "CLbmSolverGB300":
        """A solver restored from a checkpoint written by save_checkpoint."""
        self = cls.__new__(cls)
        self._lib = load_library()
        h = C.c_void_p()
        _check(self._lib.lbm_create_from_checkpoint(os.fsencode(path), int(device), C.byref(h)))
        self._h = h
        i = self.info()
        self.storage = {v: k for k, v in STORAGE.items()}[i["storage"]]
        self.size = tuple(i["size"])
        self.dtype = np.float64 if self.storage == "f64" else np.float32
        return self

    # -- lifecycle --------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_owner", None) is not None:
            self._h = None
            return
        if getattr(self, "_h", None):
            self._lib.lbm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> int:
        return self._h.value

    def info(self) -> dict:
        i = _Info()
        _check(self._lib.lbm_get_info(self._h, C.byref(i)))
        return {f: (tuple(getattr(i, f)) if f == "size" else getattr(i, f)) for f, _ in _Info._fields_}

    def getDomain(self) -> tuple:
        return self.size

    def setDrivenCavity(self) -> None:
        _check(self._lib.lbm_set_driven_cavity(self._h))

    # -- steps ------------------------------------------------------------
    def simulationStepAlpha(self, origin=None, size=None, stream=None) -> None:
        if origin is None and size is None:
            _check(self._lib.lbm_step_alpha(self._h, _stream_ptr(stream)))
        else:
            _check(self._lib.lbm_step_alpha_cuboid(self._h, _i3(origin), _i3(size), _stream_ptr(stream)))

    def simulationStepBeta(self, origin=None, size=None, stream=None) -> None:
        if origin is None and size is None:
            _check(self._lib.lbm_step_beta(self._h, _stream_ptr(stream)))
        else:
            _check(self._lib.lbm_step_beta_cuboid(self._h, _i3(origin), _i3(size), _stream_ptr(stream)))

    def run(self, steps: int, stream=None) -> None:
        _check(self._lib.lbm_run(self._h, int(steps), _stream_ptr(stream)))

    def synchronize(self) -> None:
        _check(self._lib.lbm_synchronize(self._h))

    def set_fast_variant(self, variant: int) -> None:
        _check(self._lib.lbm_set_fast_variant(self._h, int(variant)))

    def autotune(self, pairs: int = 10):
        """Time every launch variant on this domain and keep the fastest;
        the populations are restored.  Returns (best, ms per pair per variant)."""
        n = int(self._lib.lbm_fast_variant_count())
        ms = (C.c_float * n)()
        best = C.c_int32()
        _check(self._lib.lbm_autotune(self._h, int(pairs), C.byref(best), ms))
        return best.value, list(ms)

    # -- checkpoint and output --------------------------------------------
    def save_checkpoint(self, path: str) -> None:
        _check(self._lib.lbm_save_checkpoint(self._h, os.fsencode(path)))

    def load_checkpoint(self, path: str) -> None:
        _check(self._lib.lbm_load_checkpoint(self._h, os.fsencode(path)))

    def write_vtk(self, path: str, length=None, binary: bool = False) -> None:
        L = None if length is None else (C.c_double * 3)(*[float(v) for v in length])
        _check(self._lib.lbm_write_vtk(self._h, os.fsencode(path), L, int(bool(binary))))

    # -- data -------------------------------------------------------------
    def _shape(self, size, comps):
        if size is None:
            size = self.size
        return (comps, size[2], size[1], size[0]) if comps > 1 else (size[2], size[1], size[0])

    def getDensityDistributions(self, origin=None, size=None, out: Optional[np.ndarray] = None, stream=None,
                                sync: bool = True) -> np.ndarray:
        if out is None:
            out = np.empty(self._shape(size, 19), dtype=self.dtype)
        assert out.flags.c_contiguous and out.dtype == self.dtype and out.size == int(np.prod(self._shape(size, 19)))
        _check(self._lib.lbm_get_density_distributions(self._h, _i3(origin), _i3(size), out.ctypes.data,
                                                       _stream_ptr(stream)))
        if sync:
            self.synchronize()
        return out

    def setDensityDistributions(self, src: np.ndarray, origin=None, size=None, direction: int = DIRECTION_ALL,
                                stream=None, sync: bool = True) -> None:
        src = np.ascontiguousarray(src, dtype=self.dtype)
        _check(self._lib.lbm_set_density_distributions(self._h, _i3(origin), _i3(size), int(direction),
                                                       src.ctypes.data, _stream_ptr(stream)))
        if sync:
            self.synchronize()

    def getFlags(self, origin=None, size=None) -> np.ndarray:
        out = np.empty(self._shape(size, 1), dtype=np.int32)
        _check(self._lib.lbm_get_flags(self._h, _i3(origin), _i3(size), out.ctypes.data))
        return out

    def setFlags(self, src: np.ndarray, origin=None, size=None) -> None:
        src = np.ascontiguousarray(src, dtype=np.int32)
        _check(self._lib.lbm_set_flags(self._h, _i3(origin), _i3(size), src.ctypes.data))

    def getVelocities(self, origin=None, size=None, out: Optional[np.ndarray] = None) -> np.ndarray:
        if out is None:
            out = np.empty(self._shape(size, 3), dtype=self.dtype)
        assert out.flags.c_contiguous and out.dtype == self.dtype and out.size == int(np.prod(self._shape(size, 3)))
        _check(self._lib.lbm_get_velocities(self._h, _i3(origin), _i3(size), out.ctypes.data))
        return out

    def setVelocities(self, src: np.ndarray, origin=None, size=None) -> None:
        src = np.ascontiguousarray(src, dtype=self.dtype)
        _check(self._lib.lbm_set_velocities(self._h, _i3(origin), _i3(size), src.ctypes.data))

    def getDensities(self, origin=None, size=None, out: Optional[np.ndarray] = None) -> np.ndarray:
        if out is None:
            out = np.empty(self._shape(size, 1), dtype=self.dtype)
        assert out.flags.c_contiguous and out.dtype == self.dtype and out.size == int(np.prod(self._shape(size, 1)))
        _check(self._lib.lbm_get_densities(self._h, _i3(origin), _i3(size), out.ctypes.data))
        return out

    def setDensities(self, src: np.ndarray, origin=None, size=None) -> None:
        src = np.ascontiguousarray(src, dtype=self.dtype)
        _check(self._lib.lbm_set_densities(self._h, _i3(origin), _i3(size), src.ctypes.data))

    def reduce(self, stream=None) -> np.ndarray:
        """FP64 (mass, momentum x, y, z) of the last collided time level."""
        out = np.zeros(4, dtype=np.float64)
        _check(self._lib.lbm_reduce(self._h, out.ctypes.data, _stream_ptr(stream)))
        return out

    # -- whole-array helpers in the reference layout (halo included) -------
    def get_all(self) -> np.ndarray:
        n = self.size
        return self.getDensityDistributions((0, 0, 0), (n[0] + 2, n[1] + 2, n[2] + 2))

    def set_all(self, dd: np.ndarray) -> None:
        n = self.size
        self.setDensityDistributions(dd, (0, 0, 0), (n[0] + 2, n[1] + 2, n[2] + 2))

    def flags_all(self) -> np.ndarray:
        n = self.size
        return self.getFlags((0, 0, 0), (n[0] + 2, n[1] + 2, n[2] + 2))


class LbmBatch:
    """Many box cavities of uneven size and Reynolds number advanced together
    by one persistent kernel per step (lbm_batch_* of include/lbm_gb300.h)."""

    def __init__(self, domains, storage: str = "f32", device: int = 0):
        """domains: iterable of (size(3), inv_tau, lid_velocity)."""
        self._lib = load_library()
        doms = list(domains)
        arr = (_DomainSpec * len(doms))()
        for i, (size, inv_tau, lid) in enumerate(doms):
            arr[i].size[:] = [int(v) for v in size]
            arr[i].inv_tau = float(inv_tau)
            arr[i].lid_velocity = float(lid)
        h = C.c_void_p()
        _check(self._lib.lbm_batch_create(arr, len(doms), STORAGE[storage], int(device), C.byref(h)))
        self._h = h
        self.storage = storage
        self.sizes = [tuple(int(v) for v in d[0]) for d in doms]

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.lbm_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __len__(self) -> int:
        return len(self.sizes)

    def info(self) -> dict:
        i = _BatchInfo()
        _check(self._lib.lbm_batch_get_info(self._h, C.byref(i)))
        return {f: getattr(i, f) for f, _ in _BatchInfo._fields_}

    def domain(self, index: int) -> "CLbmSolverGB300":
        v = C.c_void_p()
        _check(self._lib.lbm_batch_domain(self._h, int(index), C.byref(v)))
        return CLbmSolverGB300._view(self._lib, v.value, self.sizes[index], self.storage, self)

    def run(self, steps: int, stream=None) -> None:
        _check(self._lib.lbm_batch_run(self._h, int(steps), _stream_ptr(stream)))

    def set_fast_variant(self, variant: int) -> None:
        _check(self._lib.lbm_batch_set_fast_variant(self._h, int(variant)))

    def autotune(self, pairs: int = 5):
        ms = (C.c_float * self._lib.lbm_register_variant_count())()
        best = C.c_int32()
        _check(self._lib.lbm_batch_autotune(self._h, int(pairs), C.byref(best), ms))
        return best.value, list(ms)


class _ServerConfig(C.Structure):
    _fields_ = [("storage", C.c_int32), ("device", C.c_int32), ("max_round_steps", C.c_int32),
                ("target_round_ms", C.c_int32), ("fast_variant", C.c_int32), ("reserved", C.c_int32),
                ("budget_bytes", C.c_int64)]


class _Request(C.Structure):
    _fields_ = [("size", C.c_int32 * 3), ("reserved", C.c_int32), ("inv_tau", C.c_double),
                ("lid_velocity", C.c_double), ("steps", C.c_int64)]


class _Completion(C.Structure):
    _fields_ = [("id", C.c_int64), ("steps", C.c_int64), ("cells", C.c_int64), ("status", C.c_int32),
                ("reserved", C.c_int32), ("submit_time", C.c_double), ("admit_time", C.c_double),
                ("finish_time", C.c_double)]


class _ServerStats(C.Structure):
    _fields_ = [("queued", C.c_int64), ("active", C.c_int64), ("completed", C.c_int64),
                ("bytes_in_use", C.c_int64), ("peak_bytes", C.c_int64), ("budget_bytes", C.c_int64),
                ("lattice_updates", C.c_int64), ("rounds", C.c_int64), ("busy_seconds", C.c_double),
                ("elapsed_seconds", C.c_double)]


class LbmServer:
    """Cavity-solve requests with continuous batching (lbm_server_* of
    include/lbm_gb300.h)."""

    def __init__(self, budget_bytes: int, storage: str = "f32", device: int = 0, max_round_steps: int = 256,
                 target_round_ms: int = 50, fast_variant: int = -1):
        self._lib = load_library()
        cfg = _ServerConfig()
        cfg.storage = STORAGE[storage]
        cfg.device = int(device)
        cfg.max_round_steps = int(max_round_steps)
        cfg.target_round_ms = int(target_round_ms)
        cfg.fast_variant = 0 if fast_variant < 0 else int(fast_variant) + 1
        cfg.budget_bytes = int(budget_bytes)
        h = C.c_void_p()
        _check(self._lib.lbm_server_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self.storage = storage
        self.dtype = np.float64 if storage == "f64" else np.float32
        self._sizes = {}

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.lbm_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, size, inv_tau: float, lid_velocity: float, steps: int) -> int:
        r = _Request()
        r.size[:] = [int(v) for v in size]
        r.inv_tau = float(inv_tau)
        r.lid_velocity = float(lid_velocity)
        r.steps = int(steps)
        rid = C.c_int64()
        _check(self._lib.lbm_server_submit(self._h, C.byref(r), C.byref(rid)))
        self._sizes[rid.value] = tuple(int(v) for v in size)
        return rid.value

    def round(self) -> bool:
        ran = C.c_int32()
        _check(self._lib.lbm_server_round(self._h, C.byref(ran)))
        return bool(ran.value)

    def poll(self, capacity: int = 256) -> list:
        buf = (_Completion * capacity)()
        n = C.c_int32()
        _check(self._lib.lbm_server_poll(self._h, buf, int(capacity), C.byref(n)))
        return [{f: getattr(buf[i], f) for f, _ in _Completion._fields_} for i in range(n.value)]

    def take_result(self, rid: int, copy: bool = True):
        size = self._sizes.pop(rid)
        if not copy:
            status = self._lib.lbm_server_take_result(self._h, int(rid), None, None)
            _check(status)
            return None
        rho = np.empty((size[2], size[1], size[0]), dtype=self.dtype)
        u = np.empty((3, size[2], size[1], size[0]), dtype=self.dtype)
        _check(self._lib.lbm_server_take_result(self._h, int(rid), rho.ctypes.data, u.ctypes.data))
        return rho, u

    def stats(self) -> dict:
        st = _ServerStats()
        _check(self._lib.lbm_server_get_stats(self._h, C.byref(st)))
        return {f: getattr(st, f) for f, _ in _ServerStats._fields_}
