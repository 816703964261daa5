"""lbm_reduce_noalloc: the FP64 mass/momentum reduction for callers that cannot
call cudaMalloc (device memory owned by their own pool or budget, or loops that
cannot take the implicit synchronisation of cudaMalloc/cudaFree).  It reduces
arrays the caller owns, with a static device array as its only scratch.

Checked through the C ABI against lbm_reduce on the same state, with the
tolerance the other reduction tests use, on two calls in a row (the second
call finds the first call's partial sums still in the shared scratch).  This
file is collected last so that a run that stops at the first failure has run
every other test first."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STORAGE = {"f64": 0, "f32": 1}


def _entry(lib):
    fn = lib.lbm_reduce_noalloc
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    return fn


@pytest.mark.parametrize("storage", ["f64", "f32"])
def test_noalloc_reduction_matches_lbm_reduce(gpu, storage):
    import torch

    from cavityflow_cuda_gb300 import CLbmSolverGB300

    fn = _entry(gpu)
    n = (21, 17, 13)
    stream = torch.cuda.current_stream()
    out_dev = torch.full((4,), -1.0, dtype=torch.float64, device="cuda")
    with CLbmSolverGB300(n, 1.65, 0.06, storage=storage) as s:
        for steps in (37, 1):  # the first call after an alpha step, the second after a beta step
            s.run(steps)
            want = s.reduce()
            dd = torch.from_numpy(s.get_all()).to("cuda")
            flags = torch.from_numpy(s.flags_all()).to("cuda")
            rc = fn(dd.data_ptr(), flags.data_ptr(), (C.c_int32 * 3)(*n), STORAGE[storage],
                    s.info()["last_step_was_alpha"], out_dev.data_ptr(), stream.cuda_stream)
            assert rc == 0, gpu.lbm_last_error()
            stream.synchronize()
            got = out_dev.cpu().numpy()
            np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12)


def _compare(gpu, fn, s, n, storage, steps_list):
    import torch

    stream = torch.cuda.current_stream()
    out_dev = torch.full((4,), -1.0, dtype=torch.float64, device="cuda")
    for steps in steps_list:
        s.run(steps)
        want = s.reduce()
        dd = torch.from_numpy(s.get_all()).to("cuda")
        flags = torch.from_numpy(s.flags_all()).to("cuda")
        rc = fn(dd.data_ptr(), flags.data_ptr(), (C.c_int32 * 3)(*n), STORAGE[storage],
                s.info()["last_step_was_alpha"], out_dev.data_ptr(), stream.cuda_stream)
        assert rc == 0, gpu.lbm_last_error()
        stream.synchronize()
        np.testing.assert_allclose(out_dev.cpu().numpy(), want, rtol=1e-12, atol=1e-12)


def test_noalloc_at_the_plane_limit(gpu):
    """nz = 4096, the largest domain the static scratch holds: every one of its
    4096 rows is written and summed."""
    from cavityflow_cuda_gb300 import CLbmSolverGB300

    n = (4, 4, 4096)
    with CLbmSolverGB300(n, 1.65, 0.06, storage="f32") as s:
        _compare(gpu, _entry(gpu), s, n, "f32", (9, 2))


@pytest.mark.parametrize("storage", ["f64", "f32"])
def test_noalloc_with_an_interior_obstacle(gpu, storage):
    """An obstacle block inside the fluid: the mass of the wall slots that
    fluid cells push into counts for non-halo obstacles as well."""
    from cavityflow_cuda_gb300 import OBSTACLE, CLbmSolverGB300

    n = (19, 15, 12)
    with CLbmSolverGB300(n, 1.6, 0.05, storage=storage) as s:
        s.setFlags(np.full((3, 4, 2), OBSTACLE, np.int32), (6, 5, 4), (3, 4, 2))
        assert s.info()["fast_path"] == 0
        _compare(gpu, _entry(gpu), s, n, storage, (25, 1))


def test_noalloc_rejects_domains_beyond_its_scratch(gpu):
    import torch

    fn = _entry(gpu)
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = fn(buf.data_ptr(), buf.data_ptr(), (C.c_int32 * 3)(8, 8, 5000), 0, 0, buf.data_ptr(), None)
    assert rc == 1
    assert b"4096-plane limit" in gpu.lbm_last_error()
