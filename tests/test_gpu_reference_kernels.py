"""The contract's parity bar against the reference's own CUDA kernels.

oracle/_ref/lbm_ref_kernels.cubin holds src/gpukernels/lbm_{init,alpha,beta}.cu
of the reference, compiled from source with its own nvcc flags (-O3
-use_fast_math -maxrregcount=80, so FP32 and FP64 arithmetic is contracted
into fused multiply-adds, unlike the reference's CPU kernels, which this
solver matches bit for bit).  Both solvers start from the same state and run
1000 steps of the same lid-driven cavity; the velocity j of every interior
cell must agree to max |du| <= 1e-6 (FP32) and <= 1e-12 (FP64), and FP64 mass
to 1e-10 relative.  Skipped where the cubin was not built (it needs the
reference checkout at build time).
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
                                                   ("f64", np.float64, 1e-12, True)])
@pytest.mark.parametrize("n", [(64, 64, 64), (48, 40, 36)])
def test_velocity_matches_reference_cuda_kernels(gpu, refkernels, storage, dtype, tol, fma, n):
    """Also for FP64 with fused multiply-adds (lbm_params.fused_multiply_add)."""
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
