// fast_fma.cu -- the vectorised step kernels with the collision's multiply-adds
// fused (lbm_params.fused_multiply_add), as the reference's own nvcc build
// (-use_fast_math: fused multiply-adds, FP32 subnormals flushed to zero)
// compiles its kernels: FP64 (storage type F64F) and FP32 (F32F).  The only
// translation unit compiled with -fmad=true -ftz=true
// (cavityflow_cuda_gb300/build.py); the storage types keep these
// instantiations apart from F64's and F32's unfused ones.
#include "lbm_fast.cuh"
#include "lbm_kernels.h"

namespace lbm {

cudaError_t launch_fast_f64fma(int variant, bool alpha, void* dd, const Grid& g, const Params& p, int lid_y,
                               cudaStream_t st)
{
    return launch_fast_menu<F64F>(variant, alpha, dd, g, p, lid_y, st);
}

cudaError_t launch_fast_f32fma(int variant, bool alpha, void* dd, const Grid& g, const Params& p, int lid_y,
                               cudaStream_t st)
{
    return launch_fast_menu<F32F>(variant, alpha, dd, g, p, lid_y, st);
}

}  // namespace lbm
