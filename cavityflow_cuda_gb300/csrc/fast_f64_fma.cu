// fast_f64_fma.cu -- the vectorised step kernels for FP64 storage with the
// collision's multiply-adds fused (lbm_params.fused_multiply_add), as the
// reference's own nvcc build contracts them.  The only translation unit
// compiled with -fmad=true (cavityflow_cuda_gb300/build.py); its storage type
// F64F keeps these instantiations apart from F64's unfused ones.
#include "lbm_fast.cuh"
#include "lbm_kernels.h"

namespace lbm {

cudaError_t launch_fast_f64fma(int variant, bool alpha, void* dd, const Grid& g, const Params& p, int lid_y,
                               cudaStream_t st)
{
    return launch_fast_menu<F64F>(variant, alpha, dd, g, p, lid_y, st);
}

}  // namespace lbm
