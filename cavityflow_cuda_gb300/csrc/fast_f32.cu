// fast_f32.cu -- instantiates the vectorised step kernels for F32 storage
// (one translation unit per storage type so they compile in parallel).
#include "lbm_fast.cuh"
#include "lbm_kernels.h"

namespace lbm {

cudaError_t launch_fast_f32(int variant, bool alpha, void* dd, const Grid& g, const Params& p, int lid_y,
                           cudaStream_t st)
{
    return launch_fast_menu<F32>(variant, alpha, dd, g, p, lid_y, st);
}

}  // namespace lbm
