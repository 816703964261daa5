// fast_f64.cu -- instantiates the vectorised and the row-pipelined (bulk copy)
// step kernels and the batch kernels for F64 storage (one translation unit per
// storage type, so they compile in parallel).
#include "lbm_fast.cuh"
#include "lbm_kernels.h"
#include "lbm_tma.cuh"

namespace lbm {

cudaError_t launch_fast_f64(int variant, bool alpha, void* dd, const Grid& g, const Params& p, int lid_y,
                            cudaStream_t st)
{
    return launch_fast_menu<F64>(variant, alpha, dd, g, p, lid_y, st);
}

cudaError_t launch_tma_f64(bool alpha, void* dd, const Grid& g, const Params& p, int lid_y, int rows, int stages,
                           int consumer_warps, int* err, cudaStream_t st)
{
    return launch_tma_impl<F64>(alpha, dd, g, p, lid_y, rows, stages, consumer_warps, err, st);
}

cudaError_t launch_batch_f64(int variant, bool alpha, const BatchArgs& a, cudaStream_t st)
{
    return launch_batch_menu<F64>(variant, alpha, a, st);
}

}  // namespace lbm
