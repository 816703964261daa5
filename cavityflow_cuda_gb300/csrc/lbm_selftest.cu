// lbm_selftest.cu -- a check of the bounded device-side waits without any GPU
// fault: one block waits on an mbarrier that nothing arrives at, through the
// same bounded wait the bulk-copy kernels use (lbm_tma.cuh), and raises the
// error flag when the limit passes (lbm_selftest_bounded_wait).
#include <cstdint>

#include "lbm_kernels.h"
#include "lbm_tma.cuh"

namespace lbm {

namespace {

__global__ void bounded_wait_probe(int* __restrict__ err, const uint64_t limit_ns)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        tma::mbar_init(&bar, 1);
        tma::fence_mbar_init();
    }
    __syncthreads();
    // no thread arrives, so phase 0 never completes
    if (threadIdx.x == 0 && !tma::mbar_wait(&bar, 0u, limit_ns)) atomicOr(err, 1);
}

}  // namespace

cudaError_t launch_bounded_wait_probe(int* err, uint64_t limit_ns, cudaStream_t st)
{
    bounded_wait_probe<<<1, 32, 0, st>>>(err, limit_ns);
    return cudaGetLastError();
}

}  // namespace lbm
