// Test infrastructure, not part of the product: one translation unit holding
// the reference's own CUDA kernels (lbm_init, lbm_kernel_alpha,
// lbm_kernel_beta of src/gpukernels/), compiled from the read-only reference
// checkout into a device-only cubin (oracle/Makefile, target refgpu).  The
// tests and the reference arm of bench.py load it with the CUDA driver API
// (oracle/ref_gpu.py) to compare against and to time the reference kernels on
// the same GPU.  Nothing here is copied: the includes resolve into the
// reference checkout.
#include "gpukernels/lbm_init.cu"
#include "gpukernels/lbm_alpha.cu"
#include "gpukernels/lbm_beta.cu"
