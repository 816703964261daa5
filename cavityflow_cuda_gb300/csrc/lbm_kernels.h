// lbm_kernels.h -- host-side launch interface of the solver's kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "lbm_core.cuh"

namespace lbm {

constexpr int kReduceBlock = 256;     // threads per block, FP64 reduction
constexpr int kReduceMaxBlocks = 1024;

// Face flags of the six halo faces: -x, +x, -y, +y, -z, +z.
struct Bc {
    int f[6];
};

// Stores a detail message for lbm_last_error() on this thread; returns status.
int record_error(int status, const char* fmt, ...);

// Kernel launches queued by this library since load, and a correction for
// launches that were captured into a graph rather than run.
long long kernel_launches();
void add_launches(long long n);

cudaError_t launch_init(int storage, void* dd, uint8_t* flags, const Grid& g, const Bc& bc, cudaStream_t st);
// Populations at rest only (no flag array).
cudaError_t launch_init_populations(int storage, void* dd, const Grid& g, cudaStream_t st);
cudaError_t launch_check_cavity(const uint8_t* flags, const Grid& g, unsigned long long* counts, cudaStream_t st);
// Storage types whose step kernels round stochastically, keyed by the step
// (Params::step_base/step_off); a graph replaying such launches needs the
// word at step_base set to its first step before each replay.
inline bool storage_stochastic(int storage) { return storage == 4; }
cudaError_t launch_set_step(uint32_t* word, uint32_t value, cudaStream_t st);
// One block waiting on an mbarrier that nothing arrives at, bounded by
// limit_ns; raises bit 1 of *err when it gives up (lbm_selftest_bounded_wait).
cudaError_t launch_bounded_wait_probe(int* err, uint64_t limit_ns, cudaStream_t st);
// Box-cavity step.  Variants 0..kRegisterVariants-1 index kFastMenu, the
// register kernels of lbm_fast.cuh; the rest index kTmaMenu, the
// row-pipelined bulk-copy kernels of lbm_tma.cuh.  A variant that does not
// fit the domain returns cudaErrorInvalidValue before launching anything.
// `err` receives the bulk-copy kernels' timeout flag.
//
// Launch shape of one register kernel: cells per thread as a fraction of a
// 16-byte vector (cpt_div 1: 16-byte vectors, 2: 8-byte, 4: 4-byte), threads
// per block, and the minimum resident blocks per SM requested from the
// register allocator (65536 / (block * minb) registers per thread at most).
struct KernelShape {
    int cpt_div;
    int block;
    int minb;
};
// A register variant: the alpha and the beta kernel have their own shapes
// (the population layout does not depend on them), and the beta kernel
// exchanges the odd element of its shifted slots either inside each warp
// (shuffles; warp-edge lanes use scalar accesses) or across the whole block
// (shuffles plus shared memory; only block- and row-edge lanes do).
// With `direct`, beta exchanges nothing: each thread loads and stores the
// one-cell-shifted windows of the c_x = +-1 slots itself with element-aligned
// accesses (2-4 per window), so there are no shuffles, shared memory or
// barriers and no row- or block-edge cases.
// `packed` (16-bit storage; other storages run the direct beta): the direct
// windows with two cells per 32-bit word and paired conversions
// (beta_fast_pk), loading each window as its pieces (1) or as the aligned
// vector plus one element (2).
struct FastVariant {
    KernelShape alpha;
    KernelShape beta;
    bool block_exchange;
    bool direct = false;
    int packed = 0;
};
constexpr int kRegisterVariants = 24;
constexpr FastVariant kFastMenu[kRegisterVariants] = {
    {{1, 256, 1}, {1, 256, 1}, false},  // 16-byte vectors, registers unconstrained
    {{1, 256, 2}, {1, 256, 2}, false},  // 16-byte vectors, <= 128 registers
    {{1, 128, 4}, {1, 128, 4}, false},  // 16-byte vectors, <= 128 registers, smaller blocks
    {{2, 256, 2}, {2, 256, 2}, false},  // 8-byte vectors, <= 128 registers
    {{2, 256, 3}, {2, 256, 3}, false},  // 8-byte vectors, <= 85 registers
    {{2, 128, 5}, {2, 128, 5}, false},  // 8-byte vectors, <= 102 registers
    {{4, 256, 2}, {4, 256, 2}, false},  // 4-byte vectors (FP64: one cell), <= 128 registers
    {{4, 256, 3}, {4, 256, 3}, false},  // 4-byte vectors (FP64: one cell), <= 85 registers
    {{2, 64, 8}, {2, 64, 8}, true},     // 8-byte vectors, two-warp blocks, block exchange
    {{2, 128, 4}, {2, 128, 4}, true},   // 8-byte vectors, four-warp blocks, block exchange
    {{1, 64, 4}, {2, 64, 8}, true},     // alpha 16-byte, beta 8-byte vectors, block exchange
    {{1, 64, 4}, {1, 64, 4}, true},     // 16-byte vectors, two-warp blocks, block exchange
    {{1, 64, 4}, {2, 128, 4}, true},    // alpha 16-byte two-warp, beta 8-byte four-warp blocks
    {{2, 64, 8}, {2, 64, 8}, false, true},    // 8-byte vectors, two-warp blocks, direct shifted windows
    {{2, 128, 4}, {2, 128, 4}, false, true},  // 8-byte vectors, four-warp blocks, direct
    {{1, 64, 4}, {2, 64, 8}, false, true},    // alpha 16-byte, beta 8-byte, direct
    {{1, 64, 4}, {1, 64, 4}, false, true},    // 16-byte vectors, two-warp blocks, direct
    {{2, 256, 2}, {2, 256, 2}, false, true},  // 8-byte vectors, eight-warp blocks, direct
    {{1, 64, 4}, {2, 64, 10}, false, true, 1},  // alpha 16-byte; beta 8-byte packed pieces, <= 102 registers
    {{1, 64, 4}, {2, 64, 8}, false, true, 1},   // the same, <= 128 registers
    {{1, 64, 4}, {2, 64, 10}, false, true, 2},  // alpha 16-byte; beta 8-byte packed, vector loads
    {{1, 64, 4}, {2, 64, 8}, false, true, 2},   // the same, <= 128 registers
    {{2, 64, 8}, {2, 64, 8}, false, true, 2},   // 8-byte alpha, packed beta with vector loads, <= 128 registers
    {{2, 64, 8}, {2, 64, 10}, false, true, 2},  // the same, <= 102 registers (22 and 23 fit the batch rows)
};
struct TmaConfig {
    int rows;            // rows per work unit
    int stages;          // shared-memory buffers
    int consumer_warps;  // warps that collide (plus one producer warp)
};
constexpr int kTmaVariants = 6;
constexpr TmaConfig kTmaMenu[kTmaVariants] = {
    {1, 3, 6}, {1, 4, 6}, {2, 2, 8}, {2, 3, 8}, {1, 2, 4}, {4, 2, 8},
};
constexpr int kFastVariantCount = kRegisterVariants + kTmaVariants;
// Storage code of the FP64 step kernels with fused multiply-adds (F64F, built
// in fast_fma.cu); accepted by launch_fast_step, fast_variant_fits and
// fast_variant_shape only.  Its bulk-copy variants run the unfused kernels.
constexpr int kStorageF64Fma = 5;
// The same for FP32 (F32F); its bulk-copy variants run the unfused kernels.
constexpr int kStorageF32Fma = 6;
// Bytes per stored population of a storage code (kernel storage codes included).
inline int storage_elem_bytes(int storage)
{
    return storage == 0 || storage == kStorageF64Fma ? 8 : storage == 1 || storage == kStorageF32Fma ? 4 : 2;
}
cudaError_t launch_fast_step(int storage, int variant, bool alpha, void* dd, const Grid& g, const Params& p,
                             int lid_y, int* err, cudaStream_t st);
// Whether a variant fits this domain: its vectors' alignment in the domain's
// row layout (register variants), shared memory (bulk-copy variants).
bool fast_variant_fits(int storage, int variant, const Grid& g);
// Cells per thread and threads per block of a variant's alpha or beta kernel
// (for a row of nx cells).
void fast_variant_shape(int storage, int variant, bool alpha, int nx, int& cells_per_thread, int& block_threads);

// Batches of box cavities (lbm_fast.cuh): register variants only.
struct BatchDomain;
struct BatchArgs {
    void* pool;               // the domains' populations
    const BatchDomain* doms;  // packed table
    const int* vb_dom;        // domain of each virtual block of the launched kernel
    long long vblocks;        // virtual blocks of the launched kernel (alpha or beta shape)
    const uint32_t* step_base;
    uint32_t step_off;        // domain d's step: *step_base + step_off + d.step0
};
cudaError_t launch_batch_step(int storage, int variant, bool alpha, const BatchArgs& a, cudaStream_t st);
cudaError_t launch_batch_f64(int variant, bool alpha, const BatchArgs& a, cudaStream_t st);
cudaError_t launch_batch_f32(int variant, bool alpha, const BatchArgs& a, cudaStream_t st);
cudaError_t launch_batch_f16s(int variant, bool alpha, const BatchArgs& a, cudaStream_t st);
cudaError_t launch_batch_f16sr(int variant, bool alpha, const BatchArgs& a, cudaStream_t st);
cudaError_t launch_batch_bf16s(int variant, bool alpha, const BatchArgs& a, cudaStream_t st);
// Rebuilds vb_dom for kernel `which` (0 alpha, 1 beta) from the table.
cudaError_t launch_batch_map(const BatchDomain* doms, int ndom, long long vblocks, int which, int* vb_dom,
                             cudaStream_t st);
cudaError_t launch_fast_f64(int variant, bool alpha, void* dd, const Grid& g, const Params& p, int lid_y,
                            cudaStream_t st);
cudaError_t launch_fast_f64fma(int variant, bool alpha, void* dd, const Grid& g, const Params& p, int lid_y,
                               cudaStream_t st);
cudaError_t launch_fast_f32fma(int variant, bool alpha, void* dd, const Grid& g, const Params& p, int lid_y,
                               cudaStream_t st);
cudaError_t launch_fast_f32(int variant, bool alpha, void* dd, const Grid& g, const Params& p, int lid_y,
                            cudaStream_t st);
cudaError_t launch_fast_f16s(int variant, bool alpha, void* dd, const Grid& g, const Params& p, int lid_y,
                             cudaStream_t st);
cudaError_t launch_fast_bf16s(int variant, bool alpha, void* dd, const Grid& g, const Params& p, int lid_y,
                              cudaStream_t st);
cudaError_t launch_fast_f16sr(int variant, bool alpha, void* dd, const Grid& g, const Params& p, int lid_y,
                              cudaStream_t st);
cudaError_t launch_tma_f64(bool alpha, void* dd, const Grid& g, const Params& p, int lid_y, int rows, int stages,
                           int consumer_warps, int* err, cudaStream_t st);
cudaError_t launch_tma_f32(bool alpha, void* dd, const Grid& g, const Params& p, int lid_y, int rows, int stages,
                           int consumer_warps, int* err, cudaStream_t st);
cudaError_t launch_tma_f16s(bool alpha, void* dd, const Grid& g, const Params& p, int lid_y, int rows, int stages,
                            int consumer_warps, int* err, cudaStream_t st);
cudaError_t launch_tma_bf16s(bool alpha, void* dd, const Grid& g, const Params& p, int lid_y, int rows,
                             int stages, int consumer_warps, int* err, cudaStream_t st);
cudaError_t launch_tma_f16sr(bool alpha, void* dd, const Grid& g, const Params& p, int lid_y, int rows,
                             int stages, int consumer_warps, int* err, cudaStream_t st);
cudaError_t launch_general_step(int storage, bool alpha, void* dd, const uint8_t* flags, const Grid& g,
                                const Params& p, int3 origin, int3 size, cudaStream_t st);
cudaError_t launch_macros(int storage, const void* dd, const uint8_t* flags, const Grid& g, bool last_alpha,
                          double lid_u, void* out, cudaStream_t st);
// Interior density and velocity of a box cavity with the lid on y = ny, from
// the geometry; packed x fastest (rho, jx, jy, jz planes); `out` may be
// mapped host memory.
cudaError_t launch_macros_cavity(int storage, const void* dd, const Grid& g, bool last_alpha, double lid_u,
                                 void* out, cudaStream_t st);
int reduce_blocks(const Grid& g);
cudaError_t launch_reduce(int storage, const void* dd, const uint8_t* flags, const Grid& g, bool last_alpha,
                          double* partials, double* out, cudaStream_t st);
cudaError_t launch_pack_slot(int storage, const void* dd, const Grid& g, int k, int3 origin, int3 size,
                             float* out, cudaStream_t st);
cudaError_t launch_unpack_slot(int storage, void* dd, const Grid& g, int k, int3 origin, int3 size,
                               const float* in, cudaStream_t st);

}  // namespace lbm
