// lbm_internal.h -- definitions shared by the C ABI translation units
// (lbm_capi.cu, lbm_batch.cu); not part of the public interface.
#pragma once

#include <cstdint>
#include <exception>
#include <new>
#include <cuda_runtime.h>

#include "../../include/lbm_gb300.h"
#include "lbm_kernels.h"

struct lbm_batch;

struct lbm_solver {
    lbm::Grid g{};
    int storage = 0;
    int device = 0;
    lbm::Params p{};
    int bc[6] = {0, 0, 0, 0, 0, 0};
    void* dd = nullptr;             // populations, 19 * g.S elements
    uint8_t* flags = nullptr;       // one byte per cell, reference layout
    void* macros = nullptr;         // 4 * cells values (rho, jx, jy, jz)
    bool macros_fresh = false;
    double* scratch = nullptr;      // reduction partials (4 per block) + result (4)
    unsigned long long* counts = nullptr;  // cavity-flag check counters [0..1], kernel error flag [2],
                                           // step words [4] (see step_words)
    double* host_out = nullptr;     // pinned, 4 doubles
    float* staging = nullptr;       // 16-bit storage: one packed slot cuboid
    size_t staging_elems = 0;
    int64_t counter = 0;
    bool last_alpha = false;
    int lid_y = -1;                 // fast path: lid row (ny) or 0 for none; -1: flag-array path
    int variant = 0;                // launch variant of the vectorised kernels
    bool fma = false;               // FP64: fused multiply-adds in the vectorised steps
    int lid_mode = 0;               // LBM_LID_INJECTION or LBM_LID_MOVING_WALL; the wall moves
                                    // while p.wall_y > 0
    cudaStream_t capture_stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    int64_t device_bytes = 0;
    bool owns_dd = true;            // false: populations live in a batch's pool
    lbm_batch* batch = nullptr;     // the batch this solver is a domain view of
};

namespace lbm_detail {

int fail(int status, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);
int elem_bytes(int storage);
int value_bytes(int storage);
int default_variant(int storage);
// Default register variant of the batch kernel (many small domains).
int default_batch_variant(int storage);
// Creates a solver; with `external_dd` its populations live there (a batch
// pool) and are initialised but never freed by the solver.
// x1_align: 32 (the default layout) or 8 (the packed rows of batch pools,
// see make_grid).
int create_solver(const lbm_params* prm, void* external_dd, lbm_solver** out, int x1_align = 32);
void destroy_solver(lbm_solver* s);
int* err_flag(lbm_solver* s);
// Two device words of the solver: [0] the first step of a graph replay,
// [1] always zero (the base of directly launched steps).
uint32_t* step_words(lbm_solver* s);
int check_kernel_flag(lbm_solver* s);

// Runs an entry point's body with C++ exceptions turned into status codes,
// since none may cross the C interface: a host buffer too large for memory
// (a checkpoint or VTK file of a big domain) throws std::bad_alloc.
template <class Body>
int guarded(const char* entry, Body&& body)
{
    try {
        return body();
    } catch (const std::bad_alloc&) {
        return fail(LBM_ERR_OUT_OF_MEMORY, "%s: host allocation failed", entry);
    } catch (const std::exception& e) {
        return fail(LBM_ERR_IO, "%s: %s", entry, e.what());
    }
}

// Largest domain any entry point accepts, halo included: 2^40 cells, far
// beyond device memory (8 bytes x 19 slots x 2^40 cells is 167 TB) and small
// enough that no element or byte count derived from it overflows 64 bits.
constexpr long long kMaxDomainCells = 1LL << 40;
// Each axis in [1, 2^20] and (nx+2)(ny+2)(nz+2) <= kMaxDomainCells.
inline bool domain_size_ok(const int32_t size[3])
{
    long long cells = 1;
    for (int d = 0; d < 3; ++d) {
        if (size[d] <= 0 || size[d] > (1 << 20)) return false;
        cells *= (long long)size[d] + 2;  // < 2^40 * (2^20 + 3) < 2^63
        if (cells > kMaxDomainCells) return false;
    }
    return true;
}

}  // namespace lbm_detail
