// lbm_pair.cuh -- one launch for an alpha step and the beta step after it
// (the pair src/CController.cpp:1278-1287 runs as two kernel calls), so that
// beta reads the populations alpha has just written from L2 instead of DRAM.
//
// The work is a sequence of plane jobs, each split into items of BLOCK
// threads x CPT cells (the thread grouping of alpha_fast / beta_fast_blk),
// handed out K consecutive items per ticket.
// Alpha of plane p touches only plane p's slots; beta of plane q reads and
// writes slots of planes q-1..q+1, so it needs alpha done on those planes.
// Jobs are ordered alpha(1..D), then alpha(q+D), beta(q) alternately, then
// the last betas: alpha runs D planes ahead of beta, and the D+2 planes
// between them are the L2 working set (D from the domain's plane size).
//
// A CTA takes tickets from a global counter (the next ticket is fetched while
// the current one runs).  An alpha ticket ends with a block barrier and a
// release increment of its plane's completion counter; a beta ticket first
// waits (acquire) until the counters of its three planes are full.  Every
// dependency of a ticket is a smaller ticket and alpha tickets never wait, so
// the smallest waiting ticket always has its alphas running or done: no
// co-residency is needed.  The wait is bounded (%globaltimer, 2 s): on expiry
// the kernel raises the error flag and goes on, so it cannot hang the GPU.
// Beta loads bypass L1 (ld.global.cg), which could hold lines another SM has
// rewritten in this launch.
//
// The per-cell arithmetic is that of alpha_cells / beta_cells_blk, in the
// same order, so results are bit-identical to the two separate kernels.
#pragma once

#include <cstdint>
#include <utility>

#include "lbm_core.cuh"
#include "lbm_fast.cuh"
#include "lbm_kernels.h"

namespace lbm {

namespace pair {

__device__ __forceinline__ uint64_t now_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t load_acquire(const uint32_t* p)
{
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Completion of an alpha ticket: prior writes of the block (ordered by the
// barrier before it) become visible before the increment.
__device__ __forceinline__ void add_release(uint32_t* p, uint32_t v)
{
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s

// Job j of the sequence (see the file header): alpha or beta of `plane`.
__device__ __forceinline__ void job_of(uint32_t j, int nz, int D, bool& alpha, int& plane)
{
    if (j < (uint32_t)D) {
        alpha = true;
        plane = 1 + (int)j;
        return;
    }
    const uint32_t m = j - (uint32_t)D;
    const uint32_t inter = 2u * (uint32_t)(nz - D);
    if (m < inter) {
        alpha = (m & 1u) == 0;
        plane = alpha ? D + 1 + (int)(m >> 1) : 1 + (int)(m >> 1);
        return;
    }
    alpha = false;
    plane = nz - D + 1 + (int)(m - inter);
}

// Thread 0 of a beta item: waits until alpha is done on planes q-1..q+1
// (halo planes have no alpha).  False if the time limit passed first.
__device__ __forceinline__ bool wait_alpha(const uint32_t* done, int q, int nz, uint32_t need)
{
    uint64_t deadline = 0;
    for (int p = q - 1; p <= q + 1; ++p) {
        if (p < 1 || p > nz) continue;
        while (load_acquire(done + p) < need) {
            const uint64_t t = now_ns();
            if (deadline == 0) deadline = t + kWaitLimitNs;
            else if (t > deadline) return false;
            __nanosleep(32);
        }
    }
    return true;
}

}  // namespace pair

// sync[0]: ticket counter; sync[p], p = 1..nz: alpha tickets done on plane p.
// All zero at launch.  div_tickets divides by the tickets per plane; K items
// per ticket.  The step of alpha is step_of(step_base, step_off), beta's the
// next one.
template <class St, int CPT, int BLOCK, int MINB, bool kExchange, int K>
__global__ void __launch_bounds__(BLOCK, MINB) pair_fused(typename St::bits* __restrict__ dd, const Grid g,
                                                          const typename St::T inv_tau,
                                                          const typename St::T lid_u, const int lid_y,
                                                          const uint32_t* __restrict__ step_base,
                                                          const uint32_t step_off, const FastDiv divG,
                                                          const FastDiv div_tickets, const uint32_t items,
                                                          const int lookahead, uint32_t* __restrict__ sync,
                                                          int* __restrict__ err)
{
    const int G = (g.nx + CPT - 1) / CPT;
    const uint32_t tickets = div_tickets.d;  // tickets per plane
    const int nz = g.nz;
    const int D = lookahead < nz ? lookahead : nz;
    const uint32_t total = 2u * (uint32_t)nz * tickets;
    const uint32_t step = step_of<St>(step_base, step_off);
    // Double-buffered so that a ticket's slot is not rewritten before every
    // thread has read it (two block barriers lie between).
    __shared__ uint32_t s_ticket[2];
    uint32_t next = 0;
    if (threadIdx.x == 0) next = atomicAdd(sync, 1u);
    for (int buf = 0;; buf ^= 1) {
        if (threadIdx.x == 0) {
            s_ticket[buf] = next;
            next = atomicAdd(sync, 1u);  // used by the next ticket: its latency hides behind this one
        }
        __syncthreads();
        const uint32_t t = s_ticket[buf];
        if (t >= total) break;
        const uint32_t job = div_tickets.div(t);
        const uint32_t first = (t - job * tickets) * K;
        const uint32_t last = first + K < items ? first + K : items;
        bool alpha;
        int plane;
        pair::job_of(job, nz, D, alpha, plane);
        if (alpha) {
            for (uint32_t item = first; item < last; ++item)
                alpha_cells<St, CPT>(dd, g, inv_tau, lid_u, lid_y,
                                     cells_of_plane(g, G, divG, item * BLOCK + threadIdx.x, plane), step);
            __syncthreads();
            if (threadIdx.x == 0) pair::add_release(sync + plane, 1u);
        } else {
            if (threadIdx.x == 0 && !pair::wait_alpha(sync, plane, nz, tickets)) atomicOr(err, 4);
            __syncthreads();
            for (uint32_t item = first; item < last; ++item) {
                const Cells c = cells_of_plane(g, G, divG, item * BLOCK + threadIdx.x, plane);
                if constexpr (kExchange)
                    beta_cells_blk<St, CPT, BLOCK, true>(dd, g, inv_tau, lid_u, lid_y, c, step + 1);
                else beta_cells<St, CPT, true>(dd, g, inv_tau, lid_u, lid_y, c, step + 1);
            }
        }
    }
}

// Lookahead D for a plane of `plane_bytes` (all 19 slots) and an L2 working
// set of window_mb: D + 2 planes, at least 1 and at most 8 planes ahead.
inline int pair_lookahead(long long plane_bytes, int window_mb)
{
    long long d = ((long long)window_mb << 20) / (plane_bytes > 0 ? plane_bytes : 1) - 2;
    if (d < 1) d = 1;
    if (d > 8) d = 8;
    return (int)d;
}

template <class St, int PV>
cudaError_t launch_pair_variant(void* dd, const Grid& g, const Params& p, int lid_y, uint32_t* sync, int* err,
                                cudaStream_t st)
{
    using T = typename St::T;
    constexpr PairConfig pc = kPairMenu[PV];
    constexpr FastVariant fv = kFastMenu[pc.base];
    static_assert(fv.alpha.cpt_div == fv.beta.cpt_div && fv.alpha.block == fv.beta.block &&
                      fv.alpha.minb == fv.beta.minb,
                  "a fused pair runs alpha and beta with one shape");
    constexpr KernelShape k = fv.alpha;
    constexpr int CPT = shape_cpt<St>(k);
    auto kern = pair_fused<St, CPT, k.block, k.minb, fv.block_exchange, pc.items_per_ticket>;
    const long long G = (g.nx + CPT - 1) / CPT;
    const long long items = (G * g.ny + k.block - 1) / k.block;
    const long long tickets = (items + pc.items_per_ticket - 1) / pc.items_per_ticket;
    if (items <= 0 || 2ll * g.nz * tickets >= (1ll << 31)) return cudaErrorInvalidValue;
    const int D = pair_lookahead(g.PY * (long long)Q * (long long)sizeof(typename St::bits), pc.window_mb);
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, k.block, 0);
    if (e == cudaSuccess) e = cudaMemsetAsync(sync, 0, (size_t)(g.nz + 1) * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    long long grid = (long long)(per_sm > 0 ? per_sm : 1) * sms;
    if (grid > 2ll * g.nz * tickets) grid = 2ll * g.nz * tickets;
    kern<<<(int)grid, k.block, 0, st>>>(static_cast<typename St::bits*>(dd), g, T(p.inv_tau), T(p.lid_u), lid_y,
                                        p.step_base, p.step_off, FastDiv::make((uint32_t)G),
                                        FastDiv::make((uint32_t)tickets), (uint32_t)items, D, sync, err);
    return cudaGetLastError();
}

template <class St, size_t... I>
cudaError_t launch_pair_table(int pv, void* dd, const Grid& g, const Params& p, int lid_y, uint32_t* sync, int* err,
                              cudaStream_t st, std::index_sequence<I...>)
{
    using Fn = cudaError_t (*)(void*, const Grid&, const Params&, int, uint32_t*, int*, cudaStream_t);
    static constexpr Fn table[] = {&launch_pair_variant<St, (int)I>...};
    return table[pv](dd, g, p, lid_y, sync, err, st);
}

// pv indexes kPairMenu.
template <class St>
cudaError_t launch_pair_menu(int pv, void* dd, const Grid& g, const Params& p, int lid_y, uint32_t* sync, int* err,
                             cudaStream_t st)
{
    if (pv < 0 || pv >= kPairVariants) return cudaErrorInvalidValue;
    return launch_pair_table<St>(pv, dd, g, p, lid_y, sync, err, st, std::make_index_sequence<kPairVariants>{});
}

}  // namespace lbm
