// lbm_fast.cuh -- the vectorised A-A step kernels of the box cavity (the hot
// path).  Flags are implied by coordinates: interior cells are FLUID except
// the lid row y = lid_y (VELOCITY_INJECTION); the halo is OBSTACLE.
//
//   alpha_fast  -- src/gpukernels/lbm_alpha.cu:22-532 restated: a thread owns
//                  CPT consecutive cells of one x row, reads their 19 slots
//                  with one vector access each, collides and writes every
//                  population to its opposite slot.
//   beta_fast   -- src/gpukernels/lbm_beta.cu:32-915 restated: the same
//                  thread pulls the 19 incoming populations from the
//                  neighbours' slots, collides and pushes the results back to
//                  the same addresses.  Slots with c_x = +-1 are read and
//                  written one cell off the vector grid; the element that
//                  crosses into the next thread's group is exchanged with
//                  warp shuffles, and only lanes at a warp or row edge touch
//                  that element with a scalar access.
//
// Template parameters: St storage type, CPT cells per thread (one vector of
// CPT elements per slot: 16 or 8 bytes), BLOCK threads per block, MINB the
// minimum resident blocks per SM requested from the register allocator.
#pragma once

#include <cstdint>
#include <type_traits>

#include "lbm_core.cuh"

namespace lbm {

template <int I, int N, class F>
__device__ __forceinline__ void static_for(F&& f)
{
    if constexpr (I < N) {
        f(std::integral_constant<int, I>{});
        static_for<I + 1, N>(f);
    }
}

template <int BYTES> struct RawVec;
template <> struct RawVec<16> { using type = uint4; };
template <> struct RawVec<8> { using type = uint2; };
template <> struct RawVec<4> { using type = unsigned int; };
template <> struct RawVec<2> { using type = unsigned short; };

// Aligned access to N consecutive storage elements, converted to the
// arithmetic type.
template <class St, int N>
struct Vio {
    using bits = typename St::bits;
    using T = typename St::T;
    using raw = typename RawVec<N * sizeof(bits)>::type;
    union Pack {
        raw u;
        bits b[N];
    };
    __device__ static void load(const bits* p, T (&a)[N])
    {
        Pack x;
        x.u = *reinterpret_cast<const raw*>(p);
#pragma unroll
        for (int v = 0; v < N; ++v) a[v] = St::load(x.b[v]);
    }
    __device__ static void store(bits* p, const T (&a)[N])
    {
        Pack x;
#pragma unroll
        for (int v = 0; v < N; ++v) x.b[v] = St::store(a[v]);
        *reinterpret_cast<raw*>(p) = x.u;
    }
    // Storage-typed access: 16-bit populations stay packed in registers and
    // are converted one cell at a time, which halves their register footprint.
    __device__ static void load_raw(const bits* p, bits (&a)[N])
    {
        Pack x;
        x.u = *reinterpret_cast<const raw*>(p);
#pragma unroll
        for (int v = 0; v < N; ++v) a[v] = x.b[v];
    }
    __device__ static void store_raw(bits* p, const bits (&a)[N])
    {
        Pack x;
#pragma unroll
        for (int v = 0; v < N; ++v) x.b[v] = a[v];
        *reinterpret_cast<raw*>(p) = x.u;
    }
};

// Warp shuffles of storage elements (16-bit patterns travel in 32-bit lanes).
template <typename B>
__device__ __forceinline__ B shfl_up_bits(B v, int d)
{
    if constexpr (sizeof(B) == 2) return (B)__shfl_up_sync(0xffffffffu, (unsigned)v, d);
    else return __shfl_up_sync(0xffffffffu, v, d);
}
template <typename B>
__device__ __forceinline__ B shfl_down_bits(B v, int d)
{
    if constexpr (sizeof(B) == 2) return (B)__shfl_down_sync(0xffffffffu, (unsigned)v, d);
    else return __shfl_down_sync(0xffffffffu, v, d);
}

// Alpha step of the CPT cells owned by thread index t of one domain (t runs
// over groups x rows x planes: t = ((z-1) * ny + (y-1)) * G + group).
template <class St, int CPT>
__device__ __forceinline__ void alpha_cells(typename St::bits* __restrict__ dd, const Grid& g,
                                            const typename St::T inv_tau, const typename St::T lid_u,
                                            const int lid_y, const long long t)
{
    using T = typename St::T;
    using bits = typename St::bits;
    using IO = Vio<St, CPT>;
    const int G = (g.nx + CPT - 1) / CPT;
    const long long total = (long long)G * g.ny * g.nz;
    if (t >= total) return;
    const int gi = (int)(t % G);
    const long long row = t / G;
    const int y = 1 + (int)(row % g.ny);
    const int z = 1 + (int)(row / g.ny);
    const int x0 = 1 + gi * CPT;
    const long long base = g.idx(x0, y, z);

    bits f[Q][CPT];
#pragma unroll
    for (int k = 0; k < Q; ++k) IO::load_raw(dd + k * g.S + base, f[k]);

    const bool lid = (y == lid_y);
    const T rho0 = St::shifted ? T(0) : T(1);
#pragma unroll
    for (int v = 0; v < CPT; ++v) {
        if (x0 + v > g.nx) continue;  // halo/padding lane: slots stay as they are
        T c[Q];
#pragma unroll
        for (int k = 0; k < Q; ++k) c[k] = St::load(f[k][v]);
        if (lid) inject(c, rho0, lid_u);
        else collide<St>(c, inv_tau);
#pragma unroll
        for (int k = 0; k < Q; ++k) f[opp(k)][v] = St::store(c[k]);  // population k -> slot opp(k)
    }
#pragma unroll
    for (int k = 0; k < Q; ++k) IO::store_raw(dd + k * g.S + base, f[k]);
}

template <class St, int CPT, int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) alpha_fast(typename St::bits* __restrict__ dd, const Grid g,
                                                          const typename St::T inv_tau,
                                                          const typename St::T lid_u, const int lid_y)
{
    alpha_cells<St, CPT>(dd, g, inv_tau, lid_u, lid_y, (long long)blockIdx.x * BLOCK + threadIdx.x);
}

// Beta step of the CPT cells owned by thread index t of one domain.  All 32
// lanes of the warp must call it together, with consecutive t (they exchange
// edge elements by shuffles); lanes past the domain's end take part in the
// shuffles only.
template <class St, int CPT>
__device__ __forceinline__ void beta_cells(typename St::bits* __restrict__ dd, const Grid& g,
                                           const typename St::T inv_tau, const typename St::T lid_u,
                                           const int lid_y, const long long t)
{
    using T = typename St::T;
    using IO = Vio<St, CPT>;
    const int G = (g.nx + CPT - 1) / CPT;
    const long long total = (long long)G * g.ny * g.nz;
    const bool active = t < total;
    const int lane = threadIdx.x & 31;
    const long long tt = active ? t : 0;
    const int gi = (int)(tt % G);
    const long long row = tt / G;
    const int y = 1 + (int)(row % g.ny);
    const int z = 1 + (int)(row / g.ny);
    const int x0 = 1 + gi * CPT;
    // The neighbouring group of the same row is held by the adjacent lane.
    const bool left_in = gi > 0 && lane > 0;
    const bool right_in = gi < G - 1 && lane < 31;

    // p[k][v]: value of slot k at (cell x0+v) + c_k, i.e. population opp(k)
    // arriving at cell x0+v, kept in storage type.  edge[k]: the aligned
    // element of slot k that lies outside this thread's shifted window (kept to
    // rewrite it unchanged).
    using bits = typename St::bits;
    bits p[Q][CPT];
    bits edge[Q];

    static_for<0, Q>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        constexpr int cx = dir_x(k);
        const long long rb = k * g.S + g.idx(x0, y + dir_y(k), z + dir_z(k));
        bits a[CPT];
        if (active) IO::load_raw(dd + rb, a);
        else {
#pragma unroll
            for (int v = 0; v < CPT; ++v) a[v] = bits(0);
        }
        if constexpr (cx == 0) {
#pragma unroll
            for (int v = 0; v < CPT; ++v) p[k][v] = a[v];
            edge[k] = bits(0);
        } else if constexpr (cx == 1) {
            bits nb = shfl_down_bits(a[0], 1);
            if (active && !right_in) nb = dd[rb + CPT];
#pragma unroll
            for (int v = 0; v < CPT - 1; ++v) p[k][v] = a[v + 1];
            p[k][CPT - 1] = nb;
            edge[k] = a[0];
        } else {
            bits pb = shfl_up_bits(a[CPT - 1], 1);
            if (active && !left_in) pb = dd[rb - 1];
            p[k][0] = pb;
#pragma unroll
            for (int v = 1; v < CPT; ++v) p[k][v] = a[v - 1];
            edge[k] = a[CPT - 1];
        }
    });

    const bool lid = (y == lid_y);
    const T rho0 = St::shifted ? T(0) : T(1);
#pragma unroll
    for (int v = 0; v < CPT; ++v) {
        if (x0 + v > g.nx) continue;  // halo/padding lane: write back what was read
        T c[Q];
#pragma unroll
        for (int k = 0; k < Q; ++k) c[opp(k)] = St::load(p[k][v]);
        if (lid) inject(c, rho0, lid_u);
        else collide<St>(c, inv_tau);
#pragma unroll
        for (int k = 0; k < Q; ++k) p[k][v] = St::store(c[k]);  // population k -> slot k at x + c_k
    }

    static_for<0, Q>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        constexpr int cx = dir_x(k);
        const long long rb = k * g.S + g.idx(x0, y + dir_y(k), z + dir_z(k));
        if constexpr (cx == 0) {
            if (active) IO::store_raw(dd + rb, p[k]);
        } else if constexpr (cx == 1) {
            // aligned element 0 belongs to cell x0-1 (left lane's last cell)
            const bits from_left = shfl_up_bits(p[k][CPT - 1], 1);
            if (active) {
                bits o[CPT];
#pragma unroll
                for (int v = 1; v < CPT; ++v) o[v] = p[k][v - 1];
                if (left_in || gi == 0) {
                    o[0] = left_in ? from_left : edge[k];
                    IO::store_raw(dd + rb, o);
                } else {
#pragma unroll
                    for (int v = 1; v < CPT; ++v) dd[rb + v] = o[v];
                }
                if (!right_in && x0 + CPT - 1 <= g.nx) dd[rb + CPT] = p[k][CPT - 1];
            }
        } else {
            // aligned element CPT-1 belongs to cell x0+CPT (right lane's first cell)
            const bits from_right = shfl_down_bits(p[k][0], 1);
            if (active) {
                bits o[CPT];
#pragma unroll
                for (int v = 0; v < CPT - 1; ++v) o[v] = p[k][v + 1];
                if (right_in || gi == G - 1) {
                    o[CPT - 1] = right_in ? from_right : edge[k];
                    IO::store_raw(dd + rb, o);
                } else {
#pragma unroll
                    for (int v = 0; v < CPT - 1; ++v) dd[rb + v] = o[v];
                }
                if (!left_in) dd[rb - 1] = p[k][0];
            }
        }
    });
}

template <class St, int CPT, int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) beta_fast(typename St::bits* __restrict__ dd, const Grid g,
                                                         const typename St::T inv_tau,
                                                         const typename St::T lid_u, const int lid_y)
{
    beta_cells<St, CPT>(dd, g, inv_tau, lid_u, lid_y, (long long)blockIdx.x * BLOCK + threadIdx.x);
}

// Launch menu shared by every storage type: (cells per thread as a fraction
// of a 16-byte vector, block size, minimum blocks per SM).  Index = variant.
struct FastVariant {
    int cpt_div;   // cells per thread = (16 bytes / element) / cpt_div
    int block;
    int minb;
};
constexpr int kFastVariants = 8;
constexpr FastVariant kFastMenu[kFastVariants] = {
    {1, 256, 1},  // 16-byte vectors, registers unconstrained
    {1, 256, 2},  // 16-byte vectors, <= 128 registers
    {1, 128, 4},  // 16-byte vectors, <= 128 registers, smaller blocks
    {2, 256, 2},  // 8-byte vectors, <= 128 registers
    {2, 256, 3},  // 8-byte vectors, <= 85 registers
    {2, 128, 5},  // 8-byte vectors, <= 102 registers
    {4, 256, 2},  // 4-byte vectors (FP64: one cell), <= 128 registers
    {4, 256, 3},  // 4-byte vectors (FP64: one cell), <= 85 registers
};

template <class St, int VARIANT>
cudaError_t launch_fast_variant(bool alpha, void* dd, const Grid& g, const Params& p, int lid_y, cudaStream_t st)
{
    using T = typename St::T;
    constexpr FastVariant fv = kFastMenu[VARIANT];
    constexpr int CPT = (16 / (int)sizeof(typename St::bits)) / fv.cpt_div > 0
                            ? (16 / (int)sizeof(typename St::bits)) / fv.cpt_div : 1;
    const int G = (g.nx + CPT - 1) / CPT;
    const long long threads = (long long)G * g.ny * g.nz;
    const int blocks = (int)((threads + fv.block - 1) / fv.block);
    auto* d = static_cast<typename St::bits*>(dd);
    if (alpha) alpha_fast<St, CPT, fv.block, fv.minb><<<blocks, fv.block, 0, st>>>(d, g, T(p.inv_tau), T(p.lid_u), lid_y);
    else beta_fast<St, CPT, fv.block, fv.minb><<<blocks, fv.block, 0, st>>>(d, g, T(p.inv_tau), T(p.lid_u), lid_y);
    return cudaGetLastError();
}

template <class St>
cudaError_t launch_fast_menu(int variant, bool alpha, void* dd, const Grid& g, const Params& p, int lid_y,
                             cudaStream_t st)
{
    switch (variant) {
    case 0: return launch_fast_variant<St, 0>(alpha, dd, g, p, lid_y, st);
    case 1: return launch_fast_variant<St, 1>(alpha, dd, g, p, lid_y, st);
    case 2: return launch_fast_variant<St, 2>(alpha, dd, g, p, lid_y, st);
    case 3: return launch_fast_variant<St, 3>(alpha, dd, g, p, lid_y, st);
    case 4: return launch_fast_variant<St, 4>(alpha, dd, g, p, lid_y, st);
    case 5: return launch_fast_variant<St, 5>(alpha, dd, g, p, lid_y, st);
    case 6: return launch_fast_variant<St, 6>(alpha, dd, g, p, lid_y, st);
    case 7: return launch_fast_variant<St, 7>(alpha, dd, g, p, lid_y, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace lbm

namespace lbm {

// ---------------------------------------------------------------------------
// Batches: many box cavities advanced by one launch.  The domains' padded
// population arrays share one device pool; a packed table gives each its
// layout, offset, parameters and its range of "virtual blocks" (BLOCK
// threads x CPT cells each, numbered consecutively over the domains).  A
// persistent grid walks the virtual blocks; every CTA finds its domain by
// binary search and runs the same per-thread bodies as the single-domain
// kernels, so a domain's result does not depend on its neighbours in the
// batch.
// ---------------------------------------------------------------------------
struct BatchDomain {
    Grid g;
    long long offset;       // elements from the pool base
    double inv_tau;
    double lid_u;
    int lid_y;
    long long block_start;  // first virtual block of this domain
};

template <class St, int CPT, int BLOCK, int MINB, bool kAlpha>
__global__ void __launch_bounds__(BLOCK, MINB) batch_step(typename St::bits* __restrict__ pool,
                                                          const BatchDomain* __restrict__ doms, const int ndom,
                                                          const long long vblocks)
{
    using T = typename St::T;
    for (long long vb = blockIdx.x; vb < vblocks; vb += gridDim.x) {
        int lo = 0, hi = ndom - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (doms[mid].block_start <= vb) lo = mid;
            else hi = mid - 1;
        }
        const BatchDomain d = doms[lo];
        const long long t = (vb - d.block_start) * BLOCK + threadIdx.x;
        if constexpr (kAlpha) alpha_cells<St, CPT>(pool + d.offset, d.g, T(d.inv_tau), T(d.lid_u), d.lid_y, t);
        else beta_cells<St, CPT>(pool + d.offset, d.g, T(d.inv_tau), T(d.lid_u), d.lid_y, t);
    }
}

template <class St, int VARIANT>
cudaError_t launch_batch_variant(bool alpha, void* pool, const BatchDomain* doms, int ndom, long long vblocks,
                                 cudaStream_t st)
{
    constexpr FastVariant fv = kFastMenu[VARIANT];
    constexpr int CPT = (16 / (int)sizeof(typename St::bits)) / fv.cpt_div > 0
                            ? (16 / (int)sizeof(typename St::bits)) / fv.cpt_div : 1;
    auto kern = alpha ? batch_step<St, CPT, fv.block, fv.minb, true> : batch_step<St, CPT, fv.block, fv.minb, false>;
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, fv.block, 0);
    if (e != cudaSuccess) return e;
    long long grid = (long long)(per_sm > 0 ? per_sm : 1) * sms;
    if (grid > vblocks) grid = vblocks;
    if (grid < 1) return cudaSuccess;
    kern<<<(int)grid, fv.block, 0, st>>>(static_cast<typename St::bits*>(pool), doms, ndom, vblocks);
    return cudaGetLastError();
}

template <class St>
cudaError_t launch_batch_menu(int variant, bool alpha, void* pool, const BatchDomain* doms, int ndom,
                              long long vblocks, cudaStream_t st)
{
    switch (variant) {
    case 0: return launch_batch_variant<St, 0>(alpha, pool, doms, ndom, vblocks, st);
    case 1: return launch_batch_variant<St, 1>(alpha, pool, doms, ndom, vblocks, st);
    case 2: return launch_batch_variant<St, 2>(alpha, pool, doms, ndom, vblocks, st);
    case 3: return launch_batch_variant<St, 3>(alpha, pool, doms, ndom, vblocks, st);
    case 4: return launch_batch_variant<St, 4>(alpha, pool, doms, ndom, vblocks, st);
    case 5: return launch_batch_variant<St, 5>(alpha, pool, doms, ndom, vblocks, st);
    case 6: return launch_batch_variant<St, 6>(alpha, pool, doms, ndom, vblocks, st);
    case 7: return launch_batch_variant<St, 7>(alpha, pool, doms, ndom, vblocks, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace lbm
