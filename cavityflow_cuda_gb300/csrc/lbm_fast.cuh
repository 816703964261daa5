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
//   beta_fast_blk -- the same step with the exchange widened to the whole
//                  block (shuffles inside a warp, shared memory between
//                  warps), so that only the block's two end lanes and row
//                  edges use scalar accesses.
//   beta_fast_direct -- the same step with no exchange at all: each thread
//                  reads and writes its own one-cell-shifted windows with
//                  element-aligned pieces (the default for FP32).
//   beta_fast_pk -- the direct windows for 16-bit storage with two cells'
//                  populations packed per 32-bit word and paired conversions
//                  (the default for the 16-bit storages).
//   batch_step  -- the persistent kernel of a batch of cavities, running the
//                  same per-thread bodies over a packed domain table.
//
// Template parameters: St storage type, CPT cells per thread (one vector of
// CPT elements per slot: 16, 8 or 4 bytes), BLOCK threads per block, MINB the
// minimum resident blocks per SM requested from the register allocator.  The
// launch menu (kFastMenu, lbm_kernels.h) picks them per kernel.
#pragma once

#include <cstdint>
#include <type_traits>
#include <utility>

#include "lbm_core.cuh"
#include "lbm_kernels.h"

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

// The group of CPT cells a thread owns: group gi of row y of plane z.  An
// inactive thread (past the end) carries a valid group (it reads, never
// writes).
struct Cells {
    int gi, y, z;
    bool active;
};

// From an index i over the G * ny groups of plane z (the step kernels' grid:
// x over a plane's groups, y over planes); divG divides by G.
__host__ __device__ __forceinline__ Cells cells_of_plane(const Grid& g, int G, const FastDiv& divG, uint32_t i,
                                                     int z)
{
    Cells c;
    c.active = i < (uint32_t)G * (uint32_t)g.ny;
    const uint32_t ii = c.active ? i : 0u;
    const uint32_t row = divG.div(ii);
    c.gi = (int)(ii - row * (uint32_t)G);
    c.y = 1 + (int)row;
    c.z = z;
    return c;
}

// Alpha step of the CPT cells of group `c`.
template <class St, int CPT>
__device__ __forceinline__ void alpha_cells(typename St::bits* __restrict__ dd, const Grid& g,
                                            const typename St::T inv_tau, const typename St::T lid_u,
                                            const int lid_y, const int wall_y, const Cells c,
                                            const uint32_t step)
{
    using T = typename St::T;
    using bits = typename St::bits;
    using IO = Vio<St, CPT>;
    if (!c.active) return;
    const int gi = c.gi, y = c.y, z = c.z;
    const int x0 = 1 + gi * CPT;
    const long long base = g.idx(x0, y, z);

    bits f[Q][CPT];
#pragma unroll
    for (int k = 0; k < Q; ++k) IO::load_raw(dd + k * g.S + base, f[k]);

    const bool lid = (y == lid_y);
    const bool wall = (y == wall_y);
    const T du = wall_shift<St>(lid_u);
    const T rho0 = St::shifted ? T(0) : T(1);
    const uint32_t row_hash = St::stochastic ? sr_hash((uint32_t)g.ref(0, y, z), step) : 0u;
#pragma unroll
    for (int v = 0; v < CPT; ++v) {
        if (x0 + v > g.nx) continue;  // halo/padding lane: slots stay as they are
        T c[Q];
#pragma unroll
        for (int k = 0; k < Q; ++k) c[k] = St::load_step(f[k][v]);
        if (wall) wall_correct(c, du);
        if (lid) inject_step<St>(c, rho0, lid_u);
        else collide<St>(c, inv_tau);
        uint32_t h = 0;
        if constexpr (St::stochastic) h = sr_cell(row_hash, x0 + v);
#pragma unroll
        for (int k = 0; k < Q; ++k) f[opp(k)][v] = store_pop<St>(c[k], h, k);  // population k -> slot opp(k)
    }
#pragma unroll
    for (int k = 0; k < Q; ++k) IO::store_raw(dd + k * g.S + base, f[k]);
}

template <class St, int CPT, int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) alpha_fast(typename St::bits* __restrict__ dd, const Grid g,
                                                          const typename St::T inv_tau,
                                                          const typename St::T lid_u, const int lid_y,
                                                          const int wall_y,
                                                          const uint32_t* __restrict__ step_base,
                                                          const uint32_t step_off, const FastDiv divG,
                                                          const int z_base)
{
    const int G = (g.nx + CPT - 1) / CPT;
    alpha_cells<St, CPT>(dd, g, inv_tau, lid_u, lid_y, wall_y,
                         cells_of_plane(g, G, divG, blockIdx.x * BLOCK + threadIdx.x, z_base + (int)blockIdx.y + 1),
                         step_of<St>(step_base, step_off));
}

// Beta step of the CPT cells of group `c`.  All 32 lanes of the warp must
// call it together, with consecutive groups (they exchange edge elements by
// shuffles); lanes past the domain's end take part in the shuffles only.
template <class St, int CPT>
__device__ __forceinline__ void beta_cells(typename St::bits* __restrict__ dd, const Grid& g,
                                           const typename St::T inv_tau, const typename St::T lid_u,
                                           const int lid_y, const int wall_y, const Cells c,
                                           const uint32_t step)
{
    using T = typename St::T;
    using IO = Vio<St, CPT>;
    const int G = (g.nx + CPT - 1) / CPT;
    const bool active = c.active;
    const int lane = threadIdx.x & 31;
    const int gi = c.gi, y = c.y, z = c.z;
    const int x0 = 1 + gi * CPT;
    const long long base = g.idx(x0, y, z);
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
        const long long rb = base + (k * g.S + dir_z(k) * g.PY + dir_y(k) * g.P);  // slot offset: uniform
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
    const bool wall = (y == wall_y);
    const T du = wall_shift<St>(lid_u);
    const T rho0 = St::shifted ? T(0) : T(1);
    const uint32_t row_hash = St::stochastic ? sr_hash((uint32_t)g.ref(0, y, z), step) : 0u;
#pragma unroll
    for (int v = 0; v < CPT; ++v) {
        if (x0 + v > g.nx) continue;  // halo/padding lane: write back what was read
        T c[Q];
#pragma unroll
        for (int k = 0; k < Q; ++k) c[opp(k)] = St::load_step(p[k][v]);
        if (wall) wall_correct(c, du);
        if (lid) inject_step<St>(c, rho0, lid_u);
        else collide<St>(c, inv_tau);
        uint32_t h = 0;
        if constexpr (St::stochastic) h = sr_cell(row_hash, x0 + v);
#pragma unroll
        for (int k = 0; k < Q; ++k) p[k][v] = store_pop<St>(c[k], h, k);  // population k -> slot k at x + c_k
    }

    static_for<0, Q>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        constexpr int cx = dir_x(k);
        const long long rb = base + (k * g.S + dir_z(k) * g.PY + dir_y(k) * g.P);  // slot offset: uniform
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

// Element-aligned access to a window of CPT storage elements starting `S`
// elements (+1 or -1) off an aligned CPT-element vector: the window is split
// into the widest naturally aligned pieces (at most 16 bytes), e.g. for
// 16-bit elements and CPT 4 at +1: one 2-byte, one 4-byte and one 2-byte
// access.  Compile-time recursion over the pieces.
template <class St, int CPT, int S, int E>
struct Window {
    using bits = typename St::bits;
    static constexpr int kEnd = S + CPT;
    static constexpr int width()
    {
        int w = 1;
        while (2 * w * (int)sizeof(bits) <= 16 && E % (2 * w) == 0 && E + 2 * w <= kEnd) w *= 2;
        return w;
    }
    static constexpr int W = width();
    using raw = typename RawVec<W * sizeof(bits)>::type;
    union Piece {
        raw u;
        bits b[W];
    };
    __device__ static void load(const bits* v, bits (&out)[CPT])
    {
        Piece x;
        x.u = *reinterpret_cast<const raw*>(v + E);
#pragma unroll
        for (int i = 0; i < W; ++i) out[E - S + i] = x.b[i];
        if constexpr (E + W < kEnd) Window<St, CPT, S, E + W>::load(v, out);
    }
    __device__ static void store(bits* v, const bits (&in)[CPT])
    {
        Piece x;
#pragma unroll
        for (int i = 0; i < W; ++i) x.b[i] = in[E - S + i];
        *reinterpret_cast<raw*>(v + E) = x.u;
        if constexpr (E + W < kEnd) Window<St, CPT, S, E + W>::store(v, in);
    }
};

// Beta step of the CPT cells of group `c` without any exchange between
// threads: every slot is read and written at the cells' own pull addresses,
// the c_x = +-1 slots through element-aligned windows (Window).  Each slot
// element is touched by exactly one thread, as in the exchanging bodies; the
// halo and padding columns of a row are part of the windows of its end
// groups, so rows need no special case.
template <class St, int CPT>
__device__ __forceinline__ void beta_cells_direct(typename St::bits* __restrict__ dd, const Grid& g,
                                                  const typename St::T inv_tau, const typename St::T lid_u,
                                                  const int lid_y, const int wall_y, const Cells c,
                                                  const uint32_t step)
{
    using T = typename St::T;
    using bits = typename St::bits;
    using IO = Vio<St, CPT>;
    if (!c.active) return;
    const int gi = c.gi, y = c.y, z = c.z;
    const int x0 = 1 + gi * CPT;
    const long long base = g.idx(x0, y, z);

    // p[k][v]: value of slot k at (cell x0+v) + c_k
    bits p[Q][CPT];
    static_for<0, Q>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        constexpr int cx = dir_x(k);
        const long long rb = base + (k * g.S + dir_z(k) * g.PY + dir_y(k) * g.P);  // slot offset: uniform
        if constexpr (cx == 0) IO::load_raw(dd + rb, p[k]);
        else Window<St, CPT, cx, cx>::load(dd + rb, p[k]);
    });

    const bool lid = (y == lid_y);
    const bool wall = (y == wall_y);
    const T du = wall_shift<St>(lid_u);
    const T rho0 = St::shifted ? T(0) : T(1);
    const uint32_t row_hash = St::stochastic ? sr_hash((uint32_t)g.ref(0, y, z), step) : 0u;
#pragma unroll
    for (int v = 0; v < CPT; ++v) {
        if (x0 + v > g.nx) continue;  // halo/padding lane: write back what was read
        T cc[Q];
#pragma unroll
        for (int k = 0; k < Q; ++k) cc[opp(k)] = St::load_step(p[k][v]);
        if (wall) wall_correct(cc, du);
        if (lid) inject_step<St>(cc, rho0, lid_u);
        else collide<St>(cc, inv_tau);
        uint32_t h = 0;
        if constexpr (St::stochastic) h = sr_cell(row_hash, x0 + v);
#pragma unroll
        for (int k = 0; k < Q; ++k) p[k][v] = store_pop<St>(cc[k], h, k);  // population k -> slot k at x + c_k
    }

    static_for<0, Q>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        constexpr int cx = dir_x(k);
        const long long rb = base + (k * g.S + dir_z(k) * g.PY + dir_y(k) * g.P);  // slot offset: uniform
        if constexpr (cx == 0) IO::store_raw(dd + rb, p[k]);
        else Window<St, CPT, cx, cx>::store(dd + rb, p[k]);
    });
}

// ---------------------------------------------------------------------------
// Beta step for 16-bit storage with two cells' populations per 32-bit word.
//
// The direct windows above keep each 16-bit population in a register of its
// own, convert it on its own and assemble the vectors element by element.
// Here a slot's CPT cells stay packed as the words that the slot's memory
// pieces load and store -- for a slot with c_x = 0 the pairs (0,1), (2,3) of
// its aligned vector, for c_x = +-1 the window's single first cell, its
// 4-byte pairs (1,2), ... and its single last cell (PkSlot) -- so no element
// is moved between registers: inputs are half selections of the words, and
// each pair of results is rounded and packed by one paired conversion
// (cvt.rz.f16x2.f32 after the stochastic-rounding dither, cvt.rn.f16x2 /
// cvt.rn.bf16x2 otherwise).  A cell's first result of a pair waits as a float
// (`pend`) until its partner is collided.  The results are bit-identical to
// the per-cell conversions (the same roundings), with half the registers for
// the populations (96 registers at 4 cells per thread against 128) and fewer
// instructions.
//
// Loads (kVecLoads): the window's pieces (2-, 4- and 2-byte accesses for 4
// cells), or the aligned vector that holds all but one of the window's
// elements plus that one element (2 accesses; the extra bytes come from the
// same L1 sectors).  Stores always use the window's pieces, since the aligned
// vector's other element belongs to the neighbouring group.  In a row's last
// group, cells past the row's end skip the collision and store back exactly
// what they read, so partial groups run the same code.
// ---------------------------------------------------------------------------
constexpr int kPkMaxWords = 5;

// Where cell v's 16-bit value sits in the packed words of a slot with shift S
// (its stored form: the window's pieces).
template <int CPT, int S>
struct PkSlot {
    __host__ __device__ static constexpr int word(int v) { return S == 0 ? v >> 1 : (v == 0 ? 0 : (v + 1) >> 1); }
    __host__ __device__ static constexpr int half(int v) { return S == 0 ? (v & 1) : (v == 0 ? 0 : ((v + 1) & 1)); }
    // a 2-byte piece: converted alone
    __host__ __device__ static constexpr bool single(int v) { return S != 0 && (v == 0 || v == CPT - 1); }
    // the first cell of a 4-byte pair: waits for its partner
    __host__ __device__ static constexpr bool first(int v) { return !single(v) && half(v) == 0; }
    // with vector loads, where cell v's value sits as loaded
    __host__ __device__ static constexpr int in_word(int v, bool vec)
    {
        return !vec || S == 0 ? word(v) : S > 0 ? (v == CPT - 1 ? CPT / 2 : (v + 1) >> 1) : (v == 0 ? 0 : 1 + ((v - 1) >> 1));
    }
    __host__ __device__ static constexpr int in_half(int v, bool vec)
    {
        return !vec || S == 0 ? half(v) : S > 0 ? (v == CPT - 1 ? 0 : (v + 1) & 1) : (v == 0 ? 0 : (v - 1) & 1);
    }
};

// The window [S, S + CPT) of a slot (elements relative to the cells' aligned
// vector) as its widest naturally aligned pieces, each moved whole into or out
// of the packed words.
template <int CPT, int S, int E>
struct PkPiece {
    static constexpr int kEnd = S + CPT;
    static constexpr int width()
    {
        int w = 1;
        while (2 * w * 2 <= 16 && E % (2 * w) == 0 && E + 2 * w <= kEnd) w *= 2;
        return w;
    }
    static constexpr int W = width();
    static constexpr int w0 = PkSlot<CPT, S>::word(E - S);
    __device__ static void load(const unsigned short* p, uint32_t (&w)[kPkMaxWords])
    {
        if constexpr (W == 1) w[w0] = (uint32_t)p[E];
        else if constexpr (W == 2) w[w0] = *reinterpret_cast<const uint32_t*>(p + E);
        else if constexpr (W == 4) {
            const uint2 t = *reinterpret_cast<const uint2*>(p + E);
            w[w0] = t.x; w[w0 + 1] = t.y;
        } else {
            const uint4 t = *reinterpret_cast<const uint4*>(p + E);
            w[w0] = t.x; w[w0 + 1] = t.y; w[w0 + 2] = t.z; w[w0 + 3] = t.w;
        }
        if constexpr (E + W < kEnd) PkPiece<CPT, S, E + W>::load(p, w);
    }
    __device__ static void store(unsigned short* p, const uint32_t (&w)[kPkMaxWords])
    {
        if constexpr (W == 1) p[E] = (unsigned short)w[w0];
        else if constexpr (W == 2) *reinterpret_cast<uint32_t*>(p + E) = w[w0];
        else if constexpr (W == 4) *reinterpret_cast<uint2*>(p + E) = make_uint2(w[w0], w[w0 + 1]);
        else *reinterpret_cast<uint4*>(p + E) = make_uint4(w[w0], w[w0 + 1], w[w0 + 2], w[w0 + 3]);
        if constexpr (E + W < kEnd) PkPiece<CPT, S, E + W>::store(p, w);
    }
};

// Loads of a slot with shift S: the pieces, or (kVec, S != 0) the aligned
// vector (words 0.. for S > 0, 1.. for S < 0) and the one element outside it
// (word CPT/2 for S > 0, word 0 for S < 0), as PkSlot::in_word describes.
template <int CPT, int S, bool kVec>
__device__ __forceinline__ void pk_load(const unsigned short* p, uint32_t (&w)[kPkMaxWords])
{
    if constexpr (S == 0 || !kVec) {
        PkPiece<CPT, S, S>::load(p, w);
    } else {
        constexpr int o = S > 0 ? 0 : 1;
        if constexpr (CPT == 4) {
            const uint2 t = *reinterpret_cast<const uint2*>(p);
            w[o] = t.x; w[o + 1] = t.y;
        } else {
            const uint4 t = *reinterpret_cast<const uint4*>(p);
            w[o] = t.x; w[o + 1] = t.y; w[o + 2] = t.z; w[o + 3] = t.w;
        }
        if constexpr (S > 0) w[CPT / 2] = (uint32_t)p[CPT];
        else w[0] = (uint32_t)p[-1];
    }
}

// A 16-bit pattern (low or high half of a word) in the step's arithmetic type.
template <class St>
__device__ __forceinline__ float pk_in(uint32_t w, int hi)
{
    if constexpr (std::is_same<St, BF16S>::value) return __uint_as_float(hi ? (w & 0xffff0000u) : (w << 16));
    else return __half2float(__ushort_as_half((unsigned short)(hi ? (w >> 16) : (w & 0xffffu))));
}

// A step result as the float its store converts: for stochastic rounding
// with the population's dither added below the bits half precision drops
// (store_sr), otherwise unchanged.
template <class St>
__device__ __forceinline__ float pk_pre(float v, uint32_t h, int k)
{
    if constexpr (St::stochastic) return __uint_as_float(__float_as_uint(v) + sr_dither(h, k));
    else return v;
}
// Such floats rounded to 16-bit patterns: one alone (low half), or two packed
// (lo, hi) by one paired conversion with the same rounding as the single one.
// A 16-bit value read as a float and not dithered comes back exactly.
template <class St>
__device__ __forceinline__ uint32_t pk_one(float d)
{
    if constexpr (St::stochastic) return (uint32_t)__half_as_ushort(__float2half_rz(d));
    else return (uint32_t)St::store(d);
}
template <class St>
__device__ __forceinline__ uint32_t pk_two(float lo, float hi)
{
    uint32_t r;
    if constexpr (St::stochastic) asm("cvt.rz.f16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    else if constexpr (std::is_same<St, BF16S>::value) asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    else asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

template <class St, int CPT, bool kVec>
__device__ __forceinline__ void beta_cells_pk(typename St::bits* __restrict__ dd, const Grid& g,
                                              const typename St::T inv_tau, const typename St::T lid_u,
                                              const int lid_y, const int wall_y, const Cells c,
                                              const uint32_t step)
{
    static_assert(sizeof(typename St::bits) == 2, "16-bit storage only");
    if (!c.active) return;
    const int gi = c.gi, y = c.y, z = c.z;
    const int x0 = 1 + gi * CPT;
    const int nvalid = g.nx - x0 + 1;  // cells of the group inside the row (a row's last group may be partial)
    const long long base = g.idx(x0, y, z);
    uint32_t w[Q][kPkMaxWords];
    static_for<0, Q>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        const long long rb = base + (k * g.S + dir_z(k) * g.PY + dir_y(k) * g.P);  // slot offset: uniform
        pk_load<CPT, dir_x(k), kVec>(dd + rb, w[k]);
    });
    const bool lid = (y == lid_y);
    const bool wall = (y == wall_y);
    const float du = wall_shift<St>(lid_u);
    const uint32_t row_hash = St::stochastic ? sr_hash((uint32_t)g.ref(0, y, z), step) : 0u;
    float pend[Q];
    static_for<0, CPT>([&](auto vc) {
        constexpr int v = decltype(vc)::value;
        const bool valid = v < nvalid;
        float cc[Q];
        static_for<0, Q>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            using P = PkSlot<CPT, dir_x(k)>;
            cc[opp(k)] = pk_in<St>(w[k][P::in_word(v, kVec)], P::in_half(v, kVec));
        });
        if (valid) {
            if (wall) wall_correct(cc, du);
            if (lid) inject_step<St>(cc, 0.0f, lid_u);
            else collide<St>(cc, inv_tau);
        } else {  // a cell past the row's end: every slot gets back the value read from it
#pragma unroll
            for (int k = 0; k < Q - 1; k += 2) {
                const float t = cc[k];
                cc[k] = cc[k + 1];
                cc[k + 1] = t;
            }
        }
        uint32_t h = 0;
        if constexpr (St::stochastic) h = sr_cell(row_hash, x0 + v);
        static_for<0, Q>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            using P = PkSlot<CPT, dir_x(k)>;
            const float d = valid ? pk_pre<St>(cc[k], h, k) : cc[k];
            if constexpr (P::single(v)) w[k][P::word(v)] = pk_one<St>(d);
            else if constexpr (P::first(v)) pend[k] = d;
            else w[k][P::word(v)] = pk_two<St>(pend[k], d);
        });
    });
    static_for<0, Q>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        constexpr int cx = dir_x(k);
        const long long rb = base + (k * g.S + dir_z(k) * g.PY + dir_y(k) * g.P);  // slot offset: uniform
        PkPiece<CPT, cx, cx>::store(dd + rb, w[k]);
    });
}

template <class St, int CPT, int BLOCK, int MINB, bool kVec>
__global__ void __launch_bounds__(BLOCK, MINB) beta_fast_pk(typename St::bits* __restrict__ dd, const Grid g,
                                                            const typename St::T inv_tau,
                                                            const typename St::T lid_u, const int lid_y,
                                                            const int wall_y,
                                                            const uint32_t* __restrict__ step_base,
                                                            const uint32_t step_off, const FastDiv divG,
                                                            const int z_base)
{
    const int G = (g.nx + CPT - 1) / CPT;
    beta_cells_pk<St, CPT, kVec>(dd, g, inv_tau, lid_u, lid_y, wall_y,
                                 cells_of_plane(g, G, divG, blockIdx.x * BLOCK + threadIdx.x, z_base + (int)blockIdx.y + 1),
                                 step_of<St>(step_base, step_off));
}

template <class St, int CPT, int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) beta_fast_direct(typename St::bits* __restrict__ dd, const Grid g,
                                                                const typename St::T inv_tau,
                                                                const typename St::T lid_u, const int lid_y,
                                                                const int wall_y,
                                                                const uint32_t* __restrict__ step_base,
                                                                const uint32_t step_off, const FastDiv divG,
                                                                const int z_base)
{
    const int G = (g.nx + CPT - 1) / CPT;
    beta_cells_direct<St, CPT>(dd, g, inv_tau, lid_u, lid_y, wall_y,
                               cells_of_plane(g, G, divG, blockIdx.x * BLOCK + threadIdx.x, z_base + (int)blockIdx.y + 1),
                               step_of<St>(step_base, step_off));
}

// Beta step with the neighbour exchange done block-wide: inside a warp by
// shuffles, across the warps of a block through shared memory (two block
// barriers), so only lanes at a row edge or at the block's two ends touch the
// odd element with a scalar access; every other thread issues exactly 19
// vector loads and 19 vector stores, as in alpha.  All BLOCK threads of the
// block must call it together, with consecutive groups.
template <class St, int CPT, int BLOCK>
__device__ __forceinline__ void beta_cells_blk(typename St::bits* __restrict__ dd, const Grid& g,
                                               const typename St::T inv_tau, const typename St::T lid_u,
                                               const int lid_y, const int wall_y, const Cells c,
                                               const uint32_t step)
{
    using T = typename St::T;
    using bits = typename St::bits;
    using IO = Vio<St, CPT>;
    constexpr int W = BLOCK / 32;
    // [warp][k >> 1] for the ten slots k < 12 with c_x != 0: the first and last
    // element of a warp's vectors before the collision (s_first, s_last) and
    // after it (s_head, s_tail).
    __shared__ bits s_first[W][6], s_last[W][6], s_head[W][6], s_tail[W][6];
    const int G = (g.nx + CPT - 1) / CPT;
    const bool active = c.active;  // inactive lanes read a valid cell, never write
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int gi = c.gi, y = c.y, z = c.z;
    const int x0 = 1 + gi * CPT;
    const long long base = g.idx(x0, y, z);
    // The neighbouring group of the same row belongs to thread t -+ 1 of this block.
    const bool left_in = gi > 0 && threadIdx.x > 0;
    const bool right_in = gi < G - 1 && threadIdx.x < BLOCK - 1;

    bits a[Q][CPT];
    bits ext[Q];  // the odd element fetched by a scalar load at a block or row edge
    static_for<0, Q>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        constexpr int cx = dir_x(k);
        const long long rb = base + (k * g.S + dir_z(k) * g.PY + dir_y(k) * g.P);  // slot offset: uniform
        IO::load_raw(dd + rb, a[k]);
        ext[k] = bits(0);
        if constexpr (cx == 1) {
            if (active && !right_in) ext[k] = dd[rb + CPT];
        } else if constexpr (cx == -1) {
            if (active && !left_in) ext[k] = dd[rb - 1];
        }
    });
    // warp-edge lanes publish the elements the neighbouring warps need
    static_for<0, 12>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        if constexpr (dir_x(k) == 1) {
            if (lane == 0) s_first[warp][k >> 1] = a[k][0];
        } else if constexpr (dir_x(k) == -1) {
            if (lane == 31) s_last[warp][k >> 1] = a[k][CPT - 1];
        }
    });
    __syncthreads();

    // p[k][v]: value of slot k at (cell x0+v) + c_k; edge[k]: the aligned
    // element outside the shifted window, rewritten unchanged at a row edge.
    bits p[Q][CPT];
    bits edge[Q];
    static_for<0, Q>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        constexpr int cx = dir_x(k);
        if constexpr (cx == 0) {
#pragma unroll
            for (int v = 0; v < CPT; ++v) p[k][v] = a[k][v];
            edge[k] = bits(0);
        } else if constexpr (cx == 1) {
            bits nb = shfl_down_bits(a[k][0], 1);
            if (lane == 31 && warp < W - 1) nb = s_first[warp + 1][k >> 1];
            if (!right_in) nb = ext[k];
#pragma unroll
            for (int v = 0; v < CPT - 1; ++v) p[k][v] = a[k][v + 1];
            p[k][CPT - 1] = nb;
            edge[k] = a[k][0];
        } else {
            bits pb = shfl_up_bits(a[k][CPT - 1], 1);
            if (lane == 0 && warp > 0) pb = s_last[warp - 1][k >> 1];
            if (!left_in) pb = ext[k];
            p[k][0] = pb;
#pragma unroll
            for (int v = 1; v < CPT; ++v) p[k][v] = a[k][v - 1];
            edge[k] = a[k][CPT - 1];
        }
    });

    const bool lid = (y == lid_y);
    const bool wall = (y == wall_y);
    const T du = wall_shift<St>(lid_u);
    const T rho0 = St::shifted ? T(0) : T(1);
    const uint32_t row_hash = St::stochastic ? sr_hash((uint32_t)g.ref(0, y, z), step) : 0u;
#pragma unroll
    for (int v = 0; v < CPT; ++v) {
        if (x0 + v > g.nx) continue;  // halo/padding lane: write back what was read
        T c[Q];
#pragma unroll
        for (int k = 0; k < Q; ++k) c[opp(k)] = St::load_step(p[k][v]);
        if (wall) wall_correct(c, du);
        if (lid) inject_step<St>(c, rho0, lid_u);
        else collide<St>(c, inv_tau);
        uint32_t h = 0;
        if constexpr (St::stochastic) h = sr_cell(row_hash, x0 + v);
#pragma unroll
        for (int k = 0; k < Q; ++k) p[k][v] = store_pop<St>(c[k], h, k);  // population k -> slot k at x + c_k
    }

    static_for<0, 12>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        if constexpr (dir_x(k) == 1) {
            if (lane == 31) s_tail[warp][k >> 1] = p[k][CPT - 1];
        } else if constexpr (dir_x(k) == -1) {
            if (lane == 0) s_head[warp][k >> 1] = p[k][0];
        }
    });
    __syncthreads();

    static_for<0, Q>([&](auto kc) {
        constexpr int k = decltype(kc)::value;
        constexpr int cx = dir_x(k);
        const long long rb = base + (k * g.S + dir_z(k) * g.PY + dir_y(k) * g.P);  // slot offset: uniform
        if constexpr (cx == 0) {
            if (active) IO::store_raw(dd + rb, p[k]);
        } else if constexpr (cx == 1) {
            // aligned element 0 belongs to cell x0-1 (thread t-1)
            bits from_left = shfl_up_bits(p[k][CPT - 1], 1);
            if (lane == 0 && warp > 0) from_left = s_tail[warp - 1][k >> 1];
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
            // aligned element CPT-1 belongs to cell x0+CPT (thread t+1)
            bits from_right = shfl_down_bits(p[k][0], 1);
            if (lane == 31 && warp < W - 1) from_right = s_head[warp + 1][k >> 1];
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
__global__ void __launch_bounds__(BLOCK, MINB) beta_fast_blk(typename St::bits* __restrict__ dd, const Grid g,
                                                             const typename St::T inv_tau,
                                                             const typename St::T lid_u, const int lid_y,
                                                             const int wall_y,
                                                             const uint32_t* __restrict__ step_base,
                                                             const uint32_t step_off, const FastDiv divG,
                                                             const int z_base)
{
    const int G = (g.nx + CPT - 1) / CPT;
    beta_cells_blk<St, CPT, BLOCK>(
        dd, g, inv_tau, lid_u, lid_y, wall_y,
        cells_of_plane(g, G, divG, blockIdx.x * BLOCK + threadIdx.x, z_base + (int)blockIdx.y + 1),
        step_of<St>(step_base, step_off));
}

template <class St, int CPT, int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) beta_fast(typename St::bits* __restrict__ dd, const Grid g,
                                                         const typename St::T inv_tau,
                                                         const typename St::T lid_u, const int lid_y,
                                                         const int wall_y,
                                                         const uint32_t* __restrict__ step_base,
                                                         const uint32_t step_off, const FastDiv divG,
                                                         const int z_base)
{
    const int G = (g.nx + CPT - 1) / CPT;
    beta_cells<St, CPT>(dd, g, inv_tau, lid_u, lid_y, wall_y,
                        cells_of_plane(g, G, divG, blockIdx.x * BLOCK + threadIdx.x, z_base + (int)blockIdx.y + 1),
                        step_of<St>(step_base, step_off));
}

// Cells per thread of a kernel shape for storage St (at least one).
template <class St>
constexpr int shape_cpt(const KernelShape& k)
{
    return (16 / (int)sizeof(typename St::bits)) / k.cpt_div > 0 ? (16 / (int)sizeof(typename St::bits)) / k.cpt_div
                                                                  : 1;
}

template <class St, int VARIANT>
cudaError_t launch_fast_variant(bool alpha, void* dd, const Grid& g, const Params& p, int lid_y, cudaStream_t st)
{
    using T = typename St::T;
    constexpr FastVariant fv = kFastMenu[VARIANT];
    auto* d = static_cast<typename St::bits*>(dd);
    // grid: x over the groups of one plane, y over planes (in chunks of at most
    // 65535 planes, the grid's y limit)
    constexpr int kMaxPlanes = 65535;
    auto launch = [&](auto kern, int CPT, int block) -> cudaError_t {
        const int G = (g.nx + CPT - 1) / CPT;
        const long long per_plane = (long long)G * g.ny;
        if (per_plane > 0xffffffffll) return cudaErrorInvalidValue;
        const FastDiv divG = FastDiv::make((uint32_t)G);
        const unsigned bx = (unsigned)((per_plane + block - 1) / block);
        for (int z0 = 0; z0 < g.nz; z0 += kMaxPlanes) {
            const int planes = g.nz - z0 < kMaxPlanes ? g.nz - z0 : kMaxPlanes;
            kern<<<dim3(bx, (unsigned)planes), block, 0, st>>>(d, g, T(p.inv_tau), T(p.lid_u), lid_y, p.wall_y,
                                                               p.step_base, p.step_off, divG, z0);
            if (z0 > 0) add_launches(1);
        }
        return cudaGetLastError();
    };
    if (alpha) {
        constexpr KernelShape k = fv.alpha;
        constexpr int CPT = shape_cpt<St>(k);
        return launch(alpha_fast<St, CPT, k.block, k.minb>, CPT, k.block);
    }
    constexpr KernelShape k = fv.beta;
    constexpr int CPT = shape_cpt<St>(k);
    if constexpr (fv.packed != 0 && sizeof(typename St::bits) == 2)
        return launch(beta_fast_pk<St, CPT, k.block, k.minb, fv.packed == 2>, CPT, k.block);
    else if constexpr (fv.direct) return launch(beta_fast_direct<St, CPT, k.block, k.minb>, CPT, k.block);
    else if constexpr (fv.block_exchange) return launch(beta_fast_blk<St, CPT, k.block, k.minb>, CPT, k.block);
    else return launch(beta_fast<St, CPT, k.block, k.minb>, CPT, k.block);
}

template <class St, size_t... I>
cudaError_t launch_fast_table(int variant, bool alpha, void* dd, const Grid& g, const Params& p, int lid_y,
                              cudaStream_t st, std::index_sequence<I...>)
{
    using Fn = cudaError_t (*)(bool, void*, const Grid&, const Params&, int, cudaStream_t);
    static constexpr Fn table[] = {&launch_fast_variant<St, (int)I>...};
    return table[variant](alpha, dd, g, p, lid_y, st);
}

template <class St>
cudaError_t launch_fast_menu(int variant, bool alpha, void* dd, const Grid& g, const Params& p, int lid_y,
                             cudaStream_t st)
{
    if (variant < 0 || variant >= kRegisterVariants) return cudaErrorInvalidValue;
    return launch_fast_table<St>(variant, alpha, dd, g, p, lid_y, st, std::make_index_sequence<kRegisterVariants>{});
}

}  // namespace lbm

namespace lbm {

// ---------------------------------------------------------------------------
// Batches: many box cavities advanced by one launch.  The domains' padded
// population arrays share one device pool; a packed table gives each its
// layout, offset, parameters and its range of "virtual blocks" (BLOCK
// threads x CPT cells each, numbered consecutively over the domains).  A
// persistent grid walks the virtual blocks; a per-kernel map gives each
// virtual block's domain, and every CTA runs the same per-thread bodies as
// the single-domain kernels, so a domain's result does not depend on its
// neighbours in the batch.
// ---------------------------------------------------------------------------
struct alignas(16) BatchDomain {
    Grid g;
    long long offset;          // elements from the pool base
    double inv_tau;
    double lid_u;
    int lid_y;
    uint32_t step0;            // added to the launch's step: this domain's own step count
    int wall_y;                // row under a moving top wall, 0: none (see wall_correct)
    long long block_start[2];  // first virtual block of this domain: [0] alpha, [1] beta kernel
    FastDiv div_g[2];          // division by the groups per row of the alpha / beta shape
    FastDiv div_ny;            // division by ny
};
static_assert(sizeof(BatchDomain) % 16 == 0, "descriptors are copied in 16-byte chunks");

// Fills the virtual-block geometry of kernel `kind` (0 alpha, 1 beta) for a
// shape of `cpt` cells per thread and `block` threads, and returns the
// domain's number of virtual blocks, or -1 if its thread index would not fit
// 32 bits (the batch kernel divides 32-bit thread indices).
inline long long set_batch_shape(BatchDomain& d, int kind, int cpt, int block)
{
    const long long G = (d.g.nx + cpt - 1) / cpt;
    const long long threads = G * d.g.ny * d.g.nz;
    const long long blocks = (threads + block - 1) / block;
    if (blocks * block >= (1ll << 32)) return -1;
    d.div_g[kind] = FastDiv::make((uint32_t)G);
    d.div_ny = FastDiv::make((uint32_t)d.g.ny);
    return blocks;
}

// The group of thread t of a domain's virtual blocks, t = ((z-1) * ny +
// (y-1)) * G + gi; threads past the last group get a valid group, inactive.
__host__ __device__ __forceinline__ Cells cells_of_vblock(const BatchDomain& d, int which, uint32_t t)
{
    const FastDiv& dg = d.div_g[which];
    const uint32_t row = dg.div(t);
    const uint32_t zz = d.div_ny.div(row);
    Cells c;
    c.active = zz < (uint32_t)d.g.nz;
    c.gi = c.active ? (int)(t - row * dg.d) : 0;
    c.y = c.active ? 1 + (int)(row - zz * (uint32_t)d.g.ny) : 1;
    c.z = c.active ? 1 + (int)zz : 1;
    return c;
}

// 16-byte asynchronous global -> shared copies (cp.async, no registers held
// while in flight).
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
    const unsigned a = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(a), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Persistent batch step.  CTA i walks virtual blocks i, i + grid, ... (so the
// resident CTAs work on one compact front of the pool, as a plain grid would).
// The descriptor of the next virtual block's domain is copied into shared
// memory (cp.async) while the current one is processed, so a block starts
// without a dependent table lookup; one block barrier per virtual block
// publishes it and keeps the other buffer from being overwritten while read.
// Every thread of a CTA walks the same virtual blocks, so that barrier and
// the block-wide barriers of the exchanging beta body are reached uniformly.
// kBeta: 0 warp exchange (beta_cells), 1 block exchange (beta_cells_blk),
// 2 direct windows (beta_cells_direct), 3 and 4 packed 16-bit windows
// (beta_cells_pk with piece or vector loads).
template <class St, int CPT, int BLOCK, int MINB, bool kAlpha, int kBeta>
__global__ void __launch_bounds__(BLOCK, MINB) batch_step(typename St::bits* __restrict__ pool,
                                                          const BatchDomain* __restrict__ doms,
                                                          const int* __restrict__ vb_dom,
                                                          const long long vblocks,
                                                          const uint32_t* __restrict__ step_base,
                                                          const uint32_t step_off)
{
    using T = typename St::T;
    constexpr int which = kAlpha ? 0 : 1;
    constexpr int kChunks = (int)(sizeof(BatchDomain) / 16);
    static_assert(kChunks <= BLOCK, "one thread per descriptor chunk");
    __shared__ BatchDomain desc[2];
    const long long stride = gridDim.x;
    long long vb = blockIdx.x;
    if (vb >= vblocks) return;
    const uint32_t step = step_of<St>(step_base, step_off);
    if (threadIdx.x < kChunks)
        cp_async16(reinterpret_cast<uint4*>(&desc[0]) + threadIdx.x,
                   reinterpret_cast<const uint4*>(doms + vb_dom[vb]) + threadIdx.x);
    cp_async_commit();
    int next_dom = vb + stride < vblocks ? vb_dom[vb + stride] : 0;
    for (int buf = 0; vb < vblocks; vb += stride, buf ^= 1) {
        cp_async_wait_all();
        __syncthreads();
        if (vb + stride < vblocks && threadIdx.x < kChunks)
            cp_async16(reinterpret_cast<uint4*>(&desc[buf ^ 1]) + threadIdx.x,
                       reinterpret_cast<const uint4*>(doms + next_dom) + threadIdx.x);
        cp_async_commit();
        next_dom = vb + 2 * stride < vblocks ? vb_dom[vb + 2 * stride] : 0;
        const BatchDomain& d = desc[buf];
        const Cells c = cells_of_vblock(d, which, (uint32_t)(vb - d.block_start[which]) * BLOCK + threadIdx.x);
        const uint32_t ds = step + d.step0;
        const Grid g = d.g;  // in registers for the body (its barriers would force shared-memory reloads)
        typename St::bits* const dd = pool + d.offset;
        const T inv_tau = T(d.inv_tau), lid_u = T(d.lid_u);
        const int lid_y = d.lid_y, wall_y = d.wall_y;
        if constexpr (kAlpha) alpha_cells<St, CPT>(dd, g, inv_tau, lid_u, lid_y, wall_y, c, ds);
        else if constexpr (kBeta >= 3) beta_cells_pk<St, CPT, kBeta == 4>(dd, g, inv_tau, lid_u, lid_y, wall_y, c, ds);
        else if constexpr (kBeta == 2) beta_cells_direct<St, CPT>(dd, g, inv_tau, lid_u, lid_y, wall_y, c, ds);
        else if constexpr (kBeta == 1) beta_cells_blk<St, CPT, BLOCK>(dd, g, inv_tau, lid_u, lid_y, wall_y, c, ds);
        else beta_cells<St, CPT>(dd, g, inv_tau, lid_u, lid_y, wall_y, c, ds);
    }
}

template <class St, int VARIANT, bool kAlpha>
cudaError_t launch_batch_kernel(const BatchArgs& a, cudaStream_t st)
{
    constexpr FastVariant fv = kFastMenu[VARIANT];
    constexpr KernelShape k = kAlpha ? fv.alpha : fv.beta;
    constexpr int CPT = shape_cpt<St>(k);
    constexpr bool pk = fv.packed != 0 && sizeof(typename St::bits) == 2;
    auto kern = batch_step<St, CPT, k.block, k.minb, kAlpha,
                           pk ? 2 + fv.packed : fv.direct ? 2 : fv.block_exchange ? 1 : 0>;
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, k.block, 0);
    if (e != cudaSuccess) return e;
    long long grid = (long long)(per_sm > 0 ? per_sm : 1) * sms;
    if (grid > a.vblocks) grid = a.vblocks;
    if (grid < 1) return cudaSuccess;
    kern<<<(int)grid, k.block, 0, st>>>(static_cast<typename St::bits*>(a.pool), a.doms, a.vb_dom, a.vblocks,
                                        a.step_base, a.step_off);
    return cudaGetLastError();
}

template <class St, int VARIANT>
cudaError_t launch_batch_variant(bool alpha, const BatchArgs& a, cudaStream_t st)
{
    return alpha ? launch_batch_kernel<St, VARIANT, true>(a, st) : launch_batch_kernel<St, VARIANT, false>(a, st);
}

template <class St, size_t... I>
cudaError_t launch_batch_table(int variant, bool alpha, const BatchArgs& a, cudaStream_t st, std::index_sequence<I...>)
{
    using Fn = cudaError_t (*)(bool, const BatchArgs&, cudaStream_t);
    static constexpr Fn table[] = {&launch_batch_variant<St, (int)I>...};
    return table[variant](alpha, a, st);
}

// The step of domain d is *step_base + step_off + d.step0.
template <class St>
cudaError_t launch_batch_menu(int variant, bool alpha, const BatchArgs& a, cudaStream_t st)
{
    if (variant < 0 || variant >= kRegisterVariants) return cudaErrorInvalidValue;
    return launch_batch_table<St>(variant, alpha, a, st, std::make_index_sequence<kRegisterVariants>{});
}

}  // namespace lbm
