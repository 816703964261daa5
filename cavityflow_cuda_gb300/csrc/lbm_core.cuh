// lbm_core.cuh -- lattice, storage layout and collision arithmetic shared by
// every kernel of the GB300 D3Q19 A-A solver.
//
// The translation units that include this header are compiled with
// -fmad=false: the FP64 and FP32 collisions below then execute exactly the
// IEEE operations, in the same order, as the reference kernels built for
// x86-64 (src/gpukernels/lbm_alpha.cu:86-331, src/gpukernels/lbm_beta.cu:98-636,
// src/common.h:132-160), which gives bit-identical populations.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace lbm {

constexpr int Q = 19;

// Flag values of src/common.h:54-61 (stored as one byte per cell here).
enum : uint8_t { kObstacle = 1, kFluid = 2, kInjection = 4, kGhost = 8 };

// D3Q19 ordering of src/common.h:29-47: 0 +x, 1 -x, 2 +y, 3 -y, 4 (+x+y),
// 5 (-x-y), 6 (+x-y), 7 (-x+y), 8 (+x+z), 9 (-x-z), 10 (+x-z), 11 (-x+z),
// 12 (+y+z), 13 (-y-z), 14 (+y-z), 15 (-y+z), 16 +z, 17 -z, 18 rest.
// Opposite directions pair as (2k, 2k+1).
__host__ __device__ constexpr int dir_x(int k)
{
    return k == 0 ? 1 : k == 1 ? -1 : k == 4 ? 1 : k == 5 ? -1 : k == 6 ? 1 : k == 7 ? -1
         : k == 8 ? 1 : k == 9 ? -1 : k == 10 ? 1 : k == 11 ? -1 : 0;
}
__host__ __device__ constexpr int dir_y(int k)
{
    return k == 2 ? 1 : k == 3 ? -1 : k == 4 ? 1 : k == 5 ? -1 : k == 6 ? -1 : k == 7 ? 1
         : k == 12 ? 1 : k == 13 ? -1 : k == 14 ? 1 : k == 15 ? -1 : 0;
}
__host__ __device__ constexpr int dir_z(int k)
{
    return k == 8 ? 1 : k == 9 ? -1 : k == 10 ? -1 : k == 11 ? 1 : k == 12 ? 1 : k == 13 ? -1
         : k == 14 ? -1 : k == 15 ? 1 : k == 16 ? 1 : k == 17 ? -1 : 0;
}
__host__ __device__ constexpr int opp(int k) { return k == 18 ? 18 : (k ^ 1); }

// Lattice weight of direction k in precision T, folded as the reference
// writes them: (T)1/(T)18, (T)1/(T)36, (T)1/(T)3.
template <typename T>
__host__ __device__ constexpr T weight(int k)
{
    return k == 18 ? T(1) / T(3) : (k < 4 || k >= 16) ? T(1) / T(18) : T(1) / T(36);
}

// ---------------------------------------------------------------------------
// Device layout of the population array.
//
// 19 slots; slot k is a padded 3-D array of (nz+2) planes x (ny+2) rows x P
// columns.  Cell x of a row (halo coordinates, 0..nx+1) sits at column
// x + xoff.  xoff = (32 bytes / element) - 1 puts interior cell x = 1 on a
// 32-byte sector boundary, so each 16-byte vector group of the fast kernels
// (cells 1+gV .. V+gV, V = 16 bytes / element) is aligned, and each warp's
// 32 consecutive groups start on a sector.  P leaves room for one scalar
// access right of the last group and is a multiple of 32 bytes, and every
// slot starts on a 256-byte boundary.
//
// Batches and servers pack their boxes' rows tighter (x1_align = 8): x = 1
// on an 8-byte boundary, rows sized for 8-byte vectors and P a multiple of 8
// bytes.  L2 fetches a 128-byte line whole when a short row touches part of
// it; with packed rows the neighbouring rows' cells fill more of those lines,
// and the rows of small boxes carry less padding.  The register kernels need
// x = 1 aligned to their widest vector and index through idx(), so every
// layout runs the same code with the same results for the variants whose
// vectors fit it (vector_fits); the bulk-copy kernels run on the default
// layout only.
// ---------------------------------------------------------------------------
struct Grid {
    int nx, ny, nz;      // interior cells
    int V;               // cells per widest vector the rows are sized for (16 bytes; 8 when packed)
    int xoff;            // column of halo cell x = 0
    int G;               // vector groups per row, ceil(nx / V)
    long long P;         // row pitch (elements)
    long long PY;        // plane pitch (elements) = P * (ny + 2)
    long long S;         // slot stride (elements)

    __host__ __device__ long long idx(int x, int y, int z) const
    {
        return (long long)z * PY + (long long)y * P + x + xoff;
    }
    // Index of a cell in the compact, unpadded reference layout
    // ((nz+2) x (ny+2) x (nx+2), x fastest) used by flags and macro arrays.
    __host__ __device__ long long ref(int x, int y, int z) const
    {
        return ((long long)z * (ny + 2) + y) * (nx + 2) + x;
    }
    __host__ __device__ long long cells() const { return (long long)(nx + 2) * (ny + 2) * (nz + 2); }
};

// x1_align: byte alignment of x = 1, 32 (the default layout), 16 or 8.
inline Grid make_grid(int nx, int ny, int nz, int elem_bytes, int x1_align = 32)
{
    Grid g;
    g.nx = nx; g.ny = ny; g.nz = nz;
    g.V = (x1_align < 16 ? x1_align : 16) / elem_bytes;
    const int sector = x1_align / elem_bytes;
    g.xoff = sector - 1;
    g.G = (nx + g.V - 1) / g.V;
    const long long need = (long long)g.xoff + (long long)g.G * g.V + 2;  // last scalar column + 1
    g.P = (need + sector - 1) / sector * sector;
    g.PY = g.P * (ny + 2);
    const long long slot_align = 256 / elem_bytes;
    g.S = (g.PY * (nz + 2) + slot_align - 1) / slot_align * slot_align;
    return g;
}

// Alignment of x = 1 in the rows of batch and server boxes (see above).
constexpr int kPackedX1Align = 8;

// True for the default layout (x = 1 on a 32-byte boundary).
inline bool default_layout(const Grid& g, int elem_bytes) { return g.xoff == 32 / elem_bytes - 1; }

// Whether vectors of `bytes` bytes are aligned in this layout and its rows
// have room for them.
inline bool vector_fits(const Grid& g, int elem_bytes, int bytes) { return bytes <= g.V * elem_bytes; }

// ---------------------------------------------------------------------------
// Storage types.  F64/F32 hold f_i; F16S/BF16S/F16SR hold the deviation
// f_i - w_i as raw 16-bit patterns.  `T` is the arithmetic type of the
// collision.  `stochastic` types round the step kernels' stores with a dither
// keyed by (cell, population, time step): store_sr(v, d) with d from
// sr_dither below; `store` (round to nearest) serves every other write.
// ---------------------------------------------------------------------------
struct F64 {
    using bits = double;
    using T = double;
    static constexpr bool shifted = false;
    static constexpr bool stochastic = false;
    __device__ static T load(bits b) { return b; }
    __device__ static bits store(T v) { return v; }
    __device__ static T load_step(bits b) { return load(b); }
    static constexpr int kStepLog2 = 0;
};
// FP64 whose step kernels are compiled with fused multiply-adds
// (fast_fma.cu, the one translation unit built with -fmad=true); a type of
// its own so that its kernel instantiations never merge with F64's.
struct F64F : F64 {};
struct F32 {
    using bits = float;
    using T = float;
    static constexpr bool shifted = false;
    static constexpr bool stochastic = false;
    __device__ static T load(bits b) { return b; }
    __device__ static bits store(T v) { return v; }
    __device__ static T load_step(bits b) { return load(b); }
    static constexpr int kStepLog2 = 0;
};
// FP32 whose step kernels fuse multiply-adds (fast_fma.cu), for the same
// reason as F64F.
struct F32F : F32 {};
struct F16S {
    using bits = unsigned short;
    using T = float;
    static constexpr bool shifted = true;
    static constexpr bool stochastic = false;
    __device__ static T load(bits b) { return __half2float(__ushort_as_half(b)); }
    __device__ static bits store(T v) { return __half_as_ushort(__float2half_rn(v)); }
    __device__ static T load_step(bits b) { return load(b); }
    static constexpr int kStepLog2 = 0;
};
struct BF16S {
    using bits = unsigned short;
    using T = float;
    static constexpr bool shifted = true;
    static constexpr bool stochastic = false;
    // Widening as the mixed-precision add b + (-0.0f), which is exact (zeros
    // keep their sign, subnormals stay): it reads a bfloat16 half of a
    // register in place, as the FP16 conversions do, where a shift into a
    // register of its own per element took the 8-cell alpha from 168 to 239
    // registers.
    __device__ static T load(bits b)
    {
        float r;
        asm("add.rn.f32.bf16 %0, %1, %2;" : "=f"(r) : "h"(b), "f"(-0.0f));
        return r;
    }
    __device__ static bits store(T v) { return __bfloat16_as_ushort(__float2bfloat16_rn(v)); }
    __device__ static T load_step(bits b) { return load(b); }
    static constexpr int kStepLog2 = 0;
};

// Stochastic-rounding keys.  sr_hash mixes the compact index of a row's first
// cell ((nx+2)(ny+2)(nz+2) layout, x = 0) with the time step (the "lowbias32"
// integer hash of C. Wellons); sr_cell gives cell x of that row its own key,
// so a thread hashes once for all its cells; sr_dither gives population k of
// the cell the key's top 13 bits XOR a fixed 13-bit constant of k (a Weyl
// sequence): uniform over [0, 2^13) from cell to cell and step to step, at
// one logic operation per population.
__host__ __device__ __forceinline__ uint32_t sr_hash(uint32_t row_cell, uint32_t step)
{
    uint32_t x = row_cell ^ (step * 0x9E3779B9u);
    x ^= x >> 16;
    x *= 0x7FEB352Du;
    x ^= x >> 15;
    x *= 0x846CA68Bu;
    x ^= x >> 16;
    return x;
}
__host__ __device__ __forceinline__ uint32_t sr_cell(uint32_t row_hash, int x)
{
    return (row_hash ^ ((uint32_t)x * 0x85EBCA6Bu)) * 0x2545F491u;
}
__host__ __device__ __forceinline__ uint32_t sr_dither(uint32_t h, int k)
{
    return (h >> 19) ^ (((uint32_t)(k + 1) * 0x9E3779B9u) >> 19);
}

// IEEE half deviations scaled by 2^kF16SRScale, rounded stochastically.
// Scaling by a power of two is exact; it moves deviations down to 2^-26 out
// of the half subnormal range, where a 13-bit dither would not cover every
// discarded bit.  Rounding: the dither is added to the float's bit pattern
// below the 13 bits that half precision drops (this acts on the magnitude;
// the sign bit is above it), then the value is truncated toward zero, so a
// value between two halves rounds away from zero with probability equal to
// its distance from the smaller one: the expected stored value is exact.
// Round to nearest (the rounding error's sign fixed by the value) lets slow
// changes stall below half a unit and bias the flow; the dither removes that.
//
// The step kernels work in the scaled units (load_step, store_sr): the
// collision is linear in the deviations except for |j|^2 and u^2, whose
// constants collide_shifted<kStepLog2> divides by the scale, so every result
// is exactly 2^12 times the unscaled one and no multiply by the scale is
// needed per population.  load/store (getters, setters) use plain units.
constexpr int kF16SRScale = 12;
struct F16SR {
    using bits = unsigned short;
    using T = float;
    static constexpr bool shifted = true;
    static constexpr bool stochastic = true;
    static constexpr int kStepLog2 = kF16SRScale;
    __device__ static T load(bits b)
    {
        return __half2float(__ushort_as_half(b)) * __uint_as_float((uint32_t)(127 - kF16SRScale) << 23);
    }
    __device__ static bits store(T v)
    {
        return __half_as_ushort(__float2half_rn(v * __uint_as_float((uint32_t)(127 + kF16SRScale) << 23)));
    }
    __device__ static T load_step(bits b) { return __half2float(__ushort_as_half(b)); }
    __device__ static bits store_sr(T scaled, uint32_t dither)
    {
        return __half_as_ushort(__float2half_rz(__uint_as_float(__float_as_uint(scaled) + dither)));
    }
};

// The time step that keys stochastic rounding: *step_base + step_off (a graph
// replays its launches with the word at step_base rewritten and step_off
// fixed).  Other storage types never read it.
template <class St>
__device__ __forceinline__ uint32_t step_of(const uint32_t* step_base, uint32_t step_off)
{
    if constexpr (St::stochastic) return *step_base + step_off;
    else return 0u;
}

// A step kernel's store of population k of a cell with hash h.
template <class St>
__device__ __forceinline__ typename St::bits store_pop(typename St::T v, uint32_t h, int k)
{
    if constexpr (St::stochastic) return St::store_sr(v, sr_dither(h, k));
    else return St::store(v);
}

// Unsigned 32-bit division by a divisor fixed at launch, as a multiply-high
// and shifts (the round-up method of Granlund and Montgomery, 1994): with
// l = ceil(log2 d) and m = floor(2^32 (2^l - d) / d) + 1, every n < 2^32 has
// n / d = (t + ((n - t) >> 1)) >> (l - 1), t = mulhi(n, m); d = 1 is n.
struct FastDiv {
    uint32_t d = 1, m = 0;
    int l = 0;
    static FastDiv make(uint32_t d)
    {
        FastDiv f;
        f.d = d;
        if (d > 1) {
            int l = 0;
            while ((1ull << l) < d) ++l;
            f.l = l;
            f.m = (uint32_t)((((1ull << 32) * ((1ull << l) - d)) / d) + 1);
        }
        return f;
    }
    __host__ __device__ __forceinline__ uint32_t div(uint32_t n) const
    {
        if (l == 0) return n;
#ifdef __CUDA_ARCH__
        const uint32_t t = __umulhi(n, m);
#else
        const uint32_t t = (uint32_t)(((uint64_t)n * m) >> 32);  // the same high word, for host checks
#endif
        return (t + ((n - t) >> 1)) >> (l - 1);
    }
};

// Scalar lattice parameters of one domain, and the time step of the next
// launch, *step_base + step_off (it keys stochastic rounding; step_base points
// to device memory so that captured graphs can be replayed at later steps).
// wall_y: the row of cells under a moving top wall (the opt-in
// mass-conserving lid, see wall_correct), or 0 when the top wall is at rest.
struct Params {
    double inv_tau;
    double lid_u;
    double gx, gy, gz;
    const uint32_t* step_base = nullptr;
    uint32_t step_off = 0;
    int wall_y = 0;
};

// ---------------------------------------------------------------------------
// Collision arithmetic (operation order of the reference, see file header).
// ---------------------------------------------------------------------------

// Density and momentum, each accumulator in the order of
// src/gpukernels/lbm_alpha.cu:86-186.
template <typename T>
__device__ __forceinline__ void moments(const T* f, T& rho, T& vx, T& vy, T& vz)
{
    T r = f[0], x = f[0], y, z;
    r += f[1];  x -= f[1];
    r += f[2];  y = f[2];
    r += f[3];  y -= f[3];
    r += f[4];  x += f[4];  y += f[4];
    r += f[5];  x -= f[5];  y -= f[5];
    r += f[6];  x += f[6];  y -= f[6];
    r += f[7];  x -= f[7];  y += f[7];
    r += f[8];  x += f[8];  z = f[8];
    r += f[9];  x -= f[9];  z -= f[9];
    r += f[10]; x += f[10]; z -= f[10];
    r += f[11]; x -= f[11]; z += f[11];
    r += f[12]; y += f[12]; z += f[12];
    r += f[13]; y -= f[13]; z -= f[13];
    r += f[14]; y += f[14]; z -= f[14];
    r += f[15]; y -= f[15]; z += f[15];
    r += f[16]; z += f[16];
    r += f[17]; z -= f[17];
    r += f[18];
    rho = r; vx = x; vy = y; vz = z;
}

// Incompressible equilibrium, src/common.h:132-160.
template <typename T>
__device__ __forceinline__ void pair_eq(T w, T P, T s, T& plus, T& minus)
{
    const T s2 = s * s;
    plus = w * (P + T(3) * s + (T(9) / T(2)) * s2);
    minus = w * (P + T(-3) * s + (T(9) / T(2)) * s2);
}

template <typename T>
__device__ __forceinline__ void equilibrium(T rho, T vx, T vy, T vz, T* e)
{
    const T vel2 = vx * vx + vy * vy + vz * vz;
    const T P = rho - (T(3) / T(2)) * vel2;
    const T wa = T(1) / T(18), wd = T(1) / T(36);
    pair_eq(wa, P, vx, e[0], e[1]);
    pair_eq(wa, P, vy, e[2], e[3]);
    pair_eq(wd, P, vx + vy, e[4], e[5]);
    pair_eq(wd, P, vx - vy, e[6], e[7]);
    pair_eq(wd, P, vx + vz, e[8], e[9]);
    pair_eq(wd, P, vx - vz, e[10], e[11]);
    pair_eq(wd, P, vy + vz, e[12], e[13]);
    pair_eq(wd, P, vy - vz, e[14], e[15]);
    pair_eq(wa, P, vz, e[16], e[17]);
    e[18] = (T(1) / T(3)) * P;
}

// Alpha-step gravity (src/gpukernels/lbm_alpha.cu:213-326).  In the reference
// each term is stored in `tmp`, a #define for `rho` (lbm_alpha.cu:203), so each
// term after the first scales the previous term; reproduced as written.
template <typename T>
__device__ __forceinline__ void alpha_gravity(T* f, T rho, T gx, T gy, T gz)
{
    const T wa = T(1) / T(18), wd = T(1) / T(36);
    T t = gx * wa * rho;                    f[1] -= t;  f[0] += t;
    t = gy * (T(-1) / T(18)) * t;           f[3] -= t;  f[2] += t;
    t = (gx - gy) * wd * t;                 f[5] -= t;  f[4] += t;
    t = (gx + gy) * wd * t;                 f[7] -= t;  f[6] += t;
    t = (gx + gz) * wd * t;                 f[9] -= t;  f[8] += t;
    t = (gx - gz) * wd * t;                 f[11] -= t; f[10] += t;
    t = (gz - gy) * wd * t;                 f[13] -= t; f[12] += t;
    t = (gz + gy) * (T(-1) / T(36)) * t;    f[15] -= t; f[14] += t;
    t = gz * wa * t;                        f[17] -= t; f[16] += t;
}

// Relaxation of one direction pair toward the equilibrium of pair_eq.
template <typename T>
__device__ __forceinline__ void relax_pair(T& fp, T& fm, T w, T P, T s, T inv_tau)
{
    T ep, em;
    pair_eq(w, P, s, ep, em);
    fp += inv_tau * (ep - fp);
    fm += inv_tau * (em - fm);
}

// BGK collision of a FLUID cell in place (lbm_alpha.cu:209-331,
// lbm_beta.cu:574-636), one direction pair at a time so that no array of 19
// equilibria is live.  For shifted storage f holds f - w and the same
// arithmetic yields the post-collision deviation: with rho the density
// deviation, feq(rho) - w is exactly the reference formula.
template <typename T>
__device__ __forceinline__ void collide_fluid(T* f, T inv_tau)
{
    T rho, vx, vy, vz;
    moments(f, rho, vx, vy, vz);
    const T vel2 = vx * vx + vy * vy + vz * vz;
    const T P = rho - (T(3) / T(2)) * vel2;
    const T wa = T(1) / T(18), wd = T(1) / T(36);
    relax_pair(f[0], f[1], wa, P, vx, inv_tau);
    relax_pair(f[2], f[3], wa, P, vy, inv_tau);
    relax_pair(f[4], f[5], wd, P, vx + vy, inv_tau);
    relax_pair(f[6], f[7], wd, P, vx - vy, inv_tau);
    relax_pair(f[8], f[9], wd, P, vx + vz, inv_tau);
    relax_pair(f[10], f[11], wd, P, vx - vz, inv_tau);
    relax_pair(f[12], f[13], wd, P, vy + vz, inv_tau);
    relax_pair(f[14], f[15], wd, P, vy - vz, inv_tau);
    relax_pair(f[16], f[17], wa, P, vz, inv_tau);
    f[18] += inv_tau * ((T(1) / T(3)) * P - f[18]);
}

template <typename T>
__device__ __forceinline__ void collide_fluid_gravity(T* f, T inv_tau, T gx, T gy, T gz)
{
    T rho, vx, vy, vz, e[Q];
    moments(f, rho, vx, vy, vz);
    equilibrium(rho, vx, vy, vz, e);
#pragma unroll
    for (int k = 0; k < Q; ++k) f[k] += inv_tau * (e[k] - f[k]);
    alpha_gravity(f, rho, gx, gy, gz);
}

// ---------------------------------------------------------------------------
// Collision of the shifted 16-bit storage modes.  Not bound to the
// reference's operation order (those modes have no reference counterpart), so
// it is written for throughput: moments from pair sums and differences, and
// every multiply-add fused.  Same BGK model: for a direction pair with
// projection u = c.j and weight w,
//   feq+- - w = w (P + 4.5 u^2) +- 3 w u,   P = drho - 1.5 |j|^2,
// relaxed as s += omega (feq - w - s).  oracle/lbm_oracle.c restates it with
// fmaf, so the GPU result is checked bit for bit.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void relax_pair_shifted(float& sp, float& sm, float w3, float w45, float wP, float u,
                                                   float omega)
{
    const float even = __fmaf_rn(w45, u * u, wP);
    const float odd = w3 * u;
    sp = __fmaf_rn(omega, (even + odd) - sp, sp);
    sm = __fmaf_rn(omega, (even - odd) - sm, sm);
}

template <int E = 0>
__device__ __forceinline__ void collide_shifted(float* s, float omega)
{
    const float a01 = s[0] + s[1], d01 = s[0] - s[1];
    const float a23 = s[2] + s[3], d23 = s[2] - s[3];
    const float a45 = s[4] + s[5], d45 = s[4] - s[5];
    const float a67 = s[6] + s[7], d67 = s[6] - s[7];
    const float a89 = s[8] + s[9], d89 = s[8] - s[9];
    const float a1011 = s[10] + s[11], d1011 = s[10] - s[11];
    const float a1213 = s[12] + s[13], d1213 = s[12] - s[13];
    const float a1415 = s[14] + s[15], d1415 = s[14] - s[15];
    const float a1617 = s[16] + s[17], d1617 = s[16] - s[17];
    const float drho = ((a01 + a23) + (a45 + a67)) + ((a89 + a1011) + (a1213 + a1415)) + (a1617 + s[18]);
    const float jx = ((d01 + d45) + (d67 + d89)) + d1011;
    const float jy = ((d23 + d45) - d67) + (d1213 + d1415);
    const float jz = ((d89 - d1011) + (d1213 - d1415)) + d1617;
    const float vel2 = __fmaf_rn(jz, jz, __fmaf_rn(jy, jy, jx * jx));
    // with deviations scaled by 2^E the quadratic terms carry 2^-E (exact)
    constexpr float inv_scale = 1.0f / (float)(1u << E);
    const float P = __fmaf_rn(-1.5f * inv_scale, vel2, drho);
    const float wa = 1.0f / 18.0f, wd = 1.0f / 36.0f;
    const float waP = wa * P, wdP = wd * P;
    const float wa3 = 3.0f * wa, wa45 = (4.5f * wa) * inv_scale, wd3 = 3.0f * wd, wd45 = (4.5f * wd) * inv_scale;
    relax_pair_shifted(s[0], s[1], wa3, wa45, waP, jx, omega);
    relax_pair_shifted(s[2], s[3], wa3, wa45, waP, jy, omega);
    relax_pair_shifted(s[4], s[5], wd3, wd45, wdP, jx + jy, omega);
    relax_pair_shifted(s[6], s[7], wd3, wd45, wdP, jx - jy, omega);
    relax_pair_shifted(s[8], s[9], wd3, wd45, wdP, jx + jz, omega);
    relax_pair_shifted(s[10], s[11], wd3, wd45, wdP, jx - jz, omega);
    relax_pair_shifted(s[12], s[13], wd3, wd45, wdP, jy + jz, omega);
    relax_pair_shifted(s[14], s[15], wd3, wd45, wdP, jy - jz, omega);
    relax_pair_shifted(s[16], s[17], wa3, wa45, waP, jz, omega);
    s[18] = __fmaf_rn(omega, (1.0f / 3.0f) * P - s[18], s[18]);
}

// Collision dispatch by storage: the reference's arithmetic for F64/F32, the
// fused form above for the shifted 16-bit modes.
template <class St>
__device__ __forceinline__ void collide(typename St::T* f, typename St::T inv_tau)
{
    if constexpr (St::shifted) collide_shifted<St::kStepLog2>(f, inv_tau);
    else collide_fluid(f, inv_tau);
}

// VELOCITY_INJECTION: feq(rho = 1, j = (U, 0, 0)) (lbm_alpha.cu:376-511,
// lbm_beta.cu:661-732); rho0 = 0 gives the deviation form for shifted storage.
template <typename T>
__device__ __forceinline__ void inject(T* f, T rho0, T lid_u)
{
    equilibrium(rho0, lid_u, T(0), T(0), f);
}

// Moving top wall: the opt-in alternative to the reference's injection lid
// (no reference counterpart).  The top face y = ny + 1 is an obstacle wall
// moving at U along x, and the cells of row y = ny stay FLUID.  Walls bounce
// populations back (A-A: a population that entered a wall slot is read back
// reversed), so populations 5 (-x-y) and 6 (+x-y) that such a cell reads are
// populations 4 (+x+y) and 7 (-x+y) returned by the wall.  Ladd's moving-wall
// rule, f_opp(i) = f_i - 6 w_i rho_w (c_i . U) with rho_w = 1, adds
// -6 (1/36) U = -U/6 to population 5 and +U/6 to population 6.  The two
// corrections of a cell cancel, so the total mass stays constant.  `du` is
// U/6 in a storage type's step units (wall_shift).
template <class St>
__device__ __forceinline__ typename St::T wall_shift(typename St::T lid_u)
{
    using T = typename St::T;
    T du = lid_u * (T(1) / T(6));
    if constexpr (St::kStepLog2 != 0) du *= (float)(1u << St::kStepLog2);
    return du;
}
template <typename T>
__device__ __forceinline__ void wall_correct(T* f, T du)
{
    f[5] -= du;
    f[6] += du;
}

// The same in a storage type's step units (scaled deviations for F16SR).
template <class St>
__device__ __forceinline__ void inject_step(typename St::T* f, typename St::T rho0, typename St::T lid_u)
{
    inject(f, rho0, lid_u);
    if constexpr (St::kStepLog2 != 0) {
#pragma unroll
        for (int k = 0; k < Q; ++k) f[k] *= (float)(1u << St::kStepLog2);
    }
}

}  // namespace lbm
