// lbm_kernels.cu -- sm_103a kernels of the D3Q19 A-A lid-driven cavity other
// than the vectorised hot path (lbm_fast.cuh, instantiated in fast_*.cu):
// the general flag-array step kernels (any flags, cuboid sub-steps,
// gravity; one cell per thread), initialisation, the cavity-flag check,
// macroscopic fields, the FP64 reduction and the 16-bit pack/unpack.
#include <cstdint>
#include <type_traits>
#include <utility>

#include "lbm_core.cuh"
#include "lbm_fast.cuh"
#include "lbm_kernels.h"

namespace lbm {

// ===========================================================================
// General path: flag array, cuboid, gravity, halo cells with any flag
// ===========================================================================

// Position of slot k touched by halo cell (x, y, z) in the beta step: the
// reference wraps the linear index modulo the cell count (DOMAIN_WRAP,
// src/gpukernels/lbm_beta.cu:22-25, :59-64).
__device__ __forceinline__ long long wrapped_position(const Grid& g, int x, int y, int z, int k)
{
    const long long X = g.nx + 2, XY = X * (g.ny + 2), C = XY * (g.nz + 2);
    const int cx = dir_x(k), cy = dir_y(k), cz = dir_z(k);
    long long d = (cx > 0 ? 1 : cx < 0 ? C - 1 : 0) + (cy > 0 ? X : cy < 0 ? C - X : 0) +
                  (cz > 0 ? XY : cz < 0 ? C - XY : 0);
    const long long lin = (g.ref(x, y, z) + d) % C;
    const int zn = (int)(lin / XY);
    const int yn = (int)((lin / X) % (g.ny + 2));
    const int xn = (int)(lin % X);
    return g.idx(xn, yn, zn);
}

// The moving top wall on the flag-array path: a FLUID cell of row
// prm.wall_y takes wall_correct for each of its links 4 (+x+y) and 7 (-x+y)
// that end in an OBSTACLE cell of the row above (the moving face).
template <class St>
__device__ __forceinline__ void wall_correct_flagged(typename St::T* f, const uint8_t* __restrict__ flags,
                                                     const Grid& g, const Params& prm, int x, int y, int z)
{
    using T = typename St::T;
    if (prm.wall_y <= 0 || y != prm.wall_y || x < 1 || x > g.nx || z < 1 || z > g.nz) return;
    const T du = wall_shift<St>(T(prm.lid_u));
    if (flags[g.ref(x + 1, y + 1, z)] == kObstacle) f[5] -= du;
    if (flags[g.ref(x - 1, y + 1, z)] == kObstacle) f[6] += du;
}

template <class St, bool kGravity>
__global__ void alpha_general(typename St::bits* __restrict__ dd, const uint8_t* __restrict__ flags,
                              const Grid g, const Params prm, const int3 o, const int3 s)
{
    using T = typename St::T;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)s.x * s.y * s.z;
    if (t >= n) return;
    const int x = o.x + (int)(t % s.x);
    const int y = o.y + (int)((t / s.x) % s.y);
    const int z = o.z + (int)(t / ((long long)s.x * s.y));
    const uint8_t fl = flags[g.ref(x, y, z)];
    if (fl != kFluid && fl != kInjection) return;  // OBSTACLE, GHOST: untouched
    const long long c0 = g.idx(x, y, z);
    const T inv_tau = T(prm.inv_tau);
    T f[Q];
    if (fl == kFluid) {
#pragma unroll
        for (int k = 0; k < Q; ++k) f[k] = St::load_step(dd[k * g.S + c0]);
        wall_correct_flagged<St>(f, flags, g, prm, x, y, z);
        if (kGravity) collide_fluid_gravity(f, inv_tau, T(prm.gx), T(prm.gy), T(prm.gz));
        else collide<St>(f, inv_tau);
    } else {
        inject_step<St>(f, St::shifted ? T(0) : T(1), T(prm.lid_u));
        if (kGravity) alpha_gravity(f, T(1), T(prm.gx), T(prm.gy), T(prm.gz));
    }
    uint32_t h = 0;
    if constexpr (St::stochastic)
        h = sr_cell(sr_hash((uint32_t)g.ref(0, y, z), step_of<St>(prm.step_base, prm.step_off)), x);
#pragma unroll
    for (int k = 0; k < Q; ++k) dd[opp(k) * g.S + c0] = store_pop<St>(f[k], h, k);
}

template <class St>
__global__ void beta_general(typename St::bits* __restrict__ dd, const uint8_t* __restrict__ flags,
                             const Grid g, const Params prm, const int3 o, const int3 s)
{
    using T = typename St::T;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)s.x * s.y * s.z;
    if (t >= n) return;
    const int x = o.x + (int)(t % s.x);
    const int y = o.y + (int)((t / s.x) % s.y);
    const int z = o.z + (int)(t / ((long long)s.x * s.y));
    const uint8_t fl = flags[g.ref(x, y, z)];
    if (fl == kObstacle) return;  // swaps then writes back what it read: a no-op
    const bool interior = x >= 1 && x <= g.nx && y >= 1 && y <= g.ny && z >= 1 && z <= g.nz;
    long long pos[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k)
        pos[k] = k * g.S + (interior ? g.idx(x + dir_x(k), y + dir_y(k), z + dir_z(k))
                                     : wrapped_position(g, x, y, z, k));
    T f[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) f[opp(k)] = St::load_step(dd[pos[k]]);
    if (fl == kFluid) {
        wall_correct_flagged<St>(f, flags, g, prm, x, y, z);
        collide<St>(f, T(prm.inv_tau));
    }
    else if (fl == kInjection) inject_step<St>(f, St::shifted ? T(0) : T(1), T(prm.lid_u));
    // GHOST_LAYER (and any other value): streamed through unchanged (a value
    // read from storage is stored back exactly, also by stochastic rounding)
    uint32_t h = 0;
    if constexpr (St::stochastic)
        h = sr_cell(sr_hash((uint32_t)g.ref(0, y, z), step_of<St>(prm.step_base, prm.step_off)), x);
#pragma unroll
    for (int k = 0; k < Q; ++k) dd[pos[k]] = store_pop<St>(f[k], h, k);
}

// ===========================================================================
// Initialisation, flags, macroscopic fields, reductions, packing
// ===========================================================================

template <class St>
__global__ void init_populations(typename St::bits* __restrict__ dd, const Grid g)
{
    using T = typename St::T;
    const long long n = (long long)Q * g.S;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(i / g.S);
        // feq(rho = 1, u = 0) evaluated as src/gpukernels/lbm_init.cu:97-193 does
        T e[Q];
        equilibrium(T(1), T(0), T(0), T(0), e);
        T v = T(0);
#pragma unroll
        for (int q = 0; q < Q; ++q)
            if (q == k) v = e[q];
        dd[i] = St::store(St::shifted ? T(0) : v);
    }
}

__global__ void init_flags(uint8_t* __restrict__ flags, const Grid g, const Bc bc)
{
    const long long n = g.cells();
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int X = g.nx + 2, Y = g.ny + 2, Z = g.nz + 2;
        const int x = (int)(i % X), y = (int)((i / X) % Y), z = (int)(i / ((long long)X * Y));
        // src/gpukernels/lbm_init.cu:73-93: an OBSTACLE face wins over later faces
        int fl = kFluid;
        if (x == 0) fl = bc.f[0];
        if (x == X - 1 && fl != kObstacle) fl = bc.f[1];
        if (y == 0 && fl != kObstacle) fl = bc.f[2];
        if (y == Y - 1 && fl != kObstacle) fl = bc.f[3];
        if (z == 0 && fl != kObstacle) fl = bc.f[4];
        if (z == Z - 1 && fl != kObstacle) fl = bc.f[5];
        flags[i] = (uint8_t)fl;
    }
}

// Counts cells that differ from the box cavity with all-obstacle halo:
// counts[0] against "lid plane y = ny", counts[1] against "no lid".
__global__ void check_cavity_flags(const uint8_t* __restrict__ flags, const Grid g,
                                   unsigned long long* __restrict__ counts)
{
    unsigned long long bad_lid = 0, bad_nolid = 0;
    const long long n = g.cells();
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int X = g.nx + 2, Y = g.ny + 2;
        const int x = (int)(i % X), y = (int)((i / X) % Y), z = (int)(i / ((long long)X * Y));
        const bool halo = x == 0 || x > g.nx || y == 0 || y > g.ny || z == 0 || z > g.nz;
        const uint8_t fl = flags[i];
        const uint8_t want_nolid = halo ? kObstacle : kFluid;
        const uint8_t want_lid = halo ? kObstacle : (y == g.ny ? kInjection : kFluid);
        bad_lid += fl != want_lid;
        bad_nolid += fl != want_nolid;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        bad_lid += __shfl_down_sync(0xffffffffu, bad_lid, off);
        bad_nolid += __shfl_down_sync(0xffffffffu, bad_nolid, off);
    }
    if ((threadIdx.x & 31) == 0) {
        if (bad_lid) atomicAdd(&counts[0], bad_lid);
        if (bad_nolid) atomicAdd(&counts[1], bad_nolid);
    }
}

// Post-collision populations of interior cell (x,y,z) after the last step:
// after alpha they sit swapped in the cell's own slots, after beta in slot k
// of the neighbour x + c_k.  Returned in arithmetic type (deviation form for
// shifted storage).
template <class St>
__device__ __forceinline__ void post_populations(const typename St::bits* dd, const Grid& g, int x, int y,
                                                 int z, bool last_alpha, typename St::T* f)
{
    const long long c0 = g.idx(x, y, z);
#pragma unroll
    for (int k = 0; k < Q; ++k) {
        const long long p = last_alpha ? opp(k) * g.S + c0
                                       : k * g.S + g.idx(x + dir_x(k), y + dir_y(k), z + dir_z(k));
        f[k] = St::load(dd[p]);
    }
}

// Density and velocity (u = j) of the time level collided last, on the full
// grid in the compact reference layout: out[0] rho, out[1..3] j.
template <class St>
__global__ void compute_macros(const typename St::bits* __restrict__ dd, const uint8_t* __restrict__ flags,
                               const Grid g, const bool last_alpha, const typename St::T lid_u,
                               typename St::T* __restrict__ out)
{
    using T = typename St::T;
    const long long n = g.cells();
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int X = g.nx + 2, Y = g.ny + 2;
        const int x = (int)(i % X), y = (int)((i / X) % Y), z = (int)(i / ((long long)X * Y));
        const bool interior = x >= 1 && x <= g.nx && y >= 1 && y <= g.ny && z >= 1 && z <= g.nz;
        const uint8_t fl = flags[i];
        T r = T(0), vx = T(0), vy = T(0), vz = T(0);
        if (interior && fl == kFluid) {
            T f[Q];
            post_populations<St>(dd, g, x, y, z, last_alpha, f);
            moments(f, r, vx, vy, vz);
            if (St::shifted) r = r + T(1);
        } else if (interior && fl == kInjection) {
            r = T(1);
            vx = lid_u;
        }
        out[i] = r;
        out[n + i] = vx;
        out[2 * n + i] = vy;
        out[3 * n + i] = vz;
    }
}

// The same density and velocity for a box cavity with obstacle walls and the
// lid on plane y = ny (the geometry of a solver after set_driven_cavity),
// taken from the geometry rather than a flag array, for interior cells only,
// packed x fastest: out[0..n) rho, then jx, jy, jz planes of n = nx*ny*nz.
// `out` may be mapped host memory.
template <class St>
__global__ void compute_macros_cavity(const typename St::bits* __restrict__ dd, const Grid g,
                                      const bool last_alpha, const typename St::T lid_u,
                                      typename St::T* __restrict__ out)
{
    using T = typename St::T;
    const long long n = (long long)g.nx * g.ny * g.nz;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int x = 1 + (int)(i % g.nx);
        const int y = 1 + (int)((i / g.nx) % g.ny);
        const int z = 1 + (int)(i / ((long long)g.nx * g.ny));
        T r = T(1), vx = lid_u, vy = T(0), vz = T(0);
        if (y != g.ny) {
            T f[Q];
            post_populations<St>(dd, g, x, y, z, last_alpha, f);
            moments(f, r, vx, vy, vz);
            if (St::shifted) r = r + T(1);
        }
        out[i] = r;
        out[n + i] = vx;
        out[2 * n + i] = vy;
        out[3 * n + i] = vz;
    }
}

// FP64 mass and momentum, pass 1: one partial sum per block (warp shuffles,
// then a fixed-order combine of the warps), so the result is deterministic.
// Mass counts every live slot: the 19 own slots of each active (FLUID or
// lid) interior cell, plus the slots of inactive neighbours (walls) that its
// pushes land in, where a population waits one step before it returns; the
// steps conserve that sum exactly.  Momentum is that of the cells'
// post-collision populations.
template <class St>
__global__ void __launch_bounds__(kReduceBlock) reduce_partials(const typename St::bits* __restrict__ dd,
                                                                const uint8_t* __restrict__ flags,
                                                                const Grid g, const bool last_alpha,
                                                                double* __restrict__ partials)
{
    using T = typename St::T;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const long long n = (long long)g.nx * g.ny * g.nz;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int x = 1 + (int)(i % g.nx);
        const int y = 1 + (int)((i / g.nx) % g.ny);
        const int z = 1 + (int)(i / ((long long)g.nx * g.ny));
        const uint8_t fl = flags[g.ref(x, y, z)];
        if (fl != kFluid && fl != kInjection) continue;
        const long long c0 = g.idx(x, y, z);
        double m = 0.0;
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            const double w = St::shifted ? (double)weight<float>(k) : 0.0;
            m += (double)St::load(dd[k * g.S + c0]) + w;
            const int xn = x + dir_x(k), yn = y + dir_y(k), zn = z + dir_z(k);
            const uint8_t fn = flags[g.ref(xn, yn, zn)];
            if (fn != kFluid && fn != kInjection) m += (double)St::load(dd[k * g.S + g.idx(xn, yn, zn)]) + w;
        }
        T f[Q];
        post_populations<St>(dd, g, x, y, z, last_alpha, f);
        double px = 0.0, py = 0.0, pz = 0.0;
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            const double v = (double)f[k];
            px += dir_x(k) * v;
            py += dir_y(k) * v;
            pz += dir_z(k) * v;
        }
        acc[0] += m; acc[1] += px; acc[2] += py; acc[3] += pz;
    }
    __shared__ double warp_sums[kReduceBlock / 32][4];
#pragma unroll
    for (int q = 0; q < 4; ++q)
        for (int off = 16; off > 0; off >>= 1) acc[q] += __shfl_down_sync(0xffffffffu, acc[q], off);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int q = 0; q < 4; ++q) warp_sums[w][q] = acc[q];
    __syncthreads();
    if (threadIdx.x < 4) {
        double s = 0.0;
        for (int i = 0; i < kReduceBlock / 32; ++i) s += warp_sums[i][threadIdx.x];
        partials[blockIdx.x * 4 + threadIdx.x] = s;
    }
}

// Pass 2: thread q sums column q of the partials in block order.
__global__ void reduce_final(const double* __restrict__ partials, int nblocks, double* __restrict__ out)
{
    if (threadIdx.x < 4) {
        double s = 0.0;
        for (int b = 0; b < nblocks; ++b) s += partials[b * 4 + threadIdx.x];
        out[threadIdx.x] = s;
    }
}

// Cuboid of one slot <-> packed float buffer (x fastest), unshifting (f = s +
// w) on the way out and shifting on the way in for 16-bit storage.  A block
// walks whole rows (one division per row), its threads along x, so both sides
// are coalesced.
template <class St>
__global__ void pack_slot(const typename St::bits* __restrict__ dd, const Grid g, int k, const int3 o,
                          const int3 s, float* __restrict__ out)
{
    const long long rows = (long long)s.y * s.z;
    const float w = weight<float>(k);
    for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
        const int y = o.y + (int)(r % s.y), z = o.z + (int)(r / s.y);
        const typename St::bits* src = dd + k * g.S + g.idx(o.x, y, z);
        float* dst = out + r * s.x;
        for (int x = threadIdx.x; x < s.x; x += blockDim.x) {
            const float v = St::load(src[x]);
            dst[x] = St::shifted ? v + w : v;
        }
    }
}

template <class St>
__global__ void unpack_slot(typename St::bits* __restrict__ dd, const Grid g, int k, const int3 o,
                            const int3 s, const float* __restrict__ in)
{
    const long long rows = (long long)s.y * s.z;
    const float w = weight<float>(k);
    for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
        const int y = o.y + (int)(r % s.y), z = o.z + (int)(r / s.y);
        typename St::bits* dst = dd + k * g.S + g.idx(o.x, y, z);
        const float* src = in + r * s.x;
        for (int x = threadIdx.x; x < s.x; x += blockDim.x) {
            const float v = src[x];
            dst[x] = St::store(St::shifted ? v - w : v);
        }
    }
}

// ===========================================================================
// Host-side launchers
// ===========================================================================

namespace {

long long g_launches = 0;

int grid_for(long long n, int block, int cap = 1 << 30)
{
    long long b = (n + block - 1) / block;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (int)b;
}

template <class F>
cudaError_t with_storage(int storage, F&& f)
{
    switch (storage) {
    case 0: return f(F64{});
    case 1: return f(F32{});
    case 2: return f(F16S{});
    case 3: return f(BF16S{});
    case 4: return f(F16SR{});
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

long long kernel_launches() { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }

void add_launches(long long n) { __atomic_fetch_add(&g_launches, n, __ATOMIC_RELAXED); }

static void count_launch(int n = 1) { add_launches(n); }

cudaError_t launch_init_populations(int storage, void* dd, const Grid& g, cudaStream_t st)
{
    count_launch();
    return with_storage(storage, [&](auto tag) {
        using St = decltype(tag);
        init_populations<St><<<grid_for((long long)Q * g.S, 256, 4096), 256, 0, st>>>(
            static_cast<typename St::bits*>(dd), g);
        return cudaGetLastError();
    });
}

cudaError_t launch_init(int storage, void* dd, uint8_t* flags, const Grid& g, const Bc& bc, cudaStream_t st)
{
    cudaError_t e = with_storage(storage, [&](auto tag) {
        using St = decltype(tag);
        init_populations<St><<<grid_for((long long)Q * g.S, 256, 4096), 256, 0, st>>>(
            static_cast<typename St::bits*>(dd), g);
        return cudaGetLastError();
    });
    if (e != cudaSuccess) return e;
    init_flags<<<grid_for(g.cells(), 256, 4096), 256, 0, st>>>(flags, g, bc);
    count_launch(2);
    return cudaGetLastError();
}

__global__ void set_step_word(uint32_t* word, uint32_t value) { *word = value; }

cudaError_t launch_set_step(uint32_t* word, uint32_t value, cudaStream_t st)
{
    set_step_word<<<1, 1, 0, st>>>(word, value);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_check_cavity(const uint8_t* flags, const Grid& g, unsigned long long* counts,
                                cudaStream_t st)
{
    check_cavity_flags<<<grid_for(g.cells(), 256, 4096), 256, 0, st>>>(flags, g, counts);
    count_launch();
    return cudaGetLastError();
}

bool fast_variant_fits(int storage, int variant, const Grid& g)
{
    if (variant < 0 || variant >= kFastVariantCount) return false;
    if (variant < kRegisterVariants) {  // both kernels' vectors aligned in this layout
        const int eb = storage_elem_bytes(storage);
        const int widest = 16 / (kFastMenu[variant].alpha.cpt_div < kFastMenu[variant].beta.cpt_div
                                     ? kFastMenu[variant].alpha.cpt_div
                                     : kFastMenu[variant].beta.cpt_div);
        return vector_fits(g, eb, widest < eb ? eb : widest);
    }
    const TmaConfig c = kTmaMenu[variant - kRegisterVariants];
    const int elem = storage_elem_bytes(storage);
    if (!default_layout(g, elem)) return false;  // the bulk-copy kernels run on the default layout only
    int dev = 0, max_optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return false;
    const size_t stage = (size_t)Q * c.rows * g.P * elem;
    // 1 KiB left for the kernel's static shared memory
    return (size_t)c.stages * stage + 2 * (size_t)c.stages * sizeof(uint64_t) + 16 + 1024 <= (size_t)max_optin;
}

void fast_variant_shape(int storage, int variant, bool alpha, int nx, int& cpt, int& block)
{
    if (variant >= kRegisterVariants) {
        const TmaConfig c = kTmaMenu[variant - kRegisterVariants];
        block = 32 * (1 + c.consumer_warps);
        cpt = (c.rows * nx + 32 * c.consumer_warps - 1) / (32 * c.consumer_warps);
        return;
    }
    const KernelShape k = alpha ? kFastMenu[variant].alpha : kFastMenu[variant].beta;
    const int V = 16 / storage_elem_bytes(storage);
    cpt = V / k.cpt_div > 0 ? V / k.cpt_div : 1;
    block = k.block;
}

cudaError_t launch_batch_step(int storage, int variant, bool alpha, const BatchArgs& a, cudaStream_t st)
{
    if (variant < 0 || variant >= kRegisterVariants) return cudaErrorInvalidValue;
    count_launch();
    switch (storage) {
    case 0: return launch_batch_f64(variant, alpha, a, st);
    case 1: return launch_batch_f32(variant, alpha, a, st);
    case 2: return launch_batch_f16s(variant, alpha, a, st);
    case 3: return launch_batch_bf16s(variant, alpha, a, st);
    case 4: return launch_batch_f16sr(variant, alpha, a, st);
    default: return cudaErrorInvalidValue;
    }
}

// Domain of every virtual block of kernel `which` (vb_dom[vb]), by binary
// search of the table's block_start; rebuilt whenever the table changes.
__global__ void __launch_bounds__(256) batch_map(const BatchDomain* __restrict__ doms, const int ndom,
                                                 const long long vblocks, const int which, int* __restrict__ vb_dom)
{
    for (long long vb = (long long)blockIdx.x * blockDim.x + threadIdx.x; vb < vblocks;
         vb += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = ndom - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (doms[mid].block_start[which] <= vb) lo = mid;
            else hi = mid - 1;
        }
        vb_dom[vb] = lo;
    }
}

cudaError_t launch_batch_map(const BatchDomain* doms, int ndom, long long vblocks, int which, int* vb_dom,
                             cudaStream_t st)
{
    if (vblocks <= 0 || ndom <= 0) return cudaSuccess;
    const long long want = (vblocks + 255) / 256;
    const int grid = (int)(want < 4096 ? want : 4096);
    count_launch();
    batch_map<<<grid, 256, 0, st>>>(doms, ndom, vblocks, which, vb_dom);
    return cudaGetLastError();
}

cudaError_t launch_fast_step(int storage, int variant, bool alpha, void* dd, const Grid& g, const Params& p,
                             int lid_y, int* err, cudaStream_t st)
{
    if (variant >= kRegisterVariants && variant < kFastVariantCount) {
        const TmaConfig c = kTmaMenu[variant - kRegisterVariants];
        cudaError_t e;
        switch (storage) {
        case 0:
        case kStorageF64Fma:
            e = launch_tma_f64(alpha, dd, g, p, lid_y, c.rows, c.stages, c.consumer_warps, err, st);
            break;
        case 1:
        case kStorageF32Fma:
            e = launch_tma_f32(alpha, dd, g, p, lid_y, c.rows, c.stages, c.consumer_warps, err, st);
            break;
        case 2: e = launch_tma_f16s(alpha, dd, g, p, lid_y, c.rows, c.stages, c.consumer_warps, err, st); break;
        case 3: e = launch_tma_bf16s(alpha, dd, g, p, lid_y, c.rows, c.stages, c.consumer_warps, err, st); break;
        case 4: e = launch_tma_f16sr(alpha, dd, g, p, lid_y, c.rows, c.stages, c.consumer_warps, err, st); break;
        default: return cudaErrorInvalidValue;
        }
        if (e == cudaSuccess) count_launch();
        return e;
    }
    count_launch();
    switch (storage) {
    case 0: return launch_fast_f64(variant, alpha, dd, g, p, lid_y, st);
    case kStorageF64Fma: return launch_fast_f64fma(variant, alpha, dd, g, p, lid_y, st);
    case 1: return launch_fast_f32(variant, alpha, dd, g, p, lid_y, st);
    case kStorageF32Fma: return launch_fast_f32fma(variant, alpha, dd, g, p, lid_y, st);
    case 2: return launch_fast_f16s(variant, alpha, dd, g, p, lid_y, st);
    case 3: return launch_fast_bf16s(variant, alpha, dd, g, p, lid_y, st);
    case 4: return launch_fast_f16sr(variant, alpha, dd, g, p, lid_y, st);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_general_step(int storage, bool alpha, void* dd, const uint8_t* flags, const Grid& g,
                                const Params& p, int3 o, int3 s, cudaStream_t st)
{
    const long long n = (long long)s.x * s.y * s.z;
    const int blocks = grid_for(n, 128);
    const bool gravity = p.gx != 0.0 || p.gy != 0.0 || p.gz != 0.0;
    count_launch();
    return with_storage(storage, [&](auto tag) {
        using St = decltype(tag);
        auto* d = static_cast<typename St::bits*>(dd);
        if (alpha && gravity) alpha_general<St, true><<<blocks, 128, 0, st>>>(d, flags, g, p, o, s);
        else if (alpha) alpha_general<St, false><<<blocks, 128, 0, st>>>(d, flags, g, p, o, s);
        else beta_general<St><<<blocks, 128, 0, st>>>(d, flags, g, p, o, s);
        return cudaGetLastError();
    });
}

cudaError_t launch_macros(int storage, const void* dd, const uint8_t* flags, const Grid& g, bool last_alpha,
                          double lid_u, void* out, cudaStream_t st)
{
    count_launch();
    return with_storage(storage, [&](auto tag) {
        using St = decltype(tag);
        using T = typename St::T;
        compute_macros<St><<<grid_for(g.cells(), 256, 8192), 256, 0, st>>>(
            static_cast<const typename St::bits*>(dd), flags, g, last_alpha, T(lid_u), static_cast<T*>(out));
        return cudaGetLastError();
    });
}

cudaError_t launch_macros_cavity(int storage, const void* dd, const Grid& g, bool last_alpha, double lid_u,
                                 void* out, cudaStream_t st)
{
    count_launch();
    return with_storage(storage, [&](auto tag) {
        using St = decltype(tag);
        using T = typename St::T;
        compute_macros_cavity<St><<<grid_for((long long)g.nx * g.ny * g.nz, 256, 8192), 256, 0, st>>>(
            static_cast<const typename St::bits*>(dd), g, last_alpha, T(lid_u), static_cast<T*>(out));
        return cudaGetLastError();
    });
}

int reduce_blocks(const Grid& g)
{
    return grid_for((long long)g.nx * g.ny * g.nz, kReduceBlock, kReduceMaxBlocks);
}

cudaError_t launch_reduce(int storage, const void* dd, const uint8_t* flags, const Grid& g, bool last_alpha,
                          double* partials, double* out, cudaStream_t st)
{
    const int blocks = reduce_blocks(g);
    cudaError_t e = with_storage(storage, [&](auto tag) {
        using St = decltype(tag);
        reduce_partials<St><<<blocks, kReduceBlock, 0, st>>>(static_cast<const typename St::bits*>(dd), flags,
                                                              g, last_alpha, partials);
        return cudaGetLastError();
    });
    if (e != cudaSuccess) return e;
    reduce_final<<<1, 32, 0, st>>>(partials, blocks, out);
    count_launch(2);
    return cudaGetLastError();
}

cudaError_t launch_pack_slot(int storage, const void* dd, const Grid& g, int k, int3 o, int3 s, float* out,
                             cudaStream_t st)
{
    const long long rows = (long long)s.y * s.z;
    count_launch();
    return with_storage(storage, [&](auto tag) {
        using St = decltype(tag);
        pack_slot<St><<<grid_for(rows, 1, 65536), 256, 0, st>>>(static_cast<const typename St::bits*>(dd), g, k,
                                                                 o, s, out);
        return cudaGetLastError();
    });
}

cudaError_t launch_unpack_slot(int storage, void* dd, const Grid& g, int k, int3 o, int3 s, const float* in,
                               cudaStream_t st)
{
    const long long rows = (long long)s.y * s.z;
    count_launch();
    return with_storage(storage, [&](auto tag) {
        using St = decltype(tag);
        unpack_slot<St><<<grid_for(rows, 1, 65536), 256, 0, st>>>(static_cast<typename St::bits*>(dd), g, k, o,
                                                                   s, in);
        return cudaGetLastError();
    });
}

}  // namespace lbm
