// lbm_tma.cuh -- row-pipelined A-A step kernels built on the Blackwell bulk
// copy engine (cp.async.bulk + mbarrier).
//
// Work unit: R consecutive interior rows (y0 .. y0+R-1) of one z plane.  In
// the A-A pattern every slot row a unit touches is owned by that unit alone:
//   alpha  slot k, rows y0.. of plane z           (own cells, swapped slots)
//   beta   slot k, rows y0+c_y.. of plane z+c_z   (the neighbours in +c_k)
// and every position of such a row (halo columns and padding included) is
// owned by a cell of the unit's rows, or by a halo cell nobody processes.
// So each slot of a unit moves as one contiguous bulk copy (R rows x P
// columns) in, and one bulk copy out, with no partial rows and no races.
//
// CTA = 1 producer warp + C consumer warps.  The producer's elected thread
// streams the CTA's units into a ring of `stages` shared-memory buffers (19
// slots x R rows x P elements each), signalling mbarrier `full` with the
// byte count.  The consumers wait for a buffer, collide every interior cell
// of it in place (alpha: population k to slot opp(k); beta: pull from and
// push to column x + c_x of slot k's row) and arrive on mbarrier `done`, one
// arrival per warp.  The producer then bulk-stores the 19 rows back and, as
// soon as the store engine has read the buffer, refills it with the unit
// `stages` ahead, so up to stages - 1 units load while one is collided.  The
// collision is the same arithmetic as the other kernels (lbm_core.cuh), so
// results are bit-identical.
//
// Every wait on an mbarrier is bounded (about two seconds of %globaltimer);
// on expiry the kernel raises an error flag, drains what it has in flight
// (again bounded) and returns, so a stalled copy can never hang the GPU.
#pragma once

#include <cstdint>

#include "lbm_core.cuh"

namespace lbm {

namespace tma {

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t now_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s

// Waits until the phase with `parity` of `bar` has completed; false if the
// time limit (nanoseconds) passes first.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint64_t limit_ns = kWaitLimitNs)
{
    if (mbar_test(bar, parity)) return true;
    const uint64_t deadline = now_ns() + limit_ns;
    for (;;) {
        if (mbar_test(bar, parity)) return true;
        if (now_ns() > deadline) return false;
        __nanosleep(64);
    }
}

__device__ __forceinline__ void bulk_load(void* smem_dst, const void* gmem_src, uint32_t bytes, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(smem_dst)),
        "l"(gmem_src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void bulk_store(void* gmem_dst, const void* smem_src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gmem_dst),
                 "r"(smem_addr(smem_src)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

template <int N>
__device__ __forceinline__ void bulk_wait_read()
{
    asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void consumer_barrier(int nthreads)
{
    asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
}

}  // namespace tma

// Bytes of dynamic shared memory a launch needs.
inline size_t tma_smem_bytes(const Grid& g, int elem_bytes, int rows, int stages)
{
    const size_t stage = (size_t)Q * rows * g.P * elem_bytes;
    return (size_t)stages * stage + 2 * (size_t)stages * sizeof(uint64_t) + 16;
}

constexpr int kTmaMaxThreads = 32 * 17;  // producer warp + up to 16 consumer warps

template <class St, bool kAlpha>
__global__ void __launch_bounds__(kTmaMaxThreads) step_tma(typename St::bits* __restrict__ dd, const Grid g,
                                                           const typename St::T inv_tau,
                                                           const typename St::T lid_u, const int lid_y,
                                                           const int wall_y,
                                                           const int R, const int stages, int* __restrict__ err,
                                                           const uint32_t* __restrict__ step_base,
                                                           const uint32_t step_off)
{
    using T = typename St::T;
    using bits = typename St::bits;
    const uint32_t step = step_of<St>(step_base, step_off);
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const unsigned slot_elems = (unsigned)(R * g.P);          // one slot of a buffer
    const unsigned stage_elems = (unsigned)Q * slot_elems;    // one buffer
    bits* buf = reinterpret_cast<bits*>(smem_raw);
    const size_t bar_off = ((size_t)stages * stage_elems * sizeof(bits) + 15) & ~(size_t)15;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw + bar_off);  // producer -> consumers: data landed
    uint64_t* done = full + stages;                                     // consumers -> producer: collided

    const int nyb = (g.ny + R - 1) / R;
    const long long units = (long long)nyb * g.nz;
    // this CTA's units: blockIdx.x, blockIdx.x + gridDim.x, ...
    const long long mine = units > blockIdx.x ? (units - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const int warp = threadIdx.x >> 5;
    const int nwarps_c = (int)(blockDim.x >> 5) - 1;

    if (threadIdx.x == 0) {
        for (int s = 0; s < stages; ++s) {
            tma::mbar_init(&full[s], 1);
            tma::mbar_init(&done[s], nwarps_c);
        }
        tma::fence_mbar_init();
    }
    __syncthreads();

    auto unit_rows = [&](long long i, int& z, int& y0, int& rn) {
        const long long u = blockIdx.x + i * gridDim.x;
        z = 1 + (int)(u / nyb);
        y0 = 1 + (int)(u % nyb) * R;
        rn = min(R, g.ny - y0 + 1);
    };

    if (warp == 0) {
        // ---------------- producer: loads, and stores once collided ----------------
        if (threadIdx.x != 0) return;
        auto issue_loads = [&](long long i, int s) {
            int z, y0, rn;
            unit_rows(i, z, y0, rn);
            const uint32_t bytes = (uint32_t)(rn * g.P * (long long)sizeof(bits));
            tma::mbar_arrive_expect_tx(&full[s], bytes * Q);
            bits* dst = buf + (size_t)s * stage_elems;
#pragma unroll 1
            for (int k = 0; k < Q; ++k) {
                const int yy = kAlpha ? y0 : y0 + dir_y(k);
                const int zz = kAlpha ? z : z + dir_z(k);
                tma::bulk_load(dst + (size_t)k * slot_elems, dd + k * g.S + (long long)zz * g.PY + (long long)yy * g.P,
                               bytes, &full[s]);
            }
        };
        long long i = 0;
        for (; i < mine && i < stages; ++i) issue_loads(i, (int)i);
        bool failed = false;
        for (i = 0; i < mine; ++i) {
            const int s = (int)(i % stages);
            if (!tma::mbar_wait(&done[s], (uint32_t)(i / stages) & 1u)) {
                failed = true;
                break;
            }
            int z, y0, rn;
            unit_rows(i, z, y0, rn);
            const uint32_t bytes = (uint32_t)(rn * g.P * (long long)sizeof(bits));
            const bits* src = buf + (size_t)s * stage_elems;
#pragma unroll 1
            for (int k = 0; k < Q; ++k) {
                const int yy = kAlpha ? y0 : y0 + dir_y(k);
                const int zz = kAlpha ? z : z + dir_z(k);
                tma::bulk_store(dd + k * g.S + (long long)zz * g.PY + (long long)yy * g.P, src + (size_t)k * slot_elems,
                                bytes);
            }
            tma::bulk_commit();
            if (i + stages < mine) {
                tma::bulk_wait_read<0>();  // the store engine has read the buffer: refill it
                issue_loads(i + stages, s);
            }
        }
        if (failed) {
            atomicOr(err, 1);
            // let loads already issued land before the CTA's shared memory goes away
            for (long long j = i; j < mine && j < i + stages; ++j)
                tma::mbar_wait(&full[j % stages], (uint32_t)(j / stages) & 1u);
        }
        tma::bulk_wait_all();
        return;
    }

    // ---------------- consumers: collide in shared memory ----------------
    const int ctid = (int)threadIdx.x - 32;
    const int nconsumer = nwarps_c * 32;
    const int lane = threadIdx.x & 31;
    const T rho0 = St::shifted ? T(0) : T(1);
    const T du = wall_shift<St>(lid_u);
    for (long long i = 0; i < mine; ++i) {
        const int s = (int)(i % stages);
        const uint32_t parity = (uint32_t)(i / stages) & 1u;
        // lane 0 waits (bounded) and the warp follows its decision, so that no
        // lane can leave while the others reach __syncwarp below
        int ok = 1;
        if (lane == 0) ok = tma::mbar_wait(&full[s], parity) ? 1 : 0;
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) {
            if (lane == 0) atomicOr(err, 2);
            break;
        }
        tma::mbar_test(&full[s], parity);  // phase already complete: this lane's acquire of the data
        int z, y0, rn;
        unit_rows(i, z, y0, rn);
        bits* sb = buf + (size_t)s * stage_elems;
        for (int r = 0; r < rn; ++r) {
            const bool lid = (y0 + r == lid_y);
            const bool wall = (y0 + r == wall_y);
            for (int x = 1 + ctid; x <= g.nx; x += nconsumer) {
                const unsigned col = (unsigned)(r * g.P + x + g.xoff);
                T f[Q];
                if constexpr (kAlpha) {
#pragma unroll
                    for (int k = 0; k < Q; ++k) f[k] = St::load_step(sb[k * slot_elems + col]);
                    if (wall) wall_correct(f, du);
                    if (lid) inject_step<St>(f, rho0, lid_u);
                    else collide<St>(f, inv_tau);
                    uint32_t h = 0;
                    if constexpr (St::stochastic) h = sr_cell(sr_hash((uint32_t)g.ref(0, y0 + r, z), step), x);
#pragma unroll
                    for (int k = 0; k < Q; ++k) sb[opp(k) * slot_elems + col] = store_pop<St>(f[k], h, k);
                } else {
#pragma unroll
                    for (int k = 0; k < Q; ++k) f[opp(k)] = St::load_step(sb[k * slot_elems + col + dir_x(k)]);
                    if (wall) wall_correct(f, du);
                    if (lid) inject_step<St>(f, rho0, lid_u);
                    else collide<St>(f, inv_tau);
                    uint32_t h = 0;
                    if constexpr (St::stochastic) h = sr_cell(sr_hash((uint32_t)g.ref(0, y0 + r, z), step), x);
#pragma unroll
                    for (int k = 0; k < Q; ++k) sb[k * slot_elems + col + dir_x(k)] = store_pop<St>(f[k], h, k);
                }
            }
        }
        tma::fence_proxy_async();  // this thread's writes, before the store engine reads them
        __syncwarp();
        if (lane == 0) tma::mbar_arrive(&done[s]);
    }
}

}  // namespace lbm

namespace lbm {

// Launch of the row-pipelined kernels for storage St: R rows per unit,
// `stages` buffers, C consumer warps, one persistent wave of CTAs.
// Returns cudaErrorInvalidValue when the configuration does not fit.
template <class St>
cudaError_t launch_tma_impl(bool alpha, void* dd, const Grid& g, const Params& p, int lid_y, int R, int stages,
                            int C, int* err, cudaStream_t st)
{
    using T = typename St::T;
    using bits = typename St::bits;
    if (R < 1 || stages < 1 || C < 1 || C > 16) return cudaErrorInvalidValue;
    const size_t smem = tma_smem_bytes(g, (int)sizeof(bits), R, stages);
    int dev = 0, max_optin = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    auto kern = alpha ? step_tma<St, true> : step_tma<St, false>;
    cudaFuncAttributes attr;
    e = cudaFuncGetAttributes(&attr, kern);
    if (e != cudaSuccess) return e;
    // the dynamic allowance plus the kernel's static shared memory must stay
    // within the per-block opt-in limit
    const int dyn_max = max_optin - (int)attr.sharedSizeBytes;
    if (dyn_max <= 0 || smem > (size_t)dyn_max) return cudaErrorInvalidValue;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_max);
    if (e != cudaSuccess) return e;
    const int threads = 32 * (1 + C);
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidValue;
    const long long units = (long long)((g.ny + R - 1) / R) * g.nz;
    const long long grid = units < (long long)per_sm * sms ? units : (long long)per_sm * sms;
    kern<<<(int)grid, threads, smem, st>>>(static_cast<bits*>(dd), g, T(p.inv_tau), T(p.lid_u), lid_y, p.wall_y, R, stages,
                                          err, p.step_base, p.step_off);
    return cudaGetLastError();
}

}  // namespace lbm
