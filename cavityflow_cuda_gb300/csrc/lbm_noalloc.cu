// lbm_noalloc.cu -- the FP64 mass/momentum reduction for callers that cannot
// allocate device memory.
//
// Some callers cannot call cudaMalloc: a host program whose device memory is
// entirely handed out by its own pool or caching allocator (a framework
// allocator, or a serving engine that admits work against a fixed HBM
// budget and must not grow past it behind its back), and a time loop that
// cannot afford the implicit device synchronisation cudaMalloc and cudaFree
// may cause.  lbm_reduce_noalloc serves them: it reduces population and flag
// arrays the caller already owns, in the reference's own layout, and writes
// the four totals to a device buffer the caller owns.  Its only scratch is
// the file-scope array below, which every GPU that loads this library holds
// until the process exits.
#include <cstdint>
#include <mutex>

#include "../../include/lbm_gb300.h"
#include "lbm_core.cuh"
#include "lbm_kernels.h"

namespace lbm {

// One row of partial sums (mass, momentum x, y, z) per z plane.
constexpr int kNoAllocMaxPlanes = 4096;  // 4096 planes x 4 doubles = 128 KiB per device
constexpr int kNoAllocBlock = 256;

static __device__ __align__(256) double g_noalloc_partials[kNoAllocMaxPlanes * 4];

// Pass 1: block b sums interior plane z = b + 1 of a reference-layout domain
// ((nx+2)*(ny+2)*(nz+2) cells per slot, x fastest, int32 flags).  Same sums
// as reduce_partials: mass of every live slot, momentum of the post-collision
// populations.  Every call writes all nz rows it later reads, so nothing in
// the scratch needs clearing first.
template <typename T>
__global__ void __launch_bounds__(kNoAllocBlock) noalloc_plane_sums(const T* __restrict__ dd,
                                                                    const int32_t* __restrict__ flags, int nx,
                                                                    int ny, int nz, bool last_alpha,
                                                                    double* __restrict__ partials)
{
    const long long X = nx + 2, XY = X * (ny + 2), C = XY * (nz + 2);
    const int z = blockIdx.x + 1;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const long long cells = (long long)nx * ny;  // 64-bit: i + kNoAllocBlock never wraps
    for (long long i = threadIdx.x; i < cells; i += kNoAllocBlock) {
        const long long x = 1 + i % nx, y = 1 + i / nx;
        const long long gid = z * XY + y * X + x;
        const int32_t fl = flags[gid];
        if (fl != kFluid && fl != kInjection) continue;
        double m = 0.0, px = 0.0, py = 0.0, pz = 0.0;
#pragma unroll
        for (int k = 0; k < Q; ++k) {
            const long long nb = gid + dir_x(k) + dir_y(k) * X + dir_z(k) * XY;
            const int32_t fn = flags[nb];
            m += (double)dd[k * C + gid];
            if (fn != kFluid && fn != kInjection) m += (double)dd[k * C + nb];
            const double f = (double)(last_alpha ? dd[opp(k) * C + gid] : dd[k * C + nb]);
            px += dir_x(k) * f;
            py += dir_y(k) * f;
            pz += dir_z(k) * f;
        }
        acc[0] += m; acc[1] += px; acc[2] += py; acc[3] += pz;
    }
    __shared__ double warp_sums[kNoAllocBlock / 32][4];
#pragma unroll
    for (int q = 0; q < 4; ++q)
        for (int off = 16; off > 0; off >>= 1) acc[q] += __shfl_down_sync(0xffffffffu, acc[q], off);
    if ((threadIdx.x & 31) == 0)
        for (int q = 0; q < 4; ++q) warp_sums[threadIdx.x >> 5][q] = acc[q];
    __syncthreads();
    if (threadIdx.x < 4) {
        double s = 0.0;
        for (int w = 0; w < kNoAllocBlock / 32; ++w) s += warp_sums[w][threadIdx.x];
        partials[(z - 1) * 4 + threadIdx.x] = s;
    }
}

// Pass 2: the planes in order, one thread per total.
__global__ void noalloc_total(const double* __restrict__ partials, int nz, double* __restrict__ out)
{
    if (threadIdx.x < 4) {
        double s = 0.0;
        for (int z = 0; z < nz; ++z) s += partials[z * 4 + threadIdx.x];
        out[threadIdx.x] = s;
    }
}

}  // namespace lbm

namespace {

// The driver calls that name the current context, resolved through the
// runtime (the library links no driver library).
using CtxGetCurrentFn = int (*)(void**);
using CtxGetIdFn = int (*)(void*, unsigned long long*);

// Device address of g_noalloc_partials in the CURRENT context.  In host code
// the array's name is only a host-side stand-in, so the kernels receive this
// address instead.  The array is instantiated once per context (a
// cudaDeviceReset, or a caller's own driver context, gives a new one at a
// new address), so the address is cached by the context's unique id: the
// first call in each context -- for the usual caller, the first call on each
// device, in its primary context -- does the lookup.
int scratch_address(double** out)
{
    static std::mutex mu;
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    struct Entry {
        unsigned long long ctx_id;
        double* addr;
    };
    static Entry cache[64];
    static int used = 0;
    static int next = 0;

    cudaError_t e = cudaSuccess;
    std::lock_guard<std::mutex> lock(mu);
    if (!get_current || !get_id) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
        e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
        if (e == cudaSuccess) e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
        if (e != cudaSuccess || q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return lbm::record_error(LBM_ERR_CUDA, "lbm_reduce_noalloc: driver context queries unavailable");
        get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
        get_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    void* ctx = nullptr;
    void* p = nullptr;
    if (get_current(&ctx) != 0) return lbm::record_error(LBM_ERR_CUDA, "lbm_reduce_noalloc: cuCtxGetCurrent failed");
    if (!ctx) {
        // No context current on this thread yet: the runtime's symbol lookup
        // initialises the current device's primary context and makes it current.
        e = cudaGetSymbolAddress(&p, lbm::g_noalloc_partials);
        if (e != cudaSuccess)
            return lbm::record_error(LBM_ERR_CUDA, "lbm_reduce_noalloc: cudaGetSymbolAddress: %s",
                                     cudaGetErrorString(e));
        if (get_current(&ctx) != 0 || !ctx)
            return lbm::record_error(LBM_ERR_CUDA, "lbm_reduce_noalloc: no current CUDA context");
    }
    unsigned long long id = 0;
    if (get_id(ctx, &id) != 0) return lbm::record_error(LBM_ERR_CUDA, "lbm_reduce_noalloc: cuCtxGetId failed");
    for (int i = 0; i < used; ++i)
        if (cache[i].ctx_id == id) {
            *out = cache[i].addr;
            return LBM_OK;
        }
    if (!p) {
        e = cudaGetSymbolAddress(&p, lbm::g_noalloc_partials);
        if (e != cudaSuccess)
            return lbm::record_error(LBM_ERR_CUDA, "lbm_reduce_noalloc: cudaGetSymbolAddress: %s",
                                     cudaGetErrorString(e));
    }
    // context ids are never reused, so an evicted entry is only looked up again
    const int slot = used < 64 ? used++ : (next++ & 63);
    cache[slot] = {id, static_cast<double*>(p)};
    *out = static_cast<double*>(p);
    return LBM_OK;
}

}  // namespace

extern "C" int lbm_reduce_noalloc(const void* populations, const int32_t* flags, const int32_t size[3],
                                  int32_t storage, int32_t last_step_was_alpha, double* out_device, void* stream)
{
    if (!populations || !flags || !size || !out_device)
        return lbm::record_error(LBM_ERR_INVALID_ARGUMENT, "lbm_reduce_noalloc: NULL argument");
    if (storage != LBM_STORAGE_F64 && storage != LBM_STORAGE_F32)
        return lbm::record_error(LBM_ERR_UNSUPPORTED, "lbm_reduce_noalloc: storage must be F64 or F32");
    const int nx = size[0], ny = size[1], nz = size[2];
    if (nx <= 0 || ny <= 0 || nz <= 0 || (long long)nx * ny > (1LL << 31) - 1)
        return lbm::record_error(LBM_ERR_INVALID_ARGUMENT, "lbm_reduce_noalloc: bad domain size (%d, %d, %d)", nx,
                                 ny, nz);
    if (nz > lbm::kNoAllocMaxPlanes)
        return lbm::record_error(LBM_ERR_INVALID_ARGUMENT,
                                 "lbm_reduce_noalloc: nz = %d exceeds the %d-plane limit of its static scratch", nz,
                                 lbm::kNoAllocMaxPlanes);
    double* partials = nullptr;
    if (int r = scratch_address(&partials)) return r;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const bool la = last_step_was_alpha != 0;
    if (storage == LBM_STORAGE_F64)
        lbm::noalloc_plane_sums<double><<<nz, lbm::kNoAllocBlock, 0, st>>>(static_cast<const double*>(populations),
                                                                          flags, nx, ny, nz, la, partials);
    else
        lbm::noalloc_plane_sums<float><<<nz, lbm::kNoAllocBlock, 0, st>>>(static_cast<const float*>(populations),
                                                                         flags, nx, ny, nz, la, partials);
    lbm::noalloc_total<<<1, 32, 0, st>>>(partials, nz, out_device);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return lbm::record_error(LBM_ERR_CUDA, "lbm_reduce_noalloc launch: %s", cudaGetErrorString(e));
    lbm::add_launches(2);
    return LBM_OK;
}
