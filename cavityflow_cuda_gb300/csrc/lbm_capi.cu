// lbm_capi.cu -- the C ABI (include/lbm_gb300.h) over the sm_103a kernels.
//
// One lbm_solver owns one domain on one device: the padded SoA population
// array, a one-byte flag array in the reference layout, a lazily allocated
// macroscopic-field array for the velocity/density getters, reduction
// scratch, and a CUDA graph of captured alpha/beta pairs for long runs.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <new>
#include <vector>

#include "../../include/lbm_gb300.h"
#include "lbm_internal.h"
#include "lbm_kernels.h"

using lbm::Grid;

namespace {

thread_local char t_err[512] = "";

}  // namespace

namespace lbm_detail {

int fail(int status, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_err, sizeof(t_err), fmt, ap);
    va_end(ap);
    return status;
}

int cuda_fail(cudaError_t e, const char* what)
{
    if (e == cudaErrorMemoryAllocation)
        return fail(LBM_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
    return fail(LBM_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

}  // namespace lbm_detail

using namespace lbm_detail;

int lbm::record_error(int status, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_err, sizeof(t_err), fmt, ap);
    va_end(ap);
    return status;
}

namespace {

#define CK(call, what)                                   \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

}  // namespace

int lbm_detail::elem_bytes(int storage) { return storage == LBM_STORAGE_F64 ? 8 : storage == LBM_STORAGE_F32 ? 4 : 2; }
int lbm_detail::value_bytes(int storage) { return storage == LBM_STORAGE_F64 ? 8 : 4; }

namespace {

bool valid_flag(int32_t f)
{
    return f == LBM_OBSTACLE || f == LBM_FLUID || f == LBM_VELOCITY_INJECTION || f == LBM_GHOST_LAYER;
}

constexpr int kGraphPairs = 32;  // alpha/beta pairs per captured graph

// Default launch variant per storage (index into kFastMenu), from kernel
// timings of the 384^3 cavity on GB300: two-warp blocks; FP32 with 8-byte
// vectors in both kernels and beta's shifted windows accessed directly (no
// exchange), FP16 (both roundings) with a 16-byte alpha and an 8-byte direct
// beta, BF16 with 16-byte vectors and the block-wide beta exchange.  FP64 is
// bound by FP64 arithmetic, where the shapes tie; it keeps 8-byte vectors
// (one cell).
}  // namespace

// Batch and server rows are packed for 8-byte vectors (kPackedX1Align), so
// their variants use 8-byte (or narrower) vectors in both kernels.  On the
// seeded 512-cavity workload the direct beta windows in two-warp blocks
// (variant 13) are fastest for FP32, the packed 16-bit beta at <= 128
// registers (22: the batch kernel's own state spills the 102-register
// shape) for the 16-bit storages, the FP64 warp exchange (3) for FP64.
int lbm_detail::default_batch_variant(int storage)
{
    switch (storage) {
    case LBM_STORAGE_F64: return 3;
    case LBM_STORAGE_F16S:
    case LBM_STORAGE_BF16S:
    case LBM_STORAGE_F16SR: return 22;
    default: return 13;
    }
}

int lbm_detail::default_variant(int storage)
{
    switch (storage) {
    case LBM_STORAGE_F32: return 13;
    case LBM_STORAGE_F16S: return 20;
    case LBM_STORAGE_BF16S: return 20;
    case LBM_STORAGE_F16SR: return 20;
    default: return 3;
    }
}

namespace {


}  // namespace





int* lbm_detail::err_flag(lbm_solver* s) { return reinterpret_cast<int*>(s->counts + 2); }
uint32_t* lbm_detail::step_words(lbm_solver* s) { return reinterpret_cast<uint32_t*>(s->counts + 4); }

// Reads and clears the kernels' timeout flag after the device is idle.
int lbm_detail::check_kernel_flag(lbm_solver* s)
{
    int flag = 0;
    CK(cudaMemcpy(&flag, err_flag(s), sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy error flag");
    if (flag) {
        CK(cudaMemset(err_flag(s), 0, sizeof(int)), "cudaMemset error flag");
        return fail(LBM_ERR_TIMEOUT, "a step kernel gave up waiting for its bulk copies (flag %d)", flag);
    }
    return LBM_OK;
}

namespace {

int check_solver(const lbm_solver* s)
{
    if (!s) return fail(LBM_ERR_INVALID_ARGUMENT, "solver is NULL");
    return LBM_OK;
}

// Resolves a cuboid argument pair; NULL/NULL is the interior.  Bounds as the
// reference asserts them (src/CLbmSolverGPU.cu:255-259).
int resolve_cuboid(const lbm_solver* s, const int32_t* origin, const int32_t* size, int3& o, int3& n)
{
    if ((origin == nullptr) != (size == nullptr))
        return fail(LBM_ERR_INVALID_ARGUMENT, "origin and size must both be given or both be NULL");
    if (!origin) {
        o = make_int3(1, 1, 1);
        n = make_int3(s->g.nx, s->g.ny, s->g.nz);
        return LBM_OK;
    }
    const int lim[3] = {s->g.nx + 2, s->g.ny + 2, s->g.nz + 2};
    for (int d = 0; d < 3; ++d) {
        if (origin[d] < 0 || size[d] <= 0 || (int64_t)origin[d] + size[d] > lim[d])
            return fail(LBM_ERR_OUT_OF_BOUNDS, "cuboid origin (%d,%d,%d) size (%d,%d,%d) outside (%d,%d,%d)",
                        origin[0], origin[1], origin[2], size[0], size[1], size[2], lim[0], lim[1], lim[2]);
    }
    o = make_int3(origin[0], origin[1], origin[2]);
    n = make_int3(size[0], size[1], size[2]);
    return LBM_OK;
}

void drop_graph(lbm_solver* s)
{
    if (s->graph) {
        cudaGraphExecDestroy(s->graph);
        s->graph = nullptr;
    }
}

// Decides between the vectorised kernels (flags are the box cavity with an
// all-obstacle halo, with or without the lid plane y = ny) and the
// flag-array kernels.  Gravity needs the flag-array alpha kernel.
int refresh_path(lbm_solver* s)
{
    drop_graph(s);
    CK(cudaMemsetAsync(s->counts, 0, 2 * sizeof(unsigned long long), 0), "cudaMemsetAsync");
    CK(lbm::launch_check_cavity(s->flags, s->g, s->counts, 0), "check_cavity_flags launch");
    unsigned long long h[2];
    CK(cudaMemcpy(h, s->counts, sizeof(h), cudaMemcpyDeviceToHost), "cudaMemcpy counts");
    const bool gravity = s->p.gx != 0.0 || s->p.gy != 0.0 || s->p.gz != 0.0;
    if (gravity) s->lid_y = -1;
    else if (h[0] == 0) s->lid_y = s->g.ny;
    else if (h[1] == 0) s->lid_y = 0;
    else s->lid_y = -1;
    return LBM_OK;
}

// Storage code of the vectorised step kernels: FP64 and FP32 with fused
// multiply-adds have kernel families of their own (lbm::kStorageF64Fma,
// lbm::kStorageF32Fma).
int kernel_storage(const lbm_solver* s)
{
    if (!s->fma) return s->storage;
    return s->storage == LBM_STORAGE_F64 ? lbm::kStorageF64Fma : lbm::kStorageF32Fma;
}

int step(lbm_solver* s, bool alpha, const int32_t* origin, const int32_t* size, cudaStream_t st)
{
    int3 o, n;
    cudaError_t e;
    lbm::Params p = s->p;  // this step's stochastic-rounding key
    p.step_base = step_words(s) + 1;
    p.step_off = (uint32_t)s->counter;
    if (!origin && s->lid_y >= 0) {
        e = lbm::launch_fast_step(kernel_storage(s), s->variant, alpha, s->dd, s->g, p, s->lid_y, err_flag(s), st);
    } else {
        if (origin) {
            int r = resolve_cuboid(s, origin, size, o, n);
            if (r) return r;
        } else {
            o = make_int3(0, 0, 0);
            n = make_int3(s->g.nx + 2, s->g.ny + 2, s->g.nz + 2);
        }
        e = lbm::launch_general_step(s->storage, alpha, s->dd, s->flags, s->g, p, o, n, st);
    }
    if (e != cudaSuccess) return cuda_fail(e, alpha ? "alpha step launch" : "beta step launch");
    s->counter += 1;
    s->last_alpha = alpha;
    s->macros_fresh = false;
    return LBM_OK;
}

int ensure_macros(lbm_solver* s)
{
    CK(cudaSetDevice(s->device), "cudaSetDevice");
    if (!s->macros) {
        const size_t bytes = (size_t)4 * s->g.cells() * value_bytes(s->storage);
        CK(cudaMalloc(&s->macros, bytes), "cudaMalloc macros");
        s->device_bytes += (int64_t)bytes;
        s->macros_fresh = false;
    }
    if (!s->macros_fresh) {
        CK(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
        if (int r = check_kernel_flag(s)) return r;
        CK(lbm::launch_macros(s->storage, s->dd, s->flags, s->g, s->last_alpha, s->p.lid_u, s->macros, 0),
           "compute_macros launch");
        CK(cudaDeviceSynchronize(), "compute_macros");
        s->macros_fresh = true;
    }
    return LBM_OK;
}

// Synchronous cuboid copy between a compact reference-layout device array
// (x extent nx+2) and a packed host buffer.
cudaError_t copy_compact(void* dev, size_t elem, const Grid& g, int3 o, int3 n, void* host, bool to_host)
{
    cudaMemcpy3DParms m = {};
    cudaPitchedPtr dptr = make_cudaPitchedPtr(dev, (size_t)(g.nx + 2) * elem, (size_t)(g.nx + 2), (size_t)(g.ny + 2));
    cudaPitchedPtr hptr = make_cudaPitchedPtr(host, (size_t)n.x * elem, (size_t)n.x, (size_t)n.y);
    if (to_host) {
        m.srcPtr = dptr;
        m.srcPos = make_cudaPos((size_t)o.x * elem, (size_t)o.y, (size_t)o.z);
        m.dstPtr = hptr;
        m.kind = cudaMemcpyDeviceToHost;
    } else {
        m.srcPtr = hptr;
        m.dstPtr = dptr;
        m.dstPos = make_cudaPos((size_t)o.x * elem, (size_t)o.y, (size_t)o.z);
        m.kind = cudaMemcpyHostToDevice;
    }
    m.extent = make_cudaExtent((size_t)n.x * elem, (size_t)n.y, (size_t)n.z);
    return cudaMemcpy3D(&m);
}

// Asynchronous cuboid copy of one population slot between the padded device
// layout and a packed host buffer (F64/F32 storage).
cudaError_t copy_slot(lbm_solver* s, int k, int3 o, int3 n, void* host, bool to_host, cudaStream_t st)
{
    const size_t elem = (size_t)elem_bytes(s->storage);
    char* base = static_cast<char*>(s->dd) + (size_t)k * s->g.S * elem;
    cudaMemcpy3DParms m = {};
    cudaPitchedPtr dptr = make_cudaPitchedPtr(base, (size_t)s->g.P * elem, (size_t)s->g.P, (size_t)(s->g.ny + 2));
    cudaPitchedPtr hptr = make_cudaPitchedPtr(host, (size_t)n.x * elem, (size_t)n.x, (size_t)n.y);
    const cudaPos dpos = make_cudaPos((size_t)(o.x + s->g.xoff) * elem, (size_t)o.y, (size_t)o.z);
    if (to_host) {
        m.srcPtr = dptr; m.srcPos = dpos; m.dstPtr = hptr; m.kind = cudaMemcpyDeviceToHost;
    } else {
        m.srcPtr = hptr; m.dstPtr = dptr; m.dstPos = dpos; m.kind = cudaMemcpyHostToDevice;
    }
    m.extent = make_cudaExtent((size_t)n.x * elem, (size_t)n.y, (size_t)n.z);
    return cudaMemcpy3DAsync(&m, st);
}

int ensure_staging(lbm_solver* s, size_t elems)
{
    if (s->staging_elems >= elems) return LBM_OK;
    if (s->staging) {
        cudaFree(s->staging);
        s->device_bytes -= (int64_t)(s->staging_elems * sizeof(float));
        s->staging = nullptr;
        s->staging_elems = 0;
    }
    CK(cudaMalloc(&s->staging, elems * sizeof(float)), "cudaMalloc staging");
    s->staging_elems = elems;
    s->device_bytes += (int64_t)(elems * sizeof(float));
    return LBM_OK;
}

// Slots copied by the direction-filtered set: those k with norm . e_k > 0
// (src/CLbmSolverGPU.cu:625-645, :686).
bool slot_selected(int direction, int k)
{
    if (direction == LBM_DIRECTION_ALL) return true;
    int nx = 0, ny = 0, nz = 0;
    switch (direction) {
    case LBM_LEFT: nx = 1; break;
    case LBM_RIGHT: nx = -1; break;
    case LBM_BOTTOM: ny = 1; break;
    case LBM_TOP: ny = -1; break;
    case LBM_BACK: nz = 1; break;
    case LBM_FRONT: nz = -1; break;
    default: return false;
    }
    return nx * lbm::dir_x(k) + ny * lbm::dir_y(k) + nz * lbm::dir_z(k) > 0;
}

// ---- parameter derivation (src/CLbmSolver.cpp:28-327) ----------------------
// Written with the reference's types: T is the working precision, and the
// constants below are double literals exactly as src/constants.h declares
// them, so the mixed float/double promotions of the original expressions are
// the same here.
constexpr double kReynoldsDefault = 1000.0;   // REYNOLDS_DEFAULT
constexpr double kTauDefault = 0.85;          // TAU_DEFAULT
constexpr double kTauLower = 0.51;            // TAU_LOWER_LIMIT
constexpr double kTauUpper = 1.9;             // TAU_UPPER_LIMIT

template <typename T>
T len3(const T v[3])
{
    const T s = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    return std::sqrt(s);
}

template <typename T>
int derive(const lbm_physical* in, lbm_lattice* out)
{
    const T eps = std::numeric_limits<T>::epsilon();
    const T vel[3] = {(T)in->velocity[0], (T)in->velocity[1], (T)in->velocity[2]};
    const T acc[3] = {(T)in->acceleration[0], (T)in->acceleration[1], (T)in->acceleration[2]};
    const T len[3] = {(T)in->domain_length[0], (T)in->domain_length[1], (T)in->domain_length[2]};
    const T maxVel = (T)in->max_velocity, maxAcc = (T)in->max_acceleration;
    T viscosity = (T)in->viscosity;
    T dt = (T)in->timestep;
    const T cellLength = len[0] / (T)in->domain_size[0];
    bool limitedByVelocity = false, limitedByAcceleration = false;
    T oldDt = dt, tau = 0, velDL[3], accDL[3], nuDL = 0;

    if (viscosity <= (T)0) {
        const T lmax = (len[0] > len[1] ? len[0] : len[1]);
        viscosity = (len[2] > lmax ? len[2] : lmax) * vel[0] / kReynoldsDefault;
    }
    // The reference loops until it finds a stable step or exits; this bound
    // is far above any sequence of rescalings it can take.
    for (int iter = 0;; ++iter) {
        if (iter > 1000) return fail(LBM_ERR_CONFIG, "time-step search did not settle");
        for (int d = 0; d < 3; ++d) velDL[d] = vel[d] * (dt / cellLength);
        for (int d = 0; d < 3; ++d) accDL[d] = acc[d] * ((dt * dt) / cellLength);
        nuDL = viscosity * (dt / (cellLength * cellLength));
        if (len3(velDL) > maxVel + eps) {
            limitedByVelocity = true;
            oldDt = dt;
            dt = (maxVel * cellLength) / len3(vel);
            continue;
        }
        if (len3(accDL) > maxAcc + eps) {
            limitedByAcceleration = true;
            oldDt = dt;
            dt = std::sqrt((maxAcc * cellLength) / len3(acc));
            continue;
        }
        tau = (T)0.5 * ((T)6 * nuDL + (T)1);
        if (tau - eps < (T)kTauLower || tau + eps > (T)kTauUpper) {
            oldDt = dt;
            dt = (cellLength * cellLength) * (((T)2 * kTauDefault - (T)1) / ((T)6 * viscosity));
            if ((limitedByVelocity || limitedByAcceleration) && dt > oldDt)
                return fail(LBM_ERR_CONFIG,
                            "no time step satisfies viscosity %g, max velocity %g, max acceleration %g (tau %g)",
                            (double)viscosity, (double)maxVel, (double)maxAcc, (double)tau);
            continue;
        }
        break;
    }
    out->timestep = dt;
    out->tau = tau;
    out->inv_tau = (T)1 / tau;
    for (int d = 0; d < 3; ++d) {
        out->velocity[d] = velDL[d];
        out->acceleration[d] = accDL[d];
    }
    out->viscosity = nuDL;
    return LBM_OK;
}

}  // namespace

extern "C" {

int lbm_derive_lattice(const lbm_physical* phys, int32_t storage, lbm_lattice* out)
{
    if (!phys || !out) return fail(LBM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (storage < LBM_STORAGE_F64 || storage > LBM_STORAGE_F16SR)
        return fail(LBM_ERR_INVALID_ARGUMENT, "unknown storage %d", storage);
    for (int d = 0; d < 3; ++d)
        if (phys->domain_size[d] <= 0 || !(phys->domain_length[d] > 0))
            return fail(LBM_ERR_INVALID_ARGUMENT, "domain size and length must be positive");
    if (!(phys->timestep > 0) || !(phys->max_velocity > 0) || !(phys->max_acceleration > 0))
        return fail(LBM_ERR_INVALID_ARGUMENT, "timestep, max velocity and max acceleration must be positive");
    return storage == LBM_STORAGE_F64 ? derive<double>(phys, out) : derive<float>(phys, out);
}

int lbm_create(const lbm_params* prm, lbm_solver** out)
{
    return create_solver(prm, nullptr, out);
}

}  // extern "C"

int lbm_detail::create_solver(const lbm_params* prm, void* external_dd, lbm_solver** out, int x1_align)
{
    if (!prm || !out) return fail(LBM_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    if (!domain_size_ok(prm->size))
        return fail(LBM_ERR_INVALID_ARGUMENT, "domain size must be in [1, 2^20] per axis and at most 2^40 cells");
    if (prm->storage < LBM_STORAGE_F64 || prm->storage > LBM_STORAGE_F16SR)
        return fail(LBM_ERR_INVALID_ARGUMENT, "unknown storage %d", prm->storage);
    for (int f = 0; f < 6; ++f)
        if (!valid_flag(prm->boundary[f])) return fail(LBM_ERR_INVALID_ARGUMENT, "invalid boundary flag %d", prm->boundary[f]);
    const bool gravity = prm->gravity[0] != 0.0 || prm->gravity[1] != 0.0 || prm->gravity[2] != 0.0;
    if (gravity && prm->storage >= LBM_STORAGE_F16S)
        return fail(LBM_ERR_UNSUPPORTED, "gravity is supported with F64 and F32 storage only");
    if (prm->fused_multiply_add != 0 && prm->fused_multiply_add != 1)
        return fail(LBM_ERR_INVALID_ARGUMENT, "fused_multiply_add must be 0 or 1");
    if (prm->fused_multiply_add && prm->storage != LBM_STORAGE_F64 && prm->storage != LBM_STORAGE_F32)
        return fail(LBM_ERR_INVALID_ARGUMENT, "fused_multiply_add applies to F64 and F32 storage only");
    if (!(prm->inv_tau > 0) || !std::isfinite(prm->inv_tau) || !std::isfinite(prm->lid_velocity))
        return fail(LBM_ERR_INVALID_ARGUMENT, "inv_tau must be positive and finite");
    if (prm->lid_mode != LBM_LID_INJECTION && prm->lid_mode != LBM_LID_MOVING_WALL)
        return fail(LBM_ERR_INVALID_ARGUMENT, "lid_mode must be LBM_LID_INJECTION or LBM_LID_MOVING_WALL");
    if (prm->lid_mode == LBM_LID_MOVING_WALL && prm->boundary[3] != LBM_OBSTACLE)
        return fail(LBM_ERR_INVALID_ARGUMENT, "a moving-wall lid needs an OBSTACLE top face (boundary[3])");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(LBM_ERR_NO_DEVICE, "no CUDA device visible");
    if (prm->device < 0 || prm->device >= ndev)
        return fail(LBM_ERR_INVALID_ARGUMENT, "device %d not in [0,%d)", prm->device, ndev);

    lbm_solver* s = new (std::nothrow) lbm_solver();
    if (!s) return fail(LBM_ERR_OUT_OF_MEMORY, "host allocation failed");
    s->storage = prm->storage;
    s->device = prm->device;
    s->g = lbm::make_grid(prm->size[0], prm->size[1], prm->size[2], elem_bytes(prm->storage), x1_align);
    s->p.inv_tau = prm->inv_tau;
    s->p.lid_u = prm->lid_velocity;
    s->p.gx = prm->gravity[0];
    s->p.gy = prm->gravity[1];
    s->p.gz = prm->gravity[2];
    for (int f = 0; f < 6; ++f) s->bc[f] = prm->boundary[f];
    if (prm->fast_variant < 0 || prm->fast_variant > lbm::kFastVariantCount) {
        delete s;
        return fail(LBM_ERR_INVALID_ARGUMENT, "fast_variant %d not in [0, %d]", prm->fast_variant,
                    lbm::kFastVariantCount);
    }
    s->variant = prm->fast_variant == 0 ? default_variant(s->storage) : prm->fast_variant - 1;
    s->fma = prm->fused_multiply_add == 1;
    s->lid_mode = prm->lid_mode;

    auto bail = [&](int r) { destroy_solver(s); return r; };
    cudaError_t e = cudaSetDevice(s->device);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaSetDevice"));
    const size_t dd_bytes = (size_t)lbm::Q * s->g.S * elem_bytes(s->storage);
    const size_t flag_bytes = (size_t)s->g.cells();
    const size_t scratch_bytes = (4 * (size_t)lbm::kReduceMaxBlocks + 4) * sizeof(double);
    if (external_dd) {
        s->dd = external_dd;
        s->owns_dd = false;
    } else if ((e = cudaMalloc(&s->dd, dd_bytes)) != cudaSuccess) {
        return bail(cuda_fail(e, "cudaMalloc populations"));
    }
    if ((e = cudaMalloc(&s->flags, flag_bytes)) != cudaSuccess) return bail(cuda_fail(e, "cudaMalloc flags"));
    if ((e = cudaMalloc(&s->scratch, scratch_bytes)) != cudaSuccess) return bail(cuda_fail(e, "cudaMalloc scratch"));
    if ((e = cudaMalloc(&s->counts, 6 * sizeof(unsigned long long))) != cudaSuccess)
        return bail(cuda_fail(e, "cudaMalloc counters"));
    if ((e = cudaMemset(s->counts, 0, 6 * sizeof(unsigned long long))) != cudaSuccess)
        return bail(cuda_fail(e, "cudaMemset counters"));
    s->p.step_base = step_words(s) + 1;  // direct launches: step = step_off
    s->p.step_off = 0;
    if ((e = cudaMallocHost(&s->host_out, 4 * sizeof(double))) != cudaSuccess)
        return bail(cuda_fail(e, "cudaMallocHost"));
    if ((e = cudaStreamCreateWithFlags(&s->capture_stream, cudaStreamNonBlocking)) != cudaSuccess)
        return bail(cuda_fail(e, "cudaStreamCreate"));
    s->device_bytes = (int64_t)((s->owns_dd ? dd_bytes : 0) + flag_bytes + scratch_bytes + 16);

    lbm::Bc bc;
    for (int f = 0; f < 6; ++f) bc.f[f] = prm->boundary[f];
    if ((e = lbm::launch_init(s->storage, s->dd, s->flags, s->g, bc, 0)) != cudaSuccess)
        return bail(cuda_fail(e, "init launch"));
    if (!lbm::fast_variant_fits(s->storage, s->variant, s->g))
        return bail(fail(LBM_ERR_UNSUPPORTED, "fast_variant %d needs more shared memory than this domain allows",
                         s->variant));
    int r = refresh_path(s);
    if (r) return bail(r);
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return bail(cuda_fail(e, "init"));
    *out = s;
    return LBM_OK;
}

void lbm_detail::destroy_solver(lbm_solver* s)
{
    if (!s) return;
    cudaSetDevice(s->device);
    cudaDeviceSynchronize();
    drop_graph(s);
    if (s->capture_stream) cudaStreamDestroy(s->capture_stream);
    if (s->dd && s->owns_dd) cudaFree(s->dd);
    if (s->flags) cudaFree(s->flags);
    if (s->macros) cudaFree(s->macros);
    if (s->scratch) cudaFree(s->scratch);
    if (s->counts) cudaFree(s->counts);
    if (s->staging) cudaFree(s->staging);
    if (s->host_out) cudaFreeHost(s->host_out);
    delete s;
}

extern "C" {

int lbm_destroy(lbm_solver* s)
{
    if (!s) return LBM_OK;
    if (s->batch) return fail(LBM_ERR_INVALID_ARGUMENT, "a batch domain is destroyed with its batch");
    destroy_solver(s);
    return LBM_OK;
}

int lbm_get_info(const lbm_solver* s, lbm_info* info)
{
    if (int r = check_solver(s)) return r;
    if (!info) return fail(LBM_ERR_INVALID_ARGUMENT, "info is NULL");
    info->size[0] = s->g.nx;
    info->size[1] = s->g.ny;
    info->size[2] = s->g.nz;
    info->storage = s->storage;
    info->value_size = value_bytes(s->storage);
    info->vector_cells = s->g.V;
    info->step_counter = s->counter;
    info->last_step_was_alpha = s->last_alpha ? 1 : 0;
    info->fast_path = s->lid_y >= 0 ? 1 : 0;
    info->fast_variant = s->variant;
    lbm::fast_variant_shape(s->storage, s->variant, true, s->g.nx, info->cells_per_thread, info->block_threads);
    lbm::fast_variant_shape(s->storage, s->variant, false, s->g.nx, info->beta_cells_per_thread,
                            info->beta_block_threads);
    info->fused_multiply_add = s->fma ? 1 : 0;
    info->beta_block_exchange = s->variant >= lbm::kRegisterVariants ? 0
                                : lbm::kFastMenu[s->variant].packed != 0 && elem_bytes(s->storage) == 2 ? 3
                                : lbm::kFastMenu[s->variant].direct       ? 2
                                : lbm::kFastMenu[s->variant].block_exchange ? 1
                                                                            : 0;
    info->row_pitch = s->g.P;
    info->slot_stride = s->g.S;
    info->device_bytes = s->device_bytes;
    info->lid_mode = s->lid_mode;
    info->moving_wall = s->p.wall_y > 0 ? 1 : 0;
    info->x1_column = s->g.xoff + 1;
    return LBM_OK;
}

int lbm_get_domain(const lbm_solver* s, int32_t size[3])
{
    if (int r = check_solver(s)) return r;
    if (!size) return fail(LBM_ERR_INVALID_ARGUMENT, "size is NULL");
    size[0] = s->g.nx;
    size[1] = s->g.ny;
    size[2] = s->g.nz;
    return LBM_OK;
}

int lbm_value_size(const lbm_solver* s)
{
    return s ? value_bytes(s->storage) : 0;
}

static int set_driven_cavity_unguarded(lbm_solver* s)
{
    if (int r = check_solver(s)) return r;
    if (s->lid_mode == LBM_LID_MOVING_WALL) {
        // the top wall starts moving; captured graphs hold the old parameters
        s->p.wall_y = s->g.ny;
        drop_graph(s);
        return LBM_OK;
    }
    const int32_t origin[3] = {1, s->g.ny, 1};   // src/CController.cpp:1313
    const int32_t size[3] = {s->g.nx, 1, s->g.nz};
    std::vector<int32_t> lid((size_t)s->g.nx * s->g.nz, LBM_VELOCITY_INJECTION);
    return lbm_set_flags(s, origin, size, lid.data());
}

int lbm_set_driven_cavity(lbm_solver* s)
{
    return guarded("lbm_set_driven_cavity", [&] { return set_driven_cavity_unguarded(s); });
}

int lbm_step_alpha(lbm_solver* s, void* stream)
{
    if (int r = check_solver(s)) return r;
    return step(s, true, nullptr, nullptr, static_cast<cudaStream_t>(stream));
}

int lbm_step_alpha_cuboid(lbm_solver* s, const int32_t origin[3], const int32_t size[3], void* stream)
{
    if (int r = check_solver(s)) return r;
    if (!origin || !size) return fail(LBM_ERR_INVALID_ARGUMENT, "origin and size are required");
    return step(s, true, origin, size, static_cast<cudaStream_t>(stream));
}

int lbm_step_beta(lbm_solver* s, void* stream)
{
    if (int r = check_solver(s)) return r;
    return step(s, false, nullptr, nullptr, static_cast<cudaStream_t>(stream));
}

int lbm_step_beta_cuboid(lbm_solver* s, const int32_t origin[3], const int32_t size[3], void* stream)
{
    if (int r = check_solver(s)) return r;
    if (!origin || !size) return fail(LBM_ERR_INVALID_ARGUMENT, "origin and size are required");
    return step(s, false, origin, size, static_cast<cudaStream_t>(stream));
}

int lbm_run(lbm_solver* s, int64_t steps, void* stream)
{
    if (int r = check_solver(s)) return r;
    if (steps < 0) return fail(LBM_ERR_INVALID_ARGUMENT, "negative step count");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CK(cudaSetDevice(s->device), "cudaSetDevice");
    int64_t left = steps;
    if (left > 0 && s->last_alpha) {  // next step is beta
        if (int r = step(s, false, nullptr, nullptr, st)) return r;
        --left;
    }
    const int64_t per_graph = 2 * kGraphPairs;
    if (s->lid_y >= 0 && left >= per_graph) {
        if (!s->graph) {
            cudaGraph_t graph = nullptr;
            const long long before = lbm::kernel_launches();
            CK(cudaStreamBeginCapture(s->capture_stream, cudaStreamCaptureModeThreadLocal), "begin capture");
            cudaError_t e = cudaSuccess;
            // launch i of the graph is step (word 0) + i
            lbm::Params p = s->p;
            p.step_base = step_words(s);
            for (int i = 0; i < kGraphPairs && e == cudaSuccess; ++i) {
                p.step_off = (uint32_t)(2 * i);
                e = lbm::launch_fast_step(kernel_storage(s), s->variant, true, s->dd, s->g, p, s->lid_y,
                                          err_flag(s), s->capture_stream);
                p.step_off = (uint32_t)(2 * i + 1);
                if (e == cudaSuccess)
                    e = lbm::launch_fast_step(kernel_storage(s), s->variant, false, s->dd, s->g, p, s->lid_y,
                                              err_flag(s), s->capture_stream);
            }
            cudaError_t e2 = cudaStreamEndCapture(s->capture_stream, &graph);
            // captured launches are counted when the graph runs
            lbm::add_launches(before - lbm::kernel_launches());
            if (e != cudaSuccess) return cuda_fail(e, "graph capture launch");
            if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
            e = cudaGraphInstantiate(&s->graph, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) {
                s->graph = nullptr;
                return cuda_fail(e, "cudaGraphInstantiate");
            }
        }
        while (left >= per_graph) {
            if (lbm::storage_stochastic(s->storage))
                CK(lbm::launch_set_step(step_words(s), (uint32_t)s->counter, st), "step word launch");
            CK(cudaGraphLaunch(s->graph, st), "cudaGraphLaunch");
            lbm::add_launches(per_graph);
            s->counter += per_graph;
            left -= per_graph;
        }
        s->last_alpha = false;
        s->macros_fresh = false;
    }
    while (left > 0) {
        if (int r = step(s, !s->last_alpha, nullptr, nullptr, st)) return r;
        --left;
    }
    return LBM_OK;
}

int lbm_synchronize(lbm_solver* s)
{
    if (int r = check_solver(s)) return r;
    CK(cudaSetDevice(s->device), "cudaSetDevice");
    CK(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    return check_kernel_flag(s);
}

int lbm_selftest_bounded_wait(lbm_solver* s, int32_t limit_us)
{
    if (int r = check_solver(s)) return r;
    if (limit_us < 1 || limit_us > 2000000) return fail(LBM_ERR_INVALID_ARGUMENT, "limit_us must be in [1, 2000000]");
    CK(cudaSetDevice(s->device), "cudaSetDevice");
    CK(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    if (int r = check_kernel_flag(s)) return r;  // an earlier failure is reported as such
    CK(lbm::launch_bounded_wait_probe(err_flag(s), (uint64_t)limit_us * 1000u, 0), "bounded wait probe launch");
    return lbm_synchronize(s);
}

int lbm_fast_variant_count(void) { return lbm::kFastVariantCount; }
int lbm_register_variant_count(void) { return lbm::kRegisterVariants; }

int lbm_set_fast_variant(lbm_solver* s, int32_t variant)
{
    if (int r = check_solver(s)) return r;
    if (variant < 0 || variant >= lbm::kFastVariantCount)
        return fail(LBM_ERR_INVALID_ARGUMENT, "variant %d not in [0, %d)", variant, lbm::kFastVariantCount);
    CK(cudaSetDevice(s->device), "cudaSetDevice");
    if (!lbm::fast_variant_fits(s->storage, variant, s->g))
        return fail(LBM_ERR_UNSUPPORTED, "variant %d needs more shared memory than this domain allows", variant);
    if (variant != s->variant) drop_graph(s);
    s->variant = variant;
    return LBM_OK;
}

int lbm_autotune(lbm_solver* s, int32_t pairs, int32_t* best, float* ms_per_pair)
{
    if (int r = check_solver(s)) return r;
    if (pairs <= 0) return fail(LBM_ERR_INVALID_ARGUMENT, "pairs must be positive");
    if (s->lid_y < 0) return fail(LBM_ERR_UNSUPPORTED, "autotune needs the vectorised (box cavity) path");
    CK(cudaSetDevice(s->device), "cudaSetDevice");
    CK(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    const size_t bytes = (size_t)lbm::Q * s->g.S * elem_bytes(s->storage);
    void* saved = nullptr;
    CK(cudaMalloc(&saved, bytes), "cudaMalloc autotune snapshot");
    cudaStream_t st = s->capture_stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int result = LBM_OK;
    float best_ms = 0.f;
    int best_v = s->variant;
    auto run_pairs = [&](int v, int n) -> cudaError_t {
        for (int i = 0; i < n; ++i) {
            cudaError_t e =
                lbm::launch_fast_step(kernel_storage(s), v, true, s->dd, s->g, s->p, s->lid_y, err_flag(s), st);
            if (e == cudaSuccess)
                e = lbm::launch_fast_step(kernel_storage(s), v, false, s->dd, s->g, s->p, s->lid_y, err_flag(s), st);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    };
    cudaError_t e = cudaMemcpyAsync(saved, s->dd, bytes, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (s->last_alpha && e == cudaSuccess)  // the timing runs alpha-first pairs from an even parity
        e = lbm::launch_fast_step(kernel_storage(s), s->variant, false, s->dd, s->g, s->p, s->lid_y, err_flag(s),
                                  st);
    bool any = false;
    for (int v = 0; v < lbm::kFastVariantCount && e == cudaSuccess; ++v) {
        if (!lbm::fast_variant_fits(s->storage, v, s->g)) {
            if (ms_per_pair) ms_per_pair[v] = -1.f;
            continue;
        }
        e = run_pairs(v, 1);  // warm-up
        if (e == cudaSuccess) e = cudaEventRecord(e0, st);
        if (e == cudaSuccess) e = run_pairs(v, pairs);
        if (e == cudaSuccess) e = cudaEventRecord(e1, st);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        ms /= (float)pairs;
        if (ms_per_pair) ms_per_pair[v] = ms;
        if (e == cudaSuccess && (!any || ms < best_ms)) {
            any = true;
            best_ms = ms;
            best_v = v;
        }
    }
    // restore the populations whatever happened above
    cudaError_t er = cudaMemcpyAsync(s->dd, saved, bytes, cudaMemcpyDeviceToDevice, st);
    if (er == cudaSuccess) er = cudaStreamSynchronize(st);
    if (e != cudaSuccess) result = cuda_fail(e, "autotune");
    else if (er != cudaSuccess) result = cuda_fail(er, "autotune restore");
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(saved);
    if (result != LBM_OK) return result;
    if (best) *best = best_v;
    return lbm_set_fast_variant(s, best_v);
}

int lbm_get_density_distributions(lbm_solver* s, const int32_t origin[3], const int32_t size[3], void* host,
                                  void* stream)
{
    if (int r = check_solver(s)) return r;
    if (!host) return fail(LBM_ERR_INVALID_ARGUMENT, "host buffer is NULL");
    int3 o, n;
    if (int r = resolve_cuboid(s, origin, size, o, n)) return r;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CK(cudaSetDevice(s->device), "cudaSetDevice");
    const size_t cells = (size_t)n.x * n.y * n.z;
    char* h = static_cast<char*>(host);
    if (s->storage <= LBM_STORAGE_F32) {
        for (int k = 0; k < lbm::Q; ++k)
            CK(copy_slot(s, k, o, n, h + (size_t)k * cells * elem_bytes(s->storage), true, st), "cudaMemcpy3DAsync");
        return LBM_OK;
    }
    if (int r = ensure_staging(s, cells)) return r;
    for (int k = 0; k < lbm::Q; ++k) {
        CK(lbm::launch_pack_slot(s->storage, s->dd, s->g, k, o, n, s->staging, st), "pack_slot launch");
        CK(cudaMemcpyAsync(h + (size_t)k * cells * sizeof(float), s->staging, cells * sizeof(float),
                           cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
    }
    return LBM_OK;
}

int lbm_set_density_distributions(lbm_solver* s, const int32_t origin[3], const int32_t size[3],
                                  int32_t direction, const void* host, void* stream)
{
    if (int r = check_solver(s)) return r;
    if (!host) return fail(LBM_ERR_INVALID_ARGUMENT, "host buffer is NULL");
    if (direction < LBM_DIRECTION_ALL || direction > LBM_FRONT)
        return fail(LBM_ERR_INVALID_ARGUMENT, "invalid direction %d", direction);
    int3 o, n;
    if (int r = resolve_cuboid(s, origin, size, o, n)) return r;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CK(cudaSetDevice(s->device), "cudaSetDevice");
    const size_t cells = (size_t)n.x * n.y * n.z;
    const char* h = static_cast<const char*>(host);
    s->macros_fresh = false;
    // FP64 takes a pitched 3-D copy per slot.  Every other storage stages each
    // slot as one contiguous float copy and scatters it with a kernel: for
    // FP32 that is several times faster than a host-to-device 3-D copy made of
    // short rows.
    if (s->storage == LBM_STORAGE_F64) {
        for (int k = 0; k < lbm::Q; ++k)
            if (slot_selected(direction, k))
                CK(copy_slot(s, k, o, n, const_cast<char*>(h) + (size_t)k * cells * elem_bytes(s->storage), false, st),
                   "cudaMemcpy3DAsync");
        return LBM_OK;
    }
    if (int r = ensure_staging(s, cells)) return r;
    for (int k = 0; k < lbm::Q; ++k) {
        if (!slot_selected(direction, k)) continue;
        CK(cudaMemcpyAsync(s->staging, h + (size_t)k * cells * sizeof(float), cells * sizeof(float),
                           cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
        CK(lbm::launch_unpack_slot(s->storage, s->dd, s->g, k, o, n, s->staging, st), "unpack_slot launch");
    }
    return LBM_OK;
}

static int get_flags_unguarded(lbm_solver* s, const int32_t origin[3], const int32_t size[3], int32_t* host)
{
    if (int r = check_solver(s)) return r;
    if (!host) return fail(LBM_ERR_INVALID_ARGUMENT, "host buffer is NULL");
    int3 o, n;
    if (int r = resolve_cuboid(s, origin, size, o, n)) return r;
    CK(cudaSetDevice(s->device), "cudaSetDevice");
    CK(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    std::vector<uint8_t> tmp((size_t)n.x * n.y * n.z);
    CK(copy_compact(s->flags, 1, s->g, o, n, tmp.data(), true), "cudaMemcpy3D flags");
    for (size_t i = 0; i < tmp.size(); ++i) host[i] = tmp[i];
    return LBM_OK;
}

int lbm_get_flags(lbm_solver* s, const int32_t origin[3], const int32_t size[3], int32_t* host)
{
    return guarded("lbm_get_flags", [&] { return get_flags_unguarded(s, origin, size, host); });
}

static int set_flags_unguarded(lbm_solver* s, const int32_t origin[3], const int32_t size[3], const int32_t* host)
{
    if (int r = check_solver(s)) return r;
    if (!host) return fail(LBM_ERR_INVALID_ARGUMENT, "host buffer is NULL");
    int3 o, n;
    if (int r = resolve_cuboid(s, origin, size, o, n)) return r;
    std::vector<uint8_t> tmp((size_t)n.x * n.y * n.z);
    for (size_t i = 0; i < tmp.size(); ++i) {
        if (!valid_flag(host[i])) return fail(LBM_ERR_INVALID_ARGUMENT, "invalid flag value %d at %zu", host[i], i);
        tmp[i] = (uint8_t)host[i];
    }
    CK(cudaSetDevice(s->device), "cudaSetDevice");
    CK(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    CK(copy_compact(s->flags, 1, s->g, o, n, tmp.data(), false), "cudaMemcpy3D flags");
    s->macros_fresh = false;
    return refresh_path(s);
}

int lbm_set_flags(lbm_solver* s, const int32_t origin[3], const int32_t size[3], const int32_t* host)
{
    return guarded("lbm_set_flags", [&] { return set_flags_unguarded(s, origin, size, host); });
}

static int macro_copy(lbm_solver* s, const int32_t* origin, const int32_t* size, void* host, int first, int count,
                      bool to_host)
{
    if (int r = check_solver(s)) return r;
    if (!host) return fail(LBM_ERR_INVALID_ARGUMENT, "host buffer is NULL");
    int3 o, n;
    if (int r = resolve_cuboid(s, origin, size, o, n)) return r;
    if (int r = ensure_macros(s)) return r;
    const size_t vb = (size_t)value_bytes(s->storage);
    const size_t cells = (size_t)n.x * n.y * n.z;
    for (int c = 0; c < count; ++c) {
        char* dev = static_cast<char*>(s->macros) + (size_t)(first + c) * s->g.cells() * vb;
        char* h = static_cast<char*>(host) + (size_t)c * cells * vb;
        CK(copy_compact(dev, vb, s->g, o, n, h, to_host), "cudaMemcpy3D macros");
    }
    return LBM_OK;
}

int lbm_get_velocities(lbm_solver* s, const int32_t origin[3], const int32_t size[3], void* host)
{
    return macro_copy(s, origin, size, host, 1, 3, true);
}

int lbm_set_velocities(lbm_solver* s, const int32_t origin[3], const int32_t size[3], const void* host)
{
    return macro_copy(s, origin, size, const_cast<void*>(host), 1, 3, false);
}

int lbm_get_densities(lbm_solver* s, const int32_t origin[3], const int32_t size[3], void* host)
{
    return macro_copy(s, origin, size, host, 0, 1, true);
}

int lbm_set_densities(lbm_solver* s, const int32_t origin[3], const int32_t size[3], const void* host)
{
    return macro_copy(s, origin, size, const_cast<void*>(host), 0, 1, false);
}

int lbm_reduce(lbm_solver* s, double out[4], void* stream)
{
    if (int r = check_solver(s)) return r;
    if (!out) return fail(LBM_ERR_INVALID_ARGUMENT, "out is NULL");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CK(cudaSetDevice(s->device), "cudaSetDevice");
    double* partials = s->scratch;
    double* result = s->scratch + 4 * lbm::kReduceMaxBlocks;
    CK(lbm::launch_reduce(s->storage, s->dd, s->flags, s->g, s->last_alpha, partials, result, st),
       "reduce launch");
    CK(cudaMemcpyAsync(s->host_out, result, 4 * sizeof(double), cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
    CK(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    if (int r = check_kernel_flag(s)) return r;
    for (int q = 0; q < 4; ++q) out[q] = s->host_out[q];
    return LBM_OK;
}

const char* lbm_status_string(int status)
{
    switch (status) {
    case LBM_OK: return "ok";
    case LBM_ERR_INVALID_ARGUMENT: return "invalid argument";
    case LBM_ERR_OUT_OF_BOUNDS: return "cuboid out of bounds";
    case LBM_ERR_CUDA: return "CUDA error";
    case LBM_ERR_OUT_OF_MEMORY: return "out of memory";
    case LBM_ERR_UNSUPPORTED: return "unsupported";
    case LBM_ERR_CONFIG: return "configuration error (rejected file or no stable time step)";
    case LBM_ERR_IO: return "I/O error";
    case LBM_ERR_BUDGET: return "over memory budget";
    case LBM_ERR_NOT_READY: return "not ready";
    case LBM_ERR_NO_DEVICE: return "no CUDA device";
    case LBM_ERR_TIMEOUT: return "device wait timed out";
    default: return "unknown status";
    }
}

const char* lbm_last_error(void) { return t_err; }

int64_t lbm_kernel_launches(void) { return lbm::kernel_launches(); }

}  // extern "C"
