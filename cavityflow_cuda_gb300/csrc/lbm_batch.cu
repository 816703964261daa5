// lbm_batch.cu -- many lid-driven cavities of uneven size and Reynolds number
// advanced together (include/lbm_gb300.h, "batches").
//
// The domains' padded population arrays live in one device pool.  Each domain
// is also a full lbm_solver ("view") whose populations are that pool region,
// so the per-domain getters, setters and reductions of the single-domain ABI
// apply unchanged.  A batch step is one launch of the persistent batch
// kernel (lbm_fast.cuh) over the packed domain table; long runs replay a CUDA
// graph of captured alpha/beta pairs.
#include <cmath>
#include <cstring>
#include <exception>
#include <new>
#include <vector>

#include "../../include/lbm_gb300.h"
#include "lbm_fast.cuh"
#include "lbm_internal.h"
#include "lbm_kernels.h"

using namespace lbm_detail;

namespace {

constexpr int kBatchGraphPairs = 32;

#define CK(call, what)                                     \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

}  // namespace

struct lbm_batch {
    int storage = 0;
    int device = 0;
    int variant = 0;
    void* pool = nullptr;
    size_t pool_bytes = 0;
    std::vector<lbm_solver*> views;
    std::vector<lbm::BatchDomain> table;
    lbm::BatchDomain* dtable = nullptr;
    uint32_t* step_words = nullptr;  // [0] first step of a graph replay, [1] zero
    long long vblocks[2] = {0, 0};  // virtual blocks of the alpha and the beta kernel
    int* vb_map[2] = {nullptr, nullptr};  // domain of each virtual block, per kernel
    long long vb_cap[2] = {0, 0};
    long long interior_cells = 0;
    cudaStream_t capture_stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    int64_t counter = 0;
    bool last_alpha = false;
};

namespace {

void drop_batch_graph(lbm_batch* b)
{
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
}

// Numbers the virtual blocks of the current variant, uploads the table and
// rebuilds the virtual-block maps.
int build_table(lbm_batch* b)
{
    for (int kind = 0; kind < 2; ++kind) {  // alpha, beta kernel
        long long next = 0;
        for (size_t i = 0; i < b->views.size(); ++i) {
            lbm::BatchDomain& d = b->table[i];
            int cpt = 1, block = 1;
            lbm::fast_variant_shape(b->storage, b->variant, kind == 0, d.g.nx, cpt, block);
            const long long n = lbm::set_batch_shape(d, kind, cpt, block);
            if (n < 0) return fail(LBM_ERR_INVALID_ARGUMENT, "batch domain %zu is too large", i);
            d.block_start[kind] = next;
            d.step0 = 0;  // every domain is at the batch's step
            next += n;
        }
        b->vblocks[kind] = next;
    }
    drop_batch_graph(b);
    CK(cudaDeviceSynchronize(), "batch table (pending work)");
    CK(cudaMemcpy(b->dtable, b->table.data(), b->table.size() * sizeof(lbm::BatchDomain), cudaMemcpyHostToDevice),
       "cudaMemcpy batch table");
    for (int kind = 0; kind < 2; ++kind) {
        if (b->vblocks[kind] > b->vb_cap[kind]) {
            if (b->vb_map[kind]) cudaFree(b->vb_map[kind]);
            b->vb_map[kind] = nullptr;
            b->vb_cap[kind] = 0;
            CK(cudaMalloc(&b->vb_map[kind], (size_t)b->vblocks[kind] * sizeof(int)), "cudaMalloc batch block map");
            b->vb_cap[kind] = b->vblocks[kind];
        }
        CK(lbm::launch_batch_map(b->dtable, (int)b->views.size(), b->vblocks[kind], kind, b->vb_map[kind], 0),
           "batch block map");
    }
    CK(cudaDeviceSynchronize(), "batch block map");
    return LBM_OK;
}

// One step of every domain.  Its stochastic-rounding step is step_off, or
// word 0 + step_off inside a graph (in_graph).
cudaError_t batch_launch(lbm_batch* b, int variant, bool alpha, cudaStream_t st, uint32_t step_off,
                         bool in_graph = false)
{
    const int kind = alpha ? 0 : 1;
    const lbm::BatchArgs a{b->pool, b->dtable, b->vb_map[kind], b->vblocks[kind], b->step_words + (in_graph ? 0 : 1),
                           step_off};
    return lbm::launch_batch_step(b->storage, variant, alpha, a, st);
}

void sync_views(lbm_batch* b)
{
    for (lbm_solver* v : b->views) {
        v->counter = b->counter;
        v->last_alpha = b->last_alpha;
        v->macros_fresh = false;
    }
}

void free_batch(lbm_batch* b)
{
    cudaSetDevice(b->device);
    cudaDeviceSynchronize();
    drop_batch_graph(b);
    for (lbm_solver* v : b->views) {
        v->batch = nullptr;
        destroy_solver(v);
    }
    if (b->capture_stream) cudaStreamDestroy(b->capture_stream);
    if (b->dtable) cudaFree(b->dtable);
    for (int kind = 0; kind < 2; ++kind)
        if (b->vb_map[kind]) cudaFree(b->vb_map[kind]);
    if (b->step_words) cudaFree(b->step_words);
    if (b->pool) cudaFree(b->pool);
    delete b;
}

}  // namespace

extern "C" {

static int batch_create_unguarded(const lbm_domain_spec* domains, int32_t count, int32_t storage, int32_t device, lbm_batch** out)
{
    if (!domains || !out || count <= 0) return fail(LBM_ERR_INVALID_ARGUMENT, "domains, count and out are required");
    *out = nullptr;
    if (storage < LBM_STORAGE_F64 || storage > LBM_STORAGE_F16SR)
        return fail(LBM_ERR_INVALID_ARGUMENT, "unknown storage %d", storage);
    long long pool_cells = 0;  // halo included; bounded like one domain, so the pool's byte count cannot overflow
    for (int i = 0; i < count; ++i) {
        if (!domain_size_ok(domains[i].size))
            return fail(LBM_ERR_INVALID_ARGUMENT, "domain %d: size must be in [1, 2^20] per axis and at most 2^40 cells",
                        i);
        pool_cells += ((long long)domains[i].size[0] + 2) * (domains[i].size[1] + 2) * (domains[i].size[2] + 2);
        if (pool_cells > kMaxDomainCells)
            return fail(LBM_ERR_INVALID_ARGUMENT, "the batch's domains hold more than 2^40 cells");
        if (!(domains[i].inv_tau > 0) || !std::isfinite(domains[i].inv_tau) || !std::isfinite(domains[i].lid_velocity))
            return fail(LBM_ERR_INVALID_ARGUMENT, "domain %d: inv_tau must be positive and finite", i);
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(LBM_ERR_NO_DEVICE, "no CUDA device visible");
    if (device < 0 || device >= ndev) return fail(LBM_ERR_INVALID_ARGUMENT, "device %d not in [0,%d)", device, ndev);
    CK(cudaSetDevice(device), "cudaSetDevice");

    lbm_batch* b = new (std::nothrow) lbm_batch();
    if (!b) return fail(LBM_ERR_OUT_OF_MEMORY, "host allocation failed");
    struct FreeIfThrown {  // a host allocation that throws below (turned into a status by
        lbm_batch* b;      // lbm_batch_create) must not leak the batch's device memory
        ~FreeIfThrown()
        {
            if (std::uncaught_exceptions() > 0) free_batch(b);
        }
    } free_if_thrown{b};
    b->storage = storage;
    b->device = device;
    b->variant = default_batch_variant(storage);
    auto bail = [&](int r) { free_batch(b); return r; };

    // pool layout: each domain's 19 padded slots, 256-byte aligned
    const int eb = elem_bytes(storage);
    std::vector<size_t> offsets((size_t)count);
    size_t elems = 0;
    b->table.resize((size_t)count);
    for (int i = 0; i < count; ++i) {
        const lbm::Grid g =
            lbm::make_grid(domains[i].size[0], domains[i].size[1], domains[i].size[2], eb, lbm::kPackedX1Align);
        offsets[(size_t)i] = elems;
        elems += (size_t)lbm::Q * g.S;  // S keeps every slot 256-byte aligned
        lbm::BatchDomain& d = b->table[(size_t)i];
        std::memset(&d, 0, sizeof(d));
        d.g = g;
        d.offset = (long long)offsets[(size_t)i];
        d.inv_tau = domains[i].inv_tau;
        d.lid_u = domains[i].lid_velocity;
        d.lid_y = g.ny;
        b->interior_cells += (long long)g.nx * g.ny * g.nz;
    }
    b->pool_bytes = elems * (size_t)eb;
    cudaError_t e = cudaMalloc(&b->pool, b->pool_bytes);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMalloc batch pool"));
    e = cudaMalloc(&b->dtable, (size_t)count * sizeof(lbm::BatchDomain));
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMalloc batch table"));
    e = cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaStreamCreate"));
    e = cudaMalloc(&b->step_words, 2 * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(b->step_words, 0, 2 * sizeof(uint32_t));
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaMalloc batch step words"));

    b->views.reserve((size_t)count);
    for (int i = 0; i < count; ++i) {
        lbm_params p;
        std::memset(&p, 0, sizeof(p));
        for (int d = 0; d < 3; ++d) p.size[d] = domains[i].size[d];
        p.storage = storage;
        for (int f = 0; f < 6; ++f) p.boundary[f] = LBM_OBSTACLE;
        p.inv_tau = domains[i].inv_tau;
        p.lid_velocity = domains[i].lid_velocity;
        p.device = device;
        p.fast_variant = b->variant + 1;
        lbm_solver* v = nullptr;
        int r = create_solver(&p, static_cast<char*>(b->pool) + offsets[(size_t)i] * (size_t)eb, &v,
                              lbm::kPackedX1Align);
        if (r) return bail(r);
        v->batch = b;
        b->views.push_back(v);
        r = lbm_set_driven_cavity(v);
        if (r) return bail(r);
    }
    int r = build_table(b);
    if (r) return bail(r);
    *out = b;
    return LBM_OK;
}

int lbm_batch_create(const lbm_domain_spec* domains, int32_t count, int32_t storage, int32_t device, lbm_batch** out)
{
    return guarded("lbm_batch_create", [&] { return batch_create_unguarded(domains, count, storage, device, out); });
}

int lbm_batch_destroy(lbm_batch* b)
{
    if (!b) return LBM_OK;
    free_batch(b);
    return LBM_OK;
}

int lbm_batch_get_info(const lbm_batch* b, lbm_batch_info* info)
{
    if (!b || !info) return fail(LBM_ERR_INVALID_ARGUMENT, "NULL argument");
    std::memset(info, 0, sizeof(*info));
    info->count = (int32_t)b->views.size();
    info->storage = b->storage;
    info->fast_variant = b->variant;
    lbm::fast_variant_shape(b->storage, b->variant, true, 1, info->cells_per_thread, info->block_threads);
    lbm::fast_variant_shape(b->storage, b->variant, false, 1, info->beta_cells_per_thread, info->beta_block_threads);
    info->interior_cells = b->interior_cells;
    info->step_counter = b->counter;
    int64_t bytes = (int64_t)b->pool_bytes + (int64_t)(b->table.size() * sizeof(lbm::BatchDomain)) +
                    (int64_t)((b->vb_cap[0] + b->vb_cap[1]) * (long long)sizeof(int));
    for (const lbm_solver* v : b->views) bytes += v->device_bytes;
    info->device_bytes = bytes;
    return LBM_OK;
}

int lbm_batch_domain(lbm_batch* b, int32_t index, lbm_solver** view)
{
    if (!b || !view) return fail(LBM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (index < 0 || index >= (int32_t)b->views.size())
        return fail(LBM_ERR_INVALID_ARGUMENT, "domain %d not in [0, %zu)", index, b->views.size());
    *view = b->views[(size_t)index];
    return LBM_OK;
}

int lbm_batch_run(lbm_batch* b, int64_t steps, void* stream)
{
    if (!b) return fail(LBM_ERR_INVALID_ARGUMENT, "batch is NULL");
    if (steps < 0) return fail(LBM_ERR_INVALID_ARGUMENT, "negative step count");
    for (size_t i = 0; i < b->views.size(); ++i)
        if (b->views[i]->counter != b->counter || b->views[i]->last_alpha != b->last_alpha)
            return fail(LBM_ERR_INVALID_ARGUMENT, "domain %zu was stepped outside its batch", i);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CK(cudaSetDevice(b->device), "cudaSetDevice");
    int64_t left = steps;
    auto one = [&](bool alpha) -> int {
        CK(batch_launch(b, b->variant, alpha, st, (uint32_t)b->counter), alpha ? "batch alpha launch" : "batch beta launch");
        b->counter += 1;
        b->last_alpha = alpha;
        return LBM_OK;
    };
    int r = LBM_OK;
    if (left > 0 && b->last_alpha) {
        if ((r = one(false))) return r;
        --left;
    }
    const int64_t per_graph = 2 * kBatchGraphPairs;
    if (left >= per_graph) {
        if (!b->graph) {
            cudaGraph_t graph = nullptr;
            const long long before = lbm::kernel_launches();
            CK(cudaStreamBeginCapture(b->capture_stream, cudaStreamCaptureModeThreadLocal), "begin capture");
            cudaError_t e = cudaSuccess;
            for (int i = 0; i < kBatchGraphPairs && e == cudaSuccess; ++i) {
                e = batch_launch(b, b->variant, true, b->capture_stream, (uint32_t)(2 * i), true);
                if (e == cudaSuccess) e = batch_launch(b, b->variant, false, b->capture_stream, (uint32_t)(2 * i + 1), true);
            }
            cudaError_t e2 = cudaStreamEndCapture(b->capture_stream, &graph);
            lbm::add_launches(before - lbm::kernel_launches());
            if (e != cudaSuccess) return cuda_fail(e, "batch graph capture");
            if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
            e = cudaGraphInstantiate(&b->graph, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) {
                b->graph = nullptr;
                return cuda_fail(e, "cudaGraphInstantiate");
            }
        }
        while (left >= per_graph) {
            if (lbm::storage_stochastic(b->storage))
                CK(lbm::launch_set_step(b->step_words, (uint32_t)b->counter, st), "step word launch");
            CK(cudaGraphLaunch(b->graph, st), "cudaGraphLaunch");
            lbm::add_launches(per_graph);
            b->counter += per_graph;
            left -= per_graph;
        }
        b->last_alpha = false;
    }
    while (left > 0 && r == LBM_OK) {
        r = one(!b->last_alpha);
        --left;
    }
    sync_views(b);
    return r;
}

int lbm_batch_set_fast_variant(lbm_batch* b, int32_t variant)
{
    if (!b) return fail(LBM_ERR_INVALID_ARGUMENT, "batch is NULL");
    if (variant < 0 || variant >= lbm::kRegisterVariants)
        return fail(LBM_ERR_INVALID_ARGUMENT, "batch variant %d not in [0, %d)", variant, lbm::kRegisterVariants);
    if (!b->views.empty() && !lbm::fast_variant_fits(b->storage, variant, b->views[0]->g))
        return fail(LBM_ERR_UNSUPPORTED, "variant %d's vectors do not fit the batch's packed rows", variant);
    CK(cudaSetDevice(b->device), "cudaSetDevice");
    b->variant = variant;
    for (lbm_solver* v : b->views) v->variant = variant;
    return build_table(b);
}

int lbm_batch_autotune(lbm_batch* b, int32_t pairs, int32_t* best, float* ms_per_pair)
{
    if (!b) return fail(LBM_ERR_INVALID_ARGUMENT, "batch is NULL");
    if (pairs <= 0) return fail(LBM_ERR_INVALID_ARGUMENT, "pairs must be positive");
    CK(cudaSetDevice(b->device), "cudaSetDevice");
    CK(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    void* saved = nullptr;
    CK(cudaMalloc(&saved, b->pool_bytes), "cudaMalloc autotune snapshot");
    cudaStream_t st = b->capture_stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const int start_variant = b->variant;
    int best_v = start_variant;
    float best_ms = 0.f;
    bool any = false;
    cudaError_t e = cudaMemcpyAsync(saved, b->pool, b->pool_bytes, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess && b->last_alpha) e = batch_launch(b, b->variant, false, st, 0);
    int r = LBM_OK;
    for (int v = 0; v < lbm::kRegisterVariants && e == cudaSuccess && r == LBM_OK; ++v) {
        if (!lbm::fast_variant_fits(b->storage, v, b->views[0]->g)) {  // vectors wider than the packed rows
            if (ms_per_pair) ms_per_pair[v] = -1.f;
            continue;
        }
        b->variant = v;
        if ((r = build_table(b))) break;
        for (int i = 0; i < 1 + pairs && e == cudaSuccess; ++i) {  // first pair warms up
            if (i == 1) e = cudaEventRecord(e0, st);
            if (e == cudaSuccess) e = batch_launch(b, v, true, st, 0);
            if (e == cudaSuccess) e = batch_launch(b, v, false, st, 0);
        }
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
    cudaError_t er = cudaMemcpyAsync(b->pool, saved, b->pool_bytes, cudaMemcpyDeviceToDevice, st);
    if (er == cudaSuccess) er = cudaStreamSynchronize(st);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(saved);
    if (r == LBM_OK && e != cudaSuccess) r = cuda_fail(e, "batch autotune");
    if (r == LBM_OK && er != cudaSuccess) r = cuda_fail(er, "batch autotune restore");
    b->variant = r == LBM_OK ? best_v : start_variant;
    for (lbm_solver* v : b->views) v->variant = b->variant;
    const int r2 = build_table(b);
    if (r != LBM_OK) return r;
    if (r2 != LBM_OK) return r2;
    if (best) *best = best_v;
    return LBM_OK;
}

}  // extern "C"
