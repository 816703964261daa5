// lbm_serve.cu -- a request server for lid-driven-cavity solves with
// continuous batching (include/lbm_gb300.h, "servers").
//
// Requests (one box cavity each: size, 1/tau, lid velocity, step count) wait
// in a FIFO queue.  Each round the server
//   1. admits queued requests, in order, while their populations fit the
//      device arena (a first-fit allocator over one allocation sized to the
//      memory budget) and their per-request metadata fits what is left of the
//      budget; an admitted request is a solver view on its arena block,
//      initialised at rest with the lid set;
//   2. advances every resident request by the same even number of steps with
//      the batch kernel over a packed table of the resident domains (sized so
//      the round lasts about the target time), or, when some request has a
//      single step left, runs that last alpha step for those requests alone;
//   3. retires finished requests: density and velocity of the last collided
//      time level are copied to host memory, the arena block is freed and a
//      completion is posted.
// Requests that arrive while others are on the GPU therefore join the next
// round's launches as memory frees up, and their work shares the device with
// the requests already running.  Each request's populations evolve exactly as
// they would alone (the batch kernel's per-domain arithmetic is the
// single-domain one).  One host thread drives a server.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <new>
#include <unordered_map>
#include <vector>

#include "../../include/lbm_gb300.h"
#include "lbm_fast.cuh"
#include "lbm_internal.h"
#include "lbm_kernels.h"

using namespace lbm_detail;

namespace {

#define CK(call, what)                                     \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

constexpr double kArenaShare = 0.95;   // of the budget, for populations; the rest for per-request metadata
constexpr size_t kAlign = 256;

struct Request {
    int64_t id = 0;
    lbm_request spec{};
    double submit_t = 0, admit_t = -1, finish_t = -1;
    int64_t remaining = 0;
    size_t offset = 0, bytes = 0, meta_bytes = 0;
    lbm_solver* view = nullptr;
    int status = LBM_OK;
    std::vector<unsigned char> rho, u;
};

// First-fit allocator over [0, capacity) with coalescing of free blocks.
class Arena {
public:
    void reset(size_t capacity)
    {
        free_.clear();
        if (capacity) free_[0] = capacity;
        used_ = 0;
    }
    bool alloc(size_t bytes, size_t& offset)
    {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                offset = it->first;
                const size_t rest = it->second - bytes;
                free_.erase(it);
                if (rest) free_[offset + bytes] = rest;
                used_ += bytes;
                return true;
            }
        }
        return false;
    }
    void release(size_t offset, size_t bytes)
    {
        auto it = free_.emplace(offset, bytes).first;
        used_ -= bytes;
        auto next = std::next(it);
        if (next != free_.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_.erase(next);
        }
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t used() const { return used_; }

private:
    std::map<size_t, size_t> free_;
    size_t used_ = 0;
};

}  // namespace

struct lbm_server {
    lbm_server_config cfg{};
    int variant = 0;
    char* arena = nullptr;
    size_t arena_bytes = 0;
    Arena alloc;
    size_t meta_in_use = 0;
    size_t peak_bytes = 0;
    std::deque<Request*> queue;
    std::vector<Request*> active;
    std::unordered_map<int64_t, Request*> finished;  // results not yet taken
    std::deque<lbm_completion> completions;           // not yet polled
    std::vector<lbm::BatchDomain> table;
    lbm::BatchDomain* dtable = nullptr;
    size_t dtable_cap = 0;
    int* vb_map[2] = {nullptr, nullptr};  // domain of each virtual block, per kernel
    long long vb_cap[2] = {0, 0};
    uint32_t* zero_word = nullptr;  // step base of the round launches (a request's step is its own count)
    cudaStream_t stream = nullptr;
    int64_t next_id = 1;
    int64_t completed = 0;
    int64_t lattice_updates = 0;
    int64_t rounds = 0;
    double busy_s = 0;
    double rate = 0;  // measured lattice updates per second (for round sizing)
    std::chrono::steady_clock::time_point t0;

    double now() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

namespace {

size_t population_bytes(const int32_t size[3], int storage)
{
    const lbm::Grid g = lbm::make_grid(size[0], size[1], size[2], elem_bytes(storage));
    return ((size_t)lbm::Q * g.S * elem_bytes(storage) + kAlign - 1) / kAlign * kAlign;
}

// Device bytes a solver view needs besides its populations (flags, reduction
// scratch, counters), as create_solver allocates them.
size_t metadata_bytes(const int32_t size[3])
{
    const size_t cells = (size_t)(size[0] + 2) * (size[1] + 2) * (size[2] + 2);
    return cells + (4 * (size_t)lbm::kReduceMaxBlocks + 4) * sizeof(double) + 64;
}

void free_request(lbm_server* s, Request* r)
{
    if (r->view) {
        destroy_solver(r->view);
        r->view = nullptr;
    }
    if (r->bytes) {
        s->alloc.release(r->offset, r->bytes);
        r->bytes = 0;
    }
    if (r->meta_bytes) {
        s->meta_in_use -= r->meta_bytes;
        r->meta_bytes = 0;
    }
}

int admit(lbm_server* s)
{
    const size_t meta_budget = (size_t)s->cfg.budget_bytes - s->arena_bytes;
    while (!s->queue.empty()) {
        Request* r = s->queue.front();
        const size_t bytes = population_bytes(r->spec.size, s->cfg.storage);
        const size_t meta = metadata_bytes(r->spec.size);
        if (s->meta_in_use + meta > meta_budget) break;
        size_t off = 0;
        if (!s->alloc.alloc(bytes, off)) break;  // strict FIFO: the head waits for memory
        s->queue.pop_front();
        r->offset = off;
        r->bytes = bytes;
        r->meta_bytes = meta;
        s->meta_in_use += meta;
        lbm_params p;
        std::memset(&p, 0, sizeof(p));
        for (int d = 0; d < 3; ++d) p.size[d] = r->spec.size[d];
        p.storage = s->cfg.storage;
        for (int f = 0; f < 6; ++f) p.boundary[f] = LBM_OBSTACLE;
        p.inv_tau = r->spec.inv_tau;
        p.lid_velocity = r->spec.lid_velocity;
        p.device = s->cfg.device;
        p.fast_variant = s->variant + 1;
        int rc = create_solver(&p, s->arena + off, &r->view);
        if (rc == LBM_OK) rc = lbm_set_driven_cavity(r->view);
        if (rc != LBM_OK) {
            r->status = rc;
            free_request(s, r);
            r->finish_t = s->now();
            s->finished[r->id] = r;
            s->completions.push_back({r->id, r->spec.steps, 0, rc, 0, r->submit_t, r->admit_t, r->finish_t});
            continue;
        }
        r->admit_t = s->now();
        r->remaining = r->spec.steps;
        s->active.push_back(r);
        const size_t in_use = s->alloc.used() + s->meta_in_use;
        s->peak_bytes = std::max(s->peak_bytes, in_use);
    }
    return LBM_OK;
}

// Packs the given requests into the device table for `variant`.
int upload_table(lbm_server* s, const std::vector<Request*>& reqs, long long (&vblocks)[2])
{
    s->table.resize(reqs.size());
    long long next[2] = {0, 0};
    for (size_t i = 0; i < reqs.size(); ++i) {
        const lbm_solver* v = reqs[i]->view;
        lbm::BatchDomain& d = s->table[i];
        std::memset(&d, 0, sizeof(d));
        d.g = v->g;
        d.offset = (long long)(reqs[i]->offset / (size_t)elem_bytes(s->cfg.storage));
        d.inv_tau = v->p.inv_tau;
        d.lid_u = v->p.lid_u;
        d.lid_y = v->g.ny;
        d.step0 = (uint32_t)(reqs[i]->spec.steps - reqs[i]->remaining);  // steps this request has taken
        for (int kind = 0; kind < 2; ++kind) {  // alpha, beta kernel
            int cpt = 1, block = 1;
            lbm::fast_variant_shape(s->cfg.storage, s->variant, kind == 0, d.g.nx, cpt, block);
            const long long n = lbm::set_batch_shape(d, kind, cpt, block);
            if (n < 0) return fail(LBM_ERR_INVALID_ARGUMENT, "request %lld is too large", (long long)reqs[i]->id);
            d.block_start[kind] = next[kind];
            next[kind] += n;
        }
    }
    vblocks[0] = next[0];
    vblocks[1] = next[1];
    if (reqs.size() > s->dtable_cap) {
        if (s->dtable) cudaFree(s->dtable);
        s->dtable = nullptr;
        const size_t cap = std::max<size_t>(reqs.size() * 2, 64);
        CK(cudaMalloc(&s->dtable, cap * sizeof(lbm::BatchDomain)), "cudaMalloc server table");
        s->dtable_cap = cap;
    }
    CK(cudaMemcpyAsync(s->dtable, s->table.data(), reqs.size() * sizeof(lbm::BatchDomain), cudaMemcpyHostToDevice,
                       s->stream),
       "cudaMemcpyAsync server table");
    for (int kind = 0; kind < 2; ++kind) {
        if (vblocks[kind] > s->vb_cap[kind]) {
            CK(cudaStreamSynchronize(s->stream), "server block map");
            if (s->vb_map[kind]) cudaFree(s->vb_map[kind]);
            s->vb_map[kind] = nullptr;
            s->vb_cap[kind] = 0;
            const long long cap = std::max<long long>(vblocks[kind] + vblocks[kind] / 2, 1024);
            CK(cudaMalloc(&s->vb_map[kind], (size_t)cap * sizeof(int)), "cudaMalloc server block map");
            s->vb_cap[kind] = cap;
        }
        CK(lbm::launch_batch_map(s->dtable, (int)reqs.size(), vblocks[kind], kind, s->vb_map[kind], s->stream),
           "server block map");
    }
    return LBM_OK;
}

int retire(lbm_server* s, Request* r)
{
    lbm_solver* v = r->view;
    v->counter = r->spec.steps;
    v->last_alpha = (r->spec.steps & 1) != 0;
    v->macros_fresh = false;
    const size_t cells = (size_t)r->spec.size[0] * r->spec.size[1] * r->spec.size[2];
    const size_t vb = (size_t)value_bytes(s->cfg.storage);
    r->rho.resize(cells * vb);
    r->u.resize(3 * cells * vb);
    int rc = lbm_get_densities(v, nullptr, nullptr, r->rho.data());
    if (rc == LBM_OK) rc = lbm_get_velocities(v, nullptr, nullptr, r->u.data());
    r->status = rc;
    free_request(s, r);
    r->finish_t = s->now();
    s->completed += 1;
    s->finished[r->id] = r;
    s->completions.push_back(
        {r->id, r->spec.steps, (int64_t)cells, rc, 0, r->submit_t, r->admit_t, r->finish_t});
    return LBM_OK;
}

}  // namespace

extern "C" {

int lbm_server_create(const lbm_server_config* cfg, lbm_server** out)
{
    if (!cfg || !out) return fail(LBM_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = nullptr;
    if (cfg->storage < LBM_STORAGE_F64 || cfg->storage > LBM_STORAGE_F16SR)
        return fail(LBM_ERR_INVALID_ARGUMENT, "unknown storage %d", cfg->storage);
    if (cfg->budget_bytes < (int64_t)(1 << 20)) return fail(LBM_ERR_INVALID_ARGUMENT, "budget below 1 MiB");
    if (cfg->max_round_steps < 2) return fail(LBM_ERR_INVALID_ARGUMENT, "max_round_steps must be >= 2");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(LBM_ERR_NO_DEVICE, "no CUDA device visible");
    if (cfg->device < 0 || cfg->device >= ndev)
        return fail(LBM_ERR_INVALID_ARGUMENT, "device %d not in [0,%d)", cfg->device, ndev);
    CK(cudaSetDevice(cfg->device), "cudaSetDevice");
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
    lbm_server* s = new (std::nothrow) lbm_server();
    if (!s) return fail(LBM_ERR_OUT_OF_MEMORY, "host allocation failed");
    s->cfg = *cfg;
    s->cfg.max_round_steps &= ~1;
    s->variant = cfg->fast_variant > 0 && cfg->fast_variant <= lbm::kRegisterVariants ? cfg->fast_variant - 1
                                                                                       : default_batch_variant(cfg->storage);
    s->arena_bytes = (size_t)((double)cfg->budget_bytes * kArenaShare) / kAlign * kAlign;
    if (s->arena_bytes + (size_t)(1 << 30) > free_b) {
        delete s;
        return fail(LBM_ERR_BUDGET, "budget of %lld bytes exceeds the free device memory (%zu bytes)",
                    (long long)cfg->budget_bytes, free_b);
    }
    cudaError_t e = cudaMalloc((void**)&s->arena, s->arena_bytes);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void**)&s->zero_word, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(s->zero_word, 0, sizeof(uint32_t));
    if (e != cudaSuccess) {
        lbm_server_destroy(s);
        return cuda_fail(e, "server allocation");
    }
    s->alloc.reset(s->arena_bytes);
    s->t0 = std::chrono::steady_clock::now();
    *out = s;
    return LBM_OK;
}

int lbm_server_destroy(lbm_server* s)
{
    if (!s) return LBM_OK;
    cudaSetDevice(s->cfg.device);
    cudaDeviceSynchronize();
    for (Request* r : s->active) {
        free_request(s, r);
        delete r;
    }
    for (Request* r : s->queue) delete r;
    for (auto& kv : s->finished) delete kv.second;
    if (s->dtable) cudaFree(s->dtable);
    for (int kind = 0; kind < 2; ++kind)
        if (s->vb_map[kind]) cudaFree(s->vb_map[kind]);
    if (s->zero_word) cudaFree(s->zero_word);
    if (s->arena) cudaFree(s->arena);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return LBM_OK;
}

int lbm_server_submit(lbm_server* s, const lbm_request* req, int64_t* id)
{
    if (!s || !req) return fail(LBM_ERR_INVALID_ARGUMENT, "NULL argument");
    for (int d = 0; d < 3; ++d)
        if (req->size[d] <= 0 || req->size[d] > (1 << 20))
            return fail(LBM_ERR_INVALID_ARGUMENT, "size must be in [1, 2^20]");
    if (req->steps < 0) return fail(LBM_ERR_INVALID_ARGUMENT, "negative step count");
    if (!(req->inv_tau > 0)) return fail(LBM_ERR_INVALID_ARGUMENT, "inv_tau must be positive");
    if (population_bytes(req->size, s->cfg.storage) > s->arena_bytes ||
        metadata_bytes(req->size) > (size_t)s->cfg.budget_bytes - s->arena_bytes)
        return fail(LBM_ERR_BUDGET, "request of %dx%dx%d cells can never fit the %lld-byte budget", req->size[0],
                    req->size[1], req->size[2], (long long)s->cfg.budget_bytes);
    Request* r = new (std::nothrow) Request();
    if (!r) return fail(LBM_ERR_OUT_OF_MEMORY, "host allocation failed");
    r->id = s->next_id++;
    r->spec = *req;
    r->submit_t = s->now();
    s->queue.push_back(r);
    if (id) *id = r->id;
    return LBM_OK;
}

int lbm_server_round(lbm_server* s, int32_t* ran)
{
    if (!s) return fail(LBM_ERR_INVALID_ARGUMENT, "server is NULL");
    if (ran) *ran = 0;
    CK(cudaSetDevice(s->cfg.device), "cudaSetDevice");
    if (int rc = admit(s)) return rc;
    // requests that need no steps finish at once
    for (size_t i = 0; i < s->active.size();) {
        if (s->active[i]->remaining == 0) {
            Request* r = s->active[i];
            s->active.erase(s->active.begin() + (long)i);
            if (int rc = retire(s, r)) return rc;
        } else {
            ++i;
        }
    }
    if (s->active.empty()) return LBM_OK;

    int64_t min_rem = s->active[0]->remaining;
    long long cells = 0;
    for (Request* r : s->active) {
        min_rem = std::min(min_rem, r->remaining);
        cells += (long long)r->spec.size[0] * r->spec.size[1] * r->spec.size[2];
    }
    std::vector<Request*> run;
    int64_t q;
    if (min_rem == 1) {  // the last (alpha) step of the requests with one step left
        for (Request* r : s->active)
            if (r->remaining == 1) run.push_back(r);
        q = 1;
    } else {
        run = s->active;
        q = s->cfg.max_round_steps;
        if (s->cfg.target_round_ms > 0 && s->rate > 0) {
            const double want = s->cfg.target_round_ms * 1e-3 * s->rate / (double)cells;
            q = std::min<int64_t>(q, std::max<int64_t>(2, (int64_t)want));
        }
        q = std::min<int64_t>(q, min_rem) & ~(int64_t)1;
        if (q < 2) q = 2;
    }
    long long run_cells = 0;
    for (Request* r : run) run_cells += (long long)r->spec.size[0] * r->spec.size[1] * r->spec.size[2];
    long long vblocks[2] = {0, 0};
    if (int rc = upload_table(s, run, vblocks)) return rc;
    const auto t_start = std::chrono::steady_clock::now();
    for (int64_t i = 0; i < q; ++i) {
        const int kind = (int)(i & 1);
        const lbm::BatchArgs a{s->arena, s->dtable, s->vb_map[kind], vblocks[kind], s->zero_word, (uint32_t)i};
        CK(lbm::launch_batch_step(s->cfg.storage, s->variant, kind == 0, a, s->stream), "server step launch");
    }
    CK(cudaStreamSynchronize(s->stream), "server round");
    const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    s->busy_s += dt;
    s->rounds += 1;
    s->lattice_updates += run_cells * q;
    if (dt > 0 && q >= 2) s->rate = s->rate > 0 ? 0.7 * s->rate + 0.3 * (double)(run_cells * q) / dt
                                                  : (double)(run_cells * q) / dt;
    for (Request* r : run) r->remaining -= q;
    for (size_t i = 0; i < s->active.size();) {
        if (s->active[i]->remaining == 0) {
            Request* r = s->active[i];
            s->active.erase(s->active.begin() + (long)i);
            if (int rc = retire(s, r)) return rc;
        } else {
            ++i;
        }
    }
    if (ran) *ran = 1;
    return LBM_OK;
}

int lbm_server_poll(lbm_server* s, lbm_completion* out, int32_t capacity, int32_t* count)
{
    if (!s || !count || (capacity > 0 && !out)) return fail(LBM_ERR_INVALID_ARGUMENT, "NULL argument");
    int32_t n = 0;
    while (n < capacity && !s->completions.empty()) {
        out[n++] = s->completions.front();
        s->completions.pop_front();
    }
    *count = n;
    return LBM_OK;
}

int lbm_server_take_result(lbm_server* s, int64_t id, void* rho_host, void* u_host)
{
    if (!s) return fail(LBM_ERR_INVALID_ARGUMENT, "server is NULL");
    auto it = s->finished.find(id);
    if (it == s->finished.end()) return fail(LBM_ERR_NOT_READY, "request %lld has no result (yet)", (long long)id);
    Request* r = it->second;
    if (rho_host && !r->rho.empty()) std::memcpy(rho_host, r->rho.data(), r->rho.size());
    if (u_host && !r->u.empty()) std::memcpy(u_host, r->u.data(), r->u.size());
    const int status = r->status;
    s->finished.erase(it);
    delete r;
    return status;
}

int lbm_server_get_stats(const lbm_server* s, lbm_server_stats* st)
{
    if (!s || !st) return fail(LBM_ERR_INVALID_ARGUMENT, "NULL argument");
    std::memset(st, 0, sizeof(*st));
    st->queued = (int64_t)s->queue.size();
    st->active = (int64_t)s->active.size();
    st->completed = s->completed;
    st->bytes_in_use = (int64_t)(s->alloc.used() + s->meta_in_use);
    st->peak_bytes = (int64_t)s->peak_bytes;
    st->budget_bytes = s->cfg.budget_bytes;
    st->lattice_updates = s->lattice_updates;
    st->rounds = s->rounds;
    st->busy_seconds = s->busy_s;
    st->elapsed_seconds = s->now();
    return LBM_OK;
}

}  // extern "C"
