// lbm_serve.cu -- a request server for lid-driven-cavity solves with
// continuous batching (include/lbm_gb300.h, "servers").
//
// Requests (one box cavity each: size, 1/tau, lid velocity, step count) wait
// in a FIFO queue.  Each round the server
//   1. admits queued requests, in order, while their populations fit the
//      device arena (a first-fit allocator over one allocation sized to the
//      memory budget); an admitted request is its arena block of populations,
//      initialised at rest by one kernel on the server's stream (the walls and
//      the lid come from the geometry, so a request has no flag array);
//   2. advances every resident request by the same even number of steps with
//      the batch kernel over a packed table of the resident domains (sized so
//      the round lasts about the target time); requests with a single (alpha)
//      step left sit at the end of the table and take it in the round's first
//      launch, which the later launches stop short of;
//   3. retires finished requests: one kernel per request writes density and
//      velocity of the last collided time level straight into mapped pinned
//      host memory, one stream synchronisation covers them all, then the
//      arena blocks are freed and completions posted.
// Admission and retirement allocate no device memory and make no
// device-wide synchronisation, so the GPU idles only for the host work of
// packing the next round's table.
// Requests that arrive while others are on the GPU therefore join the next
// round's launches as memory frees up, and their work shares the device with
// the requests already running.  Each request's populations evolve exactly as
// they would alone (the batch kernel's per-domain arithmetic is the
// single-domain one).  One host thread drives a server.
#include <algorithm>
#include <chrono>
#include <cmath>
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

constexpr double kArenaShare = 0.95;   // of the budget, for populations; the rest for the table and block maps
constexpr size_t kAlign = 256;
constexpr size_t kStageChunk = (size_t)1 << 30;  // host staging of one retirement batch, unless one result is larger

struct Request;
struct Staged {
    Request* r;
    size_t at;  // byte offset in its staging buffer
};

struct Request {
    int64_t id = 0;
    lbm_request spec{};
    double submit_t = 0, admit_t = -1, finish_t = -1;
    int64_t remaining = 0;
    size_t offset = 0, bytes = 0;
    lbm::Grid g{};
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
    // Results go to mapped pinned host memory, two buffers used in turn: the
    // kernels of one round write buffer `cur` while the host copies the
    // previous round's results out of the other.
    char* stage[2] = {nullptr, nullptr};
    void* stage_dev[2] = {nullptr, nullptr};  // their device addresses
    size_t stage_cap[2] = {0, 0};
    int cur = 0;
    std::vector<Staged> staged;  // results in stage[cur ^ 1] not yet copied out
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

// A request's layout: the packed rows of batch pools.
lbm::Grid request_grid(const int32_t size[3], int storage)
{
    return lbm::make_grid(size[0], size[1], size[2], elem_bytes(storage), lbm::kPackedX1Align);
}

size_t population_bytes(const int32_t size[3], int storage)
{
    const lbm::Grid g = request_grid(size, storage);
    return ((size_t)lbm::Q * g.S * elem_bytes(storage) + kAlign - 1) / kAlign * kAlign;
}

// Host bytes of a request's result: density and three velocity components of
// every interior cell.
size_t result_bytes(const Request* r, int storage)
{
    return (size_t)4 * r->spec.size[0] * r->spec.size[1] * r->spec.size[2] * (size_t)value_bytes(storage);
}

void free_request(lbm_server* s, Request* r)
{
    if (r->bytes) {
        s->alloc.release(r->offset, r->bytes);
        r->bytes = 0;
    }
}

void complete(lbm_server* s, Request* r, int status)
{
    r->status = status;
    free_request(s, r);
    r->finish_t = s->now();
    if (status == LBM_OK) s->completed += 1;
    s->finished[r->id] = r;
    const int64_t cells = (int64_t)r->spec.size[0] * r->spec.size[1] * r->spec.size[2];
    s->completions.push_back(
        {r->id, r->spec.steps, status == LBM_OK ? cells : 0, status, 0, r->submit_t, r->admit_t, r->finish_t});
}

int admit(lbm_server* s)
{
    while (!s->queue.empty()) {
        Request* r = s->queue.front();
        const size_t bytes = population_bytes(r->spec.size, s->cfg.storage);
        size_t off = 0;
        if (!s->alloc.alloc(bytes, off)) break;  // strict FIFO: the head waits for memory
        s->queue.pop_front();
        r->offset = off;
        r->bytes = bytes;
        // populations at rest; the steps that follow on the same stream see them
        if (cudaError_t e = lbm::launch_init_populations(s->cfg.storage, s->arena + off, r->g, s->stream)) {
            const int rc = cuda_fail(e, "server init launch");
            complete(s, r, rc);
            return rc;
        }
        r->admit_t = s->now();
        r->remaining = r->spec.steps;
        s->active.push_back(r);
        s->peak_bytes = std::max(s->peak_bytes, s->alloc.used());
    }
    return LBM_OK;
}

// Packs the given requests into the device table for `variant`.
int upload_table(lbm_server* s, const std::vector<Request*>& reqs, long long (&vblocks)[2])
{
    s->table.resize(reqs.size());
    long long next[2] = {0, 0};
    for (size_t i = 0; i < reqs.size(); ++i) {
        const Request* r = reqs[i];
        lbm::BatchDomain& d = s->table[i];
        std::memset(&d, 0, sizeof(d));
        d.g = r->g;
        d.offset = (long long)(r->offset / (size_t)elem_bytes(s->cfg.storage));
        d.inv_tau = r->spec.inv_tau;
        d.lid_u = r->spec.lid_velocity;
        d.lid_y = r->g.ny;
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

size_t round_up(size_t bytes) { return (bytes + kAlign - 1) / kAlign * kAlign; }

// Makes staging buffer b hold at least `bytes`; it holds no results that
// are still to be copied out.
int reserve_stage(lbm_server* s, int b, size_t bytes)
{
    if (bytes <= s->stage_cap[b]) return LBM_OK;
    CK(cudaStreamSynchronize(s->stream), "server staging");
    if (s->stage[b]) cudaFreeHost(s->stage[b]);
    s->stage[b] = nullptr;
    s->stage_dev[b] = nullptr;
    s->stage_cap[b] = 0;
    const size_t cap = round_up(bytes);
    CK(cudaHostAlloc((void**)&s->stage[b], cap, cudaHostAllocMapped), "cudaHostAlloc server staging");
    s->stage_cap[b] = cap;
    CK(cudaHostGetDevicePointer(&s->stage_dev[b], s->stage[b], 0), "cudaHostGetDevicePointer server staging");
    return LBM_OK;
}

// Queues on the server's stream the kernels that write the results of
// done[first], done[first + 1], ... into staging buffer b from its start, as
// many as fit (the first always does: the buffer holds the largest result);
// `next` follows the first request not queued, also when a launch fails.  A result is density and
// velocity of the time level collided last: after alpha for an odd step count.
int stage_results(lbm_server* s, int b, const std::vector<Request*>& done, size_t first,
                  std::vector<Staged>& staged, size_t& next)
{
    size_t used = 0;
    for (next = first; next < done.size(); ++next) {
        const Request* r = done[next];
        const size_t bytes = round_up(result_bytes(r, s->cfg.storage));
        if (next > first && used + bytes > s->stage_cap[b]) break;
        CK(lbm::launch_macros_cavity(s->cfg.storage, s->arena + r->offset, r->g, (r->spec.steps & 1) != 0,
                                     r->spec.lid_velocity, static_cast<char*>(s->stage_dev[b]) + used, s->stream),
           "server result launch");
        staged.push_back({done[next], used});
        used += bytes;
    }
    return LBM_OK;
}

// Copies results whose kernels have completed out of staging buffer b and
// posts their completions.
void post_staged(lbm_server* s, int b, std::vector<Staged>& staged)
{
    const size_t vb = (size_t)value_bytes(s->cfg.storage);
    for (const Staged& e : staged) {
        Request* r = e.r;
        const size_t cells = (size_t)r->spec.size[0] * r->spec.size[1] * r->spec.size[2];
        const char* src = s->stage[b] + e.at;
        r->rho.assign(src, src + cells * vb);
        r->u.assign(src + cells * vb, src + 4 * cells * vb);
        complete(s, r, LBM_OK);
    }
    staged.clear();
}

// Moves the active requests with no steps left to `done`, in order.
void take_finished(lbm_server* s, std::vector<Request*>& done)
{
    size_t keep = 0;
    for (Request* r : s->active) {
        if (r->remaining == 0) done.push_back(r);
        else s->active[keep++] = r;
    }
    s->active.resize(keep);
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
    const int32_t probe[3] = {8, 8, 8};  // any box: the packed rows' alignment does not depend on its size
    if (!lbm::fast_variant_fits(cfg->storage, s->variant, request_grid(probe, cfg->storage))) {
        delete s;
        return fail(LBM_ERR_UNSUPPORTED, "variant %d's vectors do not fit the server's packed rows", s->variant);
    }
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
    for (const Staged& e : s->staged) delete e.r;
    for (int b = 0; b < 2; ++b)
        if (s->stage[b]) cudaFreeHost(s->stage[b]);
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

static int server_submit_unguarded(lbm_server* s, const lbm_request* req, int64_t* id)
{
    if (!s || !req) return fail(LBM_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!domain_size_ok(req->size))
        return fail(LBM_ERR_INVALID_ARGUMENT, "size must be in [1, 2^20] per axis and at most 2^40 cells");
    if (req->steps < 0) return fail(LBM_ERR_INVALID_ARGUMENT, "negative step count");
    if (!(req->inv_tau > 0) || !std::isfinite(req->inv_tau) || !std::isfinite(req->lid_velocity))
        return fail(LBM_ERR_INVALID_ARGUMENT, "inv_tau must be positive and finite");
    if (population_bytes(req->size, s->cfg.storage) > s->arena_bytes)
        return fail(LBM_ERR_BUDGET, "request of %dx%dx%d cells can never fit the %lld-byte budget", req->size[0],
                    req->size[1], req->size[2], (long long)s->cfg.budget_bytes);
    Request* r = new (std::nothrow) Request();
    if (!r) return fail(LBM_ERR_OUT_OF_MEMORY, "host allocation failed");
    r->id = s->next_id++;
    r->spec = *req;
    r->g = request_grid(req->size, s->cfg.storage);
    r->submit_t = s->now();
    s->queue.push_back(r);
    if (id) *id = r->id;
    return LBM_OK;
}

int lbm_server_submit(lbm_server* s, const lbm_request* req, int64_t* id)
{
    return guarded("lbm_server_submit", [&] { return server_submit_unguarded(s, req, id); });
}

static int server_round_unguarded(lbm_server* s, int32_t* ran)
{
    if (!s) return fail(LBM_ERR_INVALID_ARGUMENT, "server is NULL");
    if (ran) *ran = 0;
    CK(cudaSetDevice(s->cfg.device), "cudaSetDevice");
    if (int rc = admit(s)) return rc;
    std::vector<Request*> done;  // finish this round; their results are read before their memory is freed
    take_finished(s, done);      // requests that need no steps finish at once
    std::vector<Staged> now_staged;
    // `run` = the requests advanced q (even) steps, then the `tail`: requests
    // with one (alpha) step left, which take it in the round's first launch
    // only.  Every request has taken an even number of steps before, so the
    // first launch is alpha for all of them; the later launches stop at the
    // tail's first virtual block.
    std::vector<Request*> run, tail;
    // On a CUDA error every request of the round, and every result not yet
    // posted, completes with the error and leaves the active list.
    auto abort_round = [&](int rc) {
        for (const Staged& e : s->staged) complete(s, e.r, rc);
        s->staged.clear();
        for (const std::vector<Request*>* list : {&done, &run, &tail})
            for (Request* r : *list)
                if (r->finish_t < 0) complete(s, r, rc);
        s->active.erase(std::remove_if(s->active.begin(), s->active.end(),
                                       [](const Request* r) { return r->finish_t >= 0; }),
                        s->active.end());
        return rc;
    };
    int64_t q = 0;
    long long run_cells = 0, tail_cells = 0, vblocks[2] = {0, 0}, vb_run[2] = {0, 0};
    if (!s->active.empty()) {
        int64_t min_rem = -1;
        for (Request* r : s->active) {
            const long long c = (long long)r->spec.size[0] * r->spec.size[1] * r->spec.size[2];
            if (r->remaining == 1) {
                tail.push_back(r);
                tail_cells += c;
            } else {
                run.push_back(r);
                run_cells += c;
                min_rem = min_rem < 0 ? r->remaining : std::min(min_rem, r->remaining);
            }
        }
        if (!run.empty()) {
            q = s->cfg.max_round_steps;
            if (s->cfg.target_round_ms > 0 && s->rate > 0) {
                const double want = s->cfg.target_round_ms * 1e-3 * s->rate / (double)(run_cells + tail_cells);
                q = std::min<int64_t>(q, std::max<int64_t>(2, (int64_t)want));
            }
            q = std::min<int64_t>(q, min_rem) & ~(int64_t)1;
            if (q < 2) q = 2;
        } else {
            q = 1;
        }
        const size_t n_run = run.size();
        run.insert(run.end(), tail.begin(), tail.end());
        if (int rc = upload_table(s, run, vblocks)) return abort_round(rc);
        for (int kind = 0; kind < 2; ++kind)
            vb_run[kind] = tail.empty() ? vblocks[kind] : s->table[n_run].block_start[kind];
        run.resize(n_run);
    }
    const auto t_start = std::chrono::steady_clock::now();
    for (int64_t i = 0; i < q; ++i) {
        const int kind = (int)(i & 1);
        const long long n = i == 0 ? vblocks[kind] : vb_run[kind];
        const lbm::BatchArgs a{s->arena, s->dtable, s->vb_map[kind], n, s->zero_word, (uint32_t)i};
        if (cudaError_t e = lbm::launch_batch_step(s->cfg.storage, s->variant, kind == 0, a, s->stream))
            return abort_round(cuda_fail(e, "server step launch"));
    }
    for (Request* r : run)
        if (r->remaining == q) done.push_back(r);
    done.insert(done.end(), tail.begin(), tail.end());
    // this round's results queue behind its steps, into the buffer the host is not reading
    const int b = s->cur;
    size_t want = 0, largest = 0, next = 0;
    for (const Request* r : done) {
        want += round_up(result_bytes(r, s->cfg.storage));
        largest = std::max(largest, round_up(result_bytes(r, s->cfg.storage)));
    }
    if (!done.empty()) {
        if (int rc = reserve_stage(s, b, std::max(largest, std::min(want, kStageChunk)))) return abort_round(rc);
        if (int rc = stage_results(s, b, done, 0, now_staged, next)) return abort_round(rc);
    }
    post_staged(s, b ^ 1, s->staged);  // the previous round's results, while the GPU runs
    if (cudaError_t e = cudaStreamSynchronize(s->stream)) return abort_round(cuda_fail(e, "server round"));
    if (q > 0) {
        const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
        const long long updates = run.empty() ? tail_cells : run_cells * q + tail_cells;
        s->busy_s += dt;
        s->rounds += 1;
        s->lattice_updates += updates;
        if (dt > 0 && q >= 2) s->rate = s->rate > 0 ? 0.7 * s->rate + 0.3 * (double)updates / dt
                                                      : (double)updates / dt;
        for (Request* r : run) r->remaining -= q;
        for (Request* r : tail) r->remaining -= 1;
        std::vector<Request*> finished_now;
        take_finished(s, finished_now);  // the requests of `done` that ran
    }
    s->staged = std::move(now_staged);
    // results that did not fit the buffer: copy out what it holds, then the rest a buffer at a time
    while (next < done.size()) {
        post_staged(s, b, s->staged);
        if (int rc = stage_results(s, b, done, next, s->staged, next)) return abort_round(rc);
        if (cudaError_t e = cudaStreamSynchronize(s->stream)) return abort_round(cuda_fail(e, "server results"));
    }
    for (Request* r : done) free_request(s, r);  // their results are read: the memory is free to admit
    s->cur ^= 1;
    if (s->active.empty()) post_staged(s, s->cur ^ 1, s->staged);  // no next round to overlap with
    if (ran) *ran = q > 0 ? 1 : 0;
    return LBM_OK;
}

int lbm_server_round(lbm_server* s, int32_t* ran)
{
    return guarded("lbm_server_round", [&] { return server_round_unguarded(s, ran); });
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

static int server_take_result_unguarded(lbm_server* s, int64_t id, void* rho_host, void* u_host)
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

int lbm_server_take_result(lbm_server* s, int64_t id, void* rho_host, void* u_host)
{
    return guarded("lbm_server_take_result", [&] { return server_take_result_unguarded(s, id, rho_host, u_host); });
}

int lbm_server_get_stats(const lbm_server* s, lbm_server_stats* st)
{
    if (!s || !st) return fail(LBM_ERR_INVALID_ARGUMENT, "NULL argument");
    std::memset(st, 0, sizeof(*st));
    st->queued = (int64_t)s->queue.size();
    st->active = (int64_t)s->active.size();
    st->completed = s->completed;
    st->bytes_in_use = (int64_t)s->alloc.used();
    st->peak_bytes = (int64_t)s->peak_bytes;
    st->budget_bytes = s->cfg.budget_bytes;
    st->lattice_updates = s->lattice_updates;
    st->rounds = s->rounds;
    st->busy_seconds = s->busy_s;
    st->elapsed_seconds = s->now();
    return LBM_OK;
}

}  // extern "C"
