// Serving loop: continuous batching of simulation requests over madi_walk
// (no counterpart in the reference, which walks one ensemble per call,
// madi/walker_gpu.py:1123-1203).
//
// Host-side admission (FIFO under a byte budget and a slot pool), tile-aligned
// round-robin chunking, per-launch job / geometry tables in caller-sized
// slices of a device arena, launches on server-owned streams and completion
// by events.  poll() never blocks.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <unordered_map>
#include <vector>
#include "madi_host.h"

using namespace madi;

namespace {

constexpr uint32_t PHILOX_KEY1 = 0x4D414449u;   // "MADI", the walk's second key word
constexpr int MAX_INFLIGHT = 4;

int64_t round256(int64_t x) { return (x + 255) & ~int64_t(255); }

int64_t slice_bytes(int32_t n_slots) {
    return round256((int64_t)n_slots * (int64_t)sizeof(madi_walk_job)) +
           round256((int64_t)n_slots * (int64_t)sizeof(madi_geometry)) + 256;
}

struct Request {
    madi_serve_request req;
    int64_t id;
    int32_t slot = -1;
    int64_t issued = 0, done = 0;
    double submit_s = 0, admit_s = 0;
};

struct Chunk {
    int64_t id;
    int32_t slot;
    int64_t base, n;
};

struct Launch {
    cudaEvent_t ev = nullptr;
    std::vector<Chunk> chunks;
    bool busy = false;
};

struct Server {
    madi_serve_config cfg;
    std::mutex mu;
    std::chrono::steady_clock::time_point t0;
    cudaStream_t streams[MAX_INFLIGHT] = {};
    cudaEvent_t zeroed = nullptr;
    Launch launches[MAX_INFLIGHT];
    std::deque<int64_t> order;             // launch indices in issue order
    int64_t next_id = 0;
    int64_t used = 0;
    std::vector<int32_t> free_slots;
    std::deque<int64_t> queue;             // submitted, not admitted
    std::deque<int64_t> rr;                // active, round robin
    std::unordered_map<int64_t, Request> reqs;
    std::deque<madi_serve_done> finished;  // reported once by poll
    int32_t grid_cap = 0;                  // SMs x resident blocks

    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

bool launch_pending_work(const Server& S) {
    for (int64_t id : S.rr) {
        const Request& r = S.reqs.at(id);
        if (r.issued < r.req.n_walkers) return true;
    }
    return false;
}

}  // namespace

extern "C" int64_t madi_serve_arena_bytes(const madi_serve_config* cfg) {
    if (!cfg || cfg->n_slots <= 0 || cfg->inflight <= 0 || cfg->inflight > MAX_INFLIGHT) return -1;
    return (int64_t)cfg->inflight * slice_bytes(cfg->n_slots);
}

extern "C" madi_status madi_serve_create(const madi_serve_config* cfg, void** server) {
    host::clear_error();
    if (!cfg || !server) return host::fail(MADI_ERR_INVALID, "serve_create: null argument");
    const madi_walk_desc& w = cfg->walk;
    if (cfg->n_slots <= 0 || cfg->inflight <= 0 || cfg->inflight > MAX_INFLIGHT || cfg->budget_bytes <= 0)
        return host::fail(MADI_ERR_INVALID, "serve_create: need slots > 0, 1 <= inflight <= %d, budget > 0",
                          MAX_INFLIGHT);
    if (w.precision != 32 || w.rng != MADI_RNG_PHILOX || w.out_mode != MADI_OUT_FUSED)
        return host::fail(MADI_ERR_INVALID, "serve_create: the template must be a fused fp32 Philox walk");
    if (w.tile_walkers <= 0 || cfg->chunk_walkers < w.tile_walkers || cfg->chunk_walkers % w.tile_walkers ||
        cfg->launch_walkers < cfg->chunk_walkers)
        return host::fail(MADI_ERR_INVALID,
                          "serve_create: chunk_walkers must be a multiple of tile_walkers and <= launch_walkers");
    if (!w.accum || !w.occupancy || !w.counters)
        return host::fail(MADI_ERR_INVALID, "serve_create: the template needs the slot pools");
    if (!cfg->arena || (reinterpret_cast<uintptr_t>(cfg->arena) & 255) ||
        cfg->arena_bytes < madi_serve_arena_bytes(cfg))
        return host::fail(MADI_ERR_CAPACITY, "serve_create: arena must be 256-byte aligned and >= %lld bytes",
                          (long long)madi_serve_arena_bytes(cfg));
    auto* S = new Server();
    S->cfg = *cfg;
    S->t0 = std::chrono::steady_clock::now();
    for (int i = cfg->n_slots - 1; i >= 0; --i) S->free_slots.push_back(i);
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < cfg->inflight && e == cudaSuccess; ++i) {
        e = cudaStreamCreateWithFlags(&S->streams[i], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&S->launches[i].ev, cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&S->zeroed, cudaEventDisableTiming);
    int dev = 0, sms = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) {
        madi_serve_destroy(S);
        return host::cuda_fail(e, "serve_create");
    }
    const int32_t bps = madi_walk_blocks_per_sm(&cfg->walk);
    if (bps <= 0) {
        madi_serve_destroy(S);
        return host::fail(MADI_ERR_CUDA, "serve_create: no resident walk block fits the template");
    }
    S->grid_cap = sms * bps;
    *server = S;
    return MADI_OK;
}

extern "C" madi_status madi_serve_submit(void* server, const madi_serve_request* req, int64_t* request_id) {
    host::clear_error();
    auto* S = static_cast<Server*>(server);
    if (!S || !req || !request_id) return host::fail(MADI_ERR_INVALID, "serve_submit: null argument");
    if (req->n_walkers <= 0 || req->n_walkers > INT32_MAX || !(req->pp >= 0.0 && req->pp <= 1.0) ||
        req->nbytes < 0)
        return host::fail(MADI_ERR_INVALID, "serve_submit: need 0 < n_walkers < 2^31, pp in [0, 1], nbytes >= 0");
    if (req->nbytes > S->cfg.budget_bytes)
        return host::fail(MADI_ERR_CAPACITY, "serve_submit: request needs %lld bytes, budget is %lld",
                          (long long)req->nbytes, (long long)S->cfg.budget_bytes);
    if (req->geometry.boundary != S->cfg.walk.boundary)
        return host::fail(MADI_ERR_INVALID, "serve_submit: geometry boundary differs from the server's");
    std::lock_guard<std::mutex> g(S->mu);
    Request r;
    r.req = *req;
    r.id = S->next_id++;
    r.submit_s = S->now();
    S->reqs.emplace(r.id, r);
    S->queue.push_back(r.id);
    *request_id = r.id;
    return MADI_OK;
}

static madi_status serve_admit(Server& S) {
    bool any = false;
    while (!S.queue.empty()) {
        Request& r = S.reqs.at(S.queue.front());
        if (S.used + r.req.nbytes > S.cfg.budget_bytes || S.free_slots.empty()) break;
        S.queue.pop_front();
        S.used += r.req.nbytes;
        r.slot = S.free_slots.back();
        S.free_slots.pop_back();
        r.admit_s = S.now();
        S.rr.push_back(r.id);
        const madi_walk_desc& w = S.cfg.walk;
        const int64_t n_out = (int64_t)w.n_pairs * w.n_b * w.n_dirs * 2;
        cudaStream_t s0 = S.streams[0];
        cudaError_t e = cudaMemsetAsync(w.accum + (int64_t)r.slot * n_out, 0, n_out * sizeof(int64_t), s0);
        if (e == cudaSuccess)
            e = cudaMemsetAsync(w.occupancy + (int64_t)r.slot * w.n_grid, 0, w.n_grid * sizeof(uint64_t), s0);
        if (e == cudaSuccess)
            e = cudaMemsetAsync(w.counters + (int64_t)r.slot * MADI_CNT_N, 0, MADI_CNT_N * sizeof(uint64_t), s0);
        if (e != cudaSuccess) return host::cuda_fail(e, "serve: slot zeroing");
        any = true;
    }
    if (any) {   // every stream sees the zeroed slots before its next launch
        cudaError_t e = cudaEventRecord(S.zeroed, S.streams[0]);
        for (int i = 1; i < S.cfg.inflight && e == cudaSuccess; ++i) e = cudaStreamWaitEvent(S.streams[i], S.zeroed, 0);
        if (e != cudaSuccess) return host::cuda_fail(e, "serve: stream ordering");
    }
    return MADI_OK;
}

static madi_status serve_launch(Server& S, int li) {
    const int32_t align = S.cfg.walk.tile_walkers;
    std::vector<Chunk> chunks;
    int64_t total = 0;
    const size_t n_active = S.rr.size();
    for (size_t k = 0; k < n_active && total < S.cfg.launch_walkers; ++k) {
        const int64_t id = S.rr.front();
        S.rr.pop_front();
        S.rr.push_back(id);
        Request& r = S.reqs.at(id);
        const int64_t rest = r.req.n_walkers - r.issued;
        int64_t n = std::min<int64_t>({(int64_t)S.cfg.chunk_walkers, rest, S.cfg.launch_walkers - total});
        if (n < rest) n = n / align * align;             // the next chunk stays tile-aligned
        if (n <= 0) continue;
        chunks.push_back({id, r.slot, r.issued, n});
        r.issued += n;
        total += n;
    }
    if (chunks.empty()) return MADI_OK;
    // host tables: geometries deduplicated by their stage pointer
    std::vector<madi_geometry> geoms;
    std::map<const void*, int32_t> gidx;
    std::vector<madi_walk_job> jobs;
    int32_t tiles = 0;
    for (const Chunk& c : chunks) {
        const Request& r = S.reqs.at(c.id);
        auto it = gidx.find(r.req.geometry.stage);
        int32_t gi;
        if (it == gidx.end()) {
            gi = (int32_t)geoms.size();
            gidx.emplace(r.req.geometry.stage, gi);
            geoms.push_back(r.req.geometry);
        } else {
            gi = it->second;
        }
        madi_walk_job j{};
        j.geom = gi;
        j.n_walkers = (int32_t)c.n;
        j.walker_base = (uint32_t)c.base;
        j.key0 = r.req.seed;
        j.key1 = PHILOX_KEY1;
        j.slot = c.slot;
        j.tile_begin = tiles;
        j.y_row = 0;
        j.pp = r.req.pp;
        if (r.req.pp >= 1.0) {
            j.thr1 = j.thr2 = UINT64_MAX;
        } else {   // floor(pp 2^64), floor(pp^2 2^64): exact scalings, then truncation
            j.thr1 = (uint64_t)std::ldexp(r.req.pp, 64);
            j.thr2 = (uint64_t)std::ldexp(r.req.pp * r.req.pp, 64);
        }
        jobs.push_back(j);
        tiles += (int32_t)((c.n + align - 1) / align);
    }
    unsigned char* slice = static_cast<unsigned char*>(S.cfg.arena) + (int64_t)li * slice_bytes(S.cfg.n_slots);
    auto* djobs = reinterpret_cast<madi_walk_job*>(slice);
    auto* dgeoms = reinterpret_cast<madi_geometry*>(slice + round256((int64_t)S.cfg.n_slots * sizeof(madi_walk_job)));
    auto* counter = reinterpret_cast<uint32_t*>(slice + round256((int64_t)S.cfg.n_slots * sizeof(madi_walk_job)) +
                                                round256((int64_t)S.cfg.n_slots * sizeof(madi_geometry)));
    cudaStream_t s = S.streams[li];
    // pageable sources: the copies complete (staged) before cudaMemcpyAsync returns
    cudaError_t e = cudaMemcpyAsync(djobs, jobs.data(), jobs.size() * sizeof(madi_walk_job), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dgeoms, geoms.data(), geoms.size() * sizeof(madi_geometry), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return host::cuda_fail(e, "serve: launch tables");
    madi_walk_desc d = S.cfg.walk;
    d.geoms = dgeoms;
    d.jobs = djobs;
    d.n_geoms = (int32_t)geoms.size();
    d.n_jobs = (int32_t)jobs.size();
    d.n_tiles = tiles;
    d.grid_blocks = std::min(tiles, S.grid_cap);
    d.work_counter = counter;
    const madi_status st = madi_walk(&d, s);
    if (st != MADI_OK) return st;
    e = cudaEventRecord(S.launches[li].ev, s);
    if (e != cudaSuccess) return host::cuda_fail(e, "serve: launch event");
    S.launches[li].chunks = std::move(chunks);
    S.launches[li].busy = true;
    S.order.push_back(li);
    return MADI_OK;
}

extern "C" madi_status madi_serve_poll(void* server, int32_t max_done, madi_serve_done* done, int32_t* n_done,
                                       int32_t* n_pending) {
    host::clear_error();
    auto* S = static_cast<Server*>(server);
    if (!S || !n_done || (max_done > 0 && !done)) return host::fail(MADI_ERR_INVALID, "serve_poll: null argument");
    std::lock_guard<std::mutex> g(S->mu);
    *n_done = 0;
    // reap finished launches in issue order
    while (!S->order.empty()) {
        Launch& L = S->launches[S->order.front()];
        const cudaError_t q = cudaEventQuery(L.ev);
        if (q == cudaErrorNotReady) break;
        if (q != cudaSuccess) return host::cuda_fail(q, "serve: launch failed");
        for (const Chunk& c : L.chunks) {
            Request& r = S->reqs.at(c.id);
            r.done += c.n;
            if (r.done == r.req.n_walkers) {
                S->rr.erase(std::find(S->rr.begin(), S->rr.end(), r.id));
                S->finished.push_back({r.id, r.slot, 0, r.submit_s, r.admit_s, S->now()});
            }
        }
        L.chunks.clear();
        L.busy = false;
        S->order.pop_front();
    }
    madi_status st = serve_admit(*S);
    if (st != MADI_OK) return st;
    for (int li = 0; li < S->cfg.inflight && launch_pending_work(*S); ++li) {
        if (S->launches[li].busy) continue;
        st = serve_launch(*S, li);
        if (st != MADI_OK) return st;
    }
    while (*n_done < max_done && !S->finished.empty()) {
        done[(*n_done)++] = S->finished.front();
        S->finished.pop_front();
    }
    if (n_pending) {
        int32_t p = (int32_t)S->queue.size();
        for (int64_t id : S->rr) (void)id, ++p;
        *n_pending = p + (int32_t)S->finished.size();
    }
    return MADI_OK;
}

extern "C" madi_status madi_serve_release(void* server, int64_t request_id) {
    host::clear_error();
    auto* S = static_cast<Server*>(server);
    if (!S) return host::fail(MADI_ERR_INVALID, "serve_release: null server");
    std::lock_guard<std::mutex> g(S->mu);
    auto it = S->reqs.find(request_id);
    if (it == S->reqs.end() || it->second.slot < 0 || it->second.done != it->second.req.n_walkers)
        return host::fail(MADI_ERR_INVALID, "serve_release: request %lld is not finished", (long long)request_id);
    S->free_slots.push_back(it->second.slot);
    S->used -= it->second.req.nbytes;
    S->reqs.erase(it);
    return MADI_OK;
}

extern "C" madi_status madi_serve_destroy(void* server) {
    host::clear_error();
    auto* S = static_cast<Server*>(server);
    if (!S) return MADI_OK;
    for (int i = 0; i < MAX_INFLIGHT; ++i) {
        if (S->streams[i]) cudaStreamSynchronize(S->streams[i]);
    }
    for (int i = 0; i < MAX_INFLIGHT; ++i) {
        if (S->launches[i].ev) cudaEventDestroy(S->launches[i].ev);
        if (S->streams[i]) cudaStreamDestroy(S->streams[i]);
    }
    if (S->zeroed) cudaEventDestroy(S->zeroed);
    delete S;
    return MADI_OK;
}
