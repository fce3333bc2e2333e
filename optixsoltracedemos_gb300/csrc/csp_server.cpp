// csp_server.cpp -- trace-request server with continuous batching (csp_server_* of
// include/csp_c_api.h).
//
// Requests (a resident scene, optional new heliostat poses, a sun, a ray count, seed and instance
// id) are submitted from any host thread.  One worker thread runs steps:
//   1. launch step k: every active request traces its next slice of rays in the same persistent
//      launch per kernel group (the batch kernels of csp_batch.cu), receiver records binned into the
//      request's resident flux map; requests whose last slice is in the step copy their flux map,
//      counters and sun frame to pinned host memory behind the launch;
//   2. while the GPU runs: admit pending requests while slots and device memory allow -- one
//      upload of each request's host part (its element records and field grid were built at
//      submission: the reference's geometry arithmetic, as the single-scene path, in ranges of
//      elements on the server's host threads), refit of the scene's BVH topology in place into the
//      request's nodes, sun plane, sun-ray candidate grid; all on the admission stream, which the
//      step stream waits for before step k+1, so the request joins step k+1;
//   3. wait for step k - 1, complete its finished requests (latency = completion - submission), free
//      their device memory.  Steps alternate between two streams: step k is launched before step
//      k - 1 ends, so its CTAs fill the tail of step k - 1.
// A request's result does not depend on what it was batched with or how its rays were sliced: its
// rays are traced with the same (seed, instance, ray index) and its flux map is an integer sum.
//
// Device memory: one arena of the configured budget, first-fit blocks per request (element
// records when the request has its own poses, refitted nodes, sun frame, sun grid, flux map).  A request is
// admitted when its block fits; requests larger than the whole budget fail.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "csp_c_api.h"
#include "csp_kernels.cuh"
#include "csp_math.cuh"
#include "csp_scene.h"
#include "csp_system.h"

namespace csp {
namespace {

// Fixed set of host threads for the parallel part of a submission (element records in ranges).
// run() executes body(k) for k in [0, tasks) on the pool and the calling thread and returns when all
// are done; concurrent callers take turns.
class HostPool {
public:
    void start(unsigned threads) {
        for (unsigned t = 0; t < threads; ++t) th_.emplace_back([this] { loop(); });
    }
    void stop() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            quit_ = true;
        }
        cv_.notify_all();
        for (auto& t : th_) t.join();
        th_.clear();
    }
    void run(size_t tasks, const std::function<void(size_t)>& body) {
        std::lock_guard<std::mutex> turn(run_mu_);
        {
            std::lock_guard<std::mutex> lk(mu_);
            body_ = &body;
            tasks_ = tasks;
            next_ = 0;
            left_ = tasks;
            ++gen_;
        }
        cv_.notify_all();
        work();
        std::unique_lock<std::mutex> lk(mu_);
        cv_done_.wait(lk, [&] { return left_ == 0; });
        body_ = nullptr;
    }

private:
    // take tasks of the current job until none is left
    void work() {
        for (;;) {
            size_t k;
            const std::function<void(size_t)>* body;
            {
                std::lock_guard<std::mutex> lk(mu_);
                if (!body_ || next_ >= tasks_) return;
                k = next_++;
                body = body_;
            }
            (*body)(k);
            std::lock_guard<std::mutex> lk(mu_);
            if (--left_ == 0) cv_done_.notify_all();
        }
    }
    void loop() {
        uint64_t seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return quit_ || gen_ != seen; });
                if (quit_) return;
                seen = gen_;
            }
            work();
        }
    }
    std::mutex mu_, run_mu_;
    std::condition_variable cv_, cv_done_;
    std::vector<std::thread> th_;
    const std::function<void(size_t)>* body_ = nullptr;
    size_t tasks_ = 0, next_ = 0, left_ = 0;
    uint64_t gen_ = 0;
    bool quit_ = false;
};

using Clock = std::chrono::steady_clock;

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct SScene {
    std::vector<csp_element> elements;
    HostScene base;
    HostGrid grid;
    int group = kAccelBvh;
    Node* d_topo = nullptr;
    uint32_t* d_cells = nullptr;
    Aabb* d_items = nullptr;
    Aabb* d_global = nullptr;
    // the scene's own element records, for requests without poses
    Prim* d_prims = nullptr;
    Optics* d_optics = nullptr;
    Aabb* d_aabbs = nullptr;
    Node* d_nodes = nullptr;
};

enum ReqState { kPending = 0, kActive = 1, kDone = 2, kFailed = 3 };

struct SRequest {
    uint64_t id = 0;
    uint32_t scene = 0;
    const SScene* sc = nullptr;  // set at submission (the scene list may grow meanwhile)
    std::vector<csp_element> poses;
    HostScene hs;   // element records of the poses (built at submission)
    HostGrid grid;  // grid of the poses (field-like scenes)
    double sun[3] = {0, 0, 1};
    int shape = CSP_SUN_PILLBOX;
    double param = 0;
    uint64_t rays = 0, seed = 0;
    uint32_t instance = 0;
    int out_flags = 0;  // CSP_OUT_* of its flux map (the server's setting at submission)

    ReqState state = kPending;
    InstanceDesc desc{};      // its step descriptor except the ray window and tile offset
    bool desc_ready = false;  // built at its first step (its arena block and scene are fixed)
    std::string error;
    int error_status = CSP_ERR_CUDA;  // status csp_server_wait returns for a failed request
    uint64_t next_ray = 0;
    int group = kAccelBvh;
    size_t off = 0, bytes = 0;  // arena block
    size_t o_prims = 0, o_optics = 0, o_aabbs = 0, o_prune = 0, o_nodes = 0, o_sun = 0, o_grid = 0, o_counts = 0,
           o_stats = 0, o_cells = 0, o_items = 0, o_global = 0, o_sgrid = 0;
    bool own_records = false;
    int result_slot = -1;
    Clock::time_point t_submit, t_admit, t_done;
    std::vector<uint32_t> counts;
    uint64_t stats[4] = {0, 0, 0, 0};
    SunFrame sunf{};
};

// First-fit allocator over [0, cap) with coalescing frees.
struct Arena {
    size_t cap = 0, used = 0, peak = 0;
    std::map<size_t, size_t> free_blocks;  // offset -> size
    void reset(size_t c) {
        cap = c;
        used = peak = 0;
        free_blocks.clear();
        if (c) free_blocks[0] = c;
    }
    bool alloc(size_t bytes, size_t& off) {
        for (auto it = free_blocks.begin(); it != free_blocks.end(); ++it) {
            if (it->second >= bytes) {
                off = it->first;
                const size_t rest = it->second - bytes;
                free_blocks.erase(it);
                if (rest) free_blocks[off + bytes] = rest;
                used += bytes;
                peak = std::max(peak, used);
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        used -= bytes;
        auto it = free_blocks.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_blocks.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_blocks.erase(nx);
        }
        if (it != free_blocks.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_blocks.erase(it);
            }
        }
    }
};

}  // namespace

struct Server {
    int device = -1;
    // steps alternate between two streams, each with its own descriptor tables and work counters:
    // step k + 1 is launched before step k ends, so its CTAs fill step k's tail
    cudaStream_t stream[2] = {nullptr, nullptr};
    cudaEvent_t step_done[2] = {nullptr, nullptr};
    // admissions (uploads, refits, sun planes, sun-ray grids) go to their own stream: the uploads
    // overlap the running step, the kernels fill its tail; the step stream waits on adm_done
    // before the next step
    cudaStream_t adm_stream = nullptr;
    cudaEvent_t adm_done = nullptr;
    HostPool pool;  // element records of large submissions, in ranges
    uint32_t nx = 100, ny = 100;
    int out_flags = 0;  // CSP_OUT_* given to requests at submission
    int max_active = 64;
    uint64_t step_rays = 64ull << 20;  // rays per step across all active requests (target; see kMinSlice)
    size_t budget = 0;

    std::vector<std::unique_ptr<SScene>> scenes;
    std::map<uint64_t, std::unique_ptr<SRequest>> requests;
    std::deque<SRequest*> pending;
    std::vector<SRequest*> active;
    uint64_t next_id = 1;
    // refit, sun-plane and sun-grid job tables of one admission pass (at most max_active requests);
    // the kernels that read them finish at the step synchronisation before the next pass
    unsigned char* d_jobs = nullptr;
    size_t jobs_cap = 0;

    unsigned char* d_arena = nullptr;
    Arena arena;
    // per-step device tables and their pinned staging
    unsigned char* d_step[2] = {nullptr, nullptr};
    unsigned char* h_step[2] = {nullptr, nullptr};
    size_t step_bytes = 0;
    // admission staging (pinned) and results (pinned, one slot per active request)
    unsigned char* h_adm = nullptr;
    size_t adm_cap = 0;
    unsigned char* h_res = nullptr;
    size_t res_slot_bytes = 0;
    std::vector<int> free_res_slots;
    unsigned long long* d_counter[2] = {nullptr, nullptr};
    const float* h3t12 = nullptr;  // Halton table of the device

    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::thread worker;
    bool stopping = false;
    int waiting = 0;  // threads inside csp_server_wait (stop() frees nothing while one is there)
    bool hold = false;  // admission paused (requests queue; active ones finish)
    std::string fatal;

    // statistics
    std::vector<double> latencies;  // seconds, completed requests
    uint64_t rays_done = 0, completed = 0, steps = 0;
    int peak_active = 0;
    bool have_first = false;
    Clock::time_point t_first_submit, t_last_done;

    ~Server();
    int start(int dev, size_t budget_bytes, int max_act, uint64_t step_target);
    void stop();
    int add_scene(const csp_element* el, uint32_t n, uint32_t* id);
    int submit(const SRequest& r, uint64_t* id);
    void run_worker();
    size_t request_bytes(const SRequest& r) const;
    int admit(std::vector<SRequest*>& admitted, std::string& err);
    int step_launch(int par, bool after_other, std::vector<SRequest*>& finishing, uint64_t& rays);
};

Server::~Server() { stop(); }

void Server::stop() {
    {
        std::lock_guard<std::mutex> lk(mu);
        stopping = true;
    }
    cv_work.notify_all();
    if (worker.joinable()) worker.join();
    pool.stop();
    {
        // requests still queued (admission held, or the worker stopped on an error) will never
        // run: fail them, wake their waiters and let every waiter leave before anything is freed
        std::unique_lock<std::mutex> lk(mu);
        for (SRequest* r : pending) {
            r->state = kFailed;
            r->error = "server destroyed before the request was admitted";
            r->error_status = CSP_ERR_STATE;
        }
        pending.clear();
        cv_done.notify_all();
        cv_done.wait(lk, [&] { return waiting == 0; });
    }
    if (device >= 0) cudaSetDevice(device);
    for (cudaStream_t st : stream)
        if (st) cudaStreamSynchronize(st);
    if (adm_stream) cudaStreamSynchronize(adm_stream);
    for (auto& s : scenes) {
        cudaFree(s->d_topo);
        cudaFree(s->d_cells);
        cudaFree(s->d_items);
        cudaFree(s->d_global);
        cudaFree(s->d_prims);
        cudaFree(s->d_optics);
        cudaFree(s->d_aabbs);
        cudaFree(s->d_nodes);
    }
    scenes.clear();
    cudaFree(d_arena);
    for (int p = 0; p < 2; ++p) {
        cudaFree(d_step[p]);
        cudaFree(d_counter[p]);
        if (h_step[p]) cudaFreeHost(h_step[p]);
        d_step[p] = h_step[p] = nullptr;
        d_counter[p] = nullptr;
    }
    cudaFree(d_jobs);
    d_jobs = nullptr;
    if (h_adm) cudaFreeHost(h_adm);
    if (h_res) cudaFreeHost(h_res);
    d_arena = nullptr;
    h_adm = h_res = nullptr;
    if (adm_done) cudaEventDestroy(adm_done);
    adm_done = nullptr;
    if (adm_stream) cudaStreamDestroy(adm_stream);
    adm_stream = nullptr;
    for (int p = 0; p < 2; ++p) {
        if (step_done[p]) cudaEventDestroy(step_done[p]);
        if (stream[p]) cudaStreamDestroy(stream[p]);
        step_done[p] = nullptr;
        stream[p] = nullptr;
    }
}

int Server::start(int dev, size_t budget_bytes, int max_act, uint64_t step_target) {
    device = dev;
    max_active = std::max(1, std::min(max_act, 4096));
    step_rays = std::max<uint64_t>(step_target, 1u << 20);
    int rc = cuda_status(cudaSetDevice(device), "cudaSetDevice");
    if (rc) return rc;
    h3t12 = halton3_table();
    for (int p = 0; p < 2; ++p) {
        if ((rc = cuda_status(cudaStreamCreateWithFlags(&stream[p], cudaStreamNonBlocking), "cudaStreamCreate")))
            return rc;
        if ((rc = cuda_status(cudaEventCreateWithFlags(&step_done[p], cudaEventDisableTiming), "cudaEventCreate")))
            return rc;
    }
    if ((rc = cuda_status(cudaStreamCreateWithFlags(&adm_stream, cudaStreamNonBlocking), "cudaStreamCreate"))) return rc;
    if ((rc = cuda_status(cudaEventCreateWithFlags(&adm_done, cudaEventDisableTiming), "cudaEventCreate"))) return rc;
    pool.start(std::min(7u, std::thread::hardware_concurrency() / 2));
    size_t free_b = 0, total_b = 0;
    if ((rc = cuda_status(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo"))) return rc;
    budget = budget_bytes ? budget_bytes : std::min<size_t>(free_b / 2, (size_t)8 << 30);
    if (budget > free_b) return set_error(CSP_ERR_OUT_OF_MEMORY, "server memory budget exceeds free device memory");
    if ((rc = cuda_status(dev_alloc((void**)&d_arena, budget), "cudaMalloc server arena"))) return rc;
    arena.reset(budget);
    step_bytes = align256((size_t)max_active * sizeof(InstanceDesc)) * kBatchGroups +
                 align256((size_t)(max_active + 1) * sizeof(uint64_t)) * kBatchGroups;
    for (int p = 0; p < 2; ++p) {
        if ((rc = cuda_status(dev_alloc((void**)&d_step[p], step_bytes), "cudaMalloc step tables"))) return rc;
        if ((rc = cuda_status(host_alloc((void**)&h_step[p], step_bytes), "cudaHostAlloc"))) return rc;
        if ((rc = cuda_status(dev_alloc((void**)&d_counter[p], kBatchGroups * sizeof(unsigned long long)),
                              "cudaMalloc")))
            return rc;
    }
    jobs_cap = align256((size_t)max_active * sizeof(RefitJob)) + align256((size_t)max_active * sizeof(SunJob)) +
               align256((size_t)max_active * sizeof(SunGridJob));
    if ((rc = cuda_status(dev_alloc((void**)&d_jobs, jobs_cap), "cudaMalloc job tables"))) return rc;
    res_slot_bytes = align256((size_t)nx * ny * sizeof(uint32_t) + 4 * sizeof(unsigned long long) + sizeof(SunFrame));
    if ((rc = cuda_status(host_alloc((void**)&h_res, res_slot_bytes * max_active),
                          "cudaHostAlloc results")))
        return rc;
    for (int k = max_active - 1; k >= 0; --k) free_res_slots.push_back(k);
    worker = std::thread([this] { run_worker(); });
    return CSP_OK;
}

int Server::add_scene(const csp_element* el, uint32_t n, uint32_t* id) {
    auto s = std::make_unique<SScene>();
    s->elements.assign(el, el + n);
    std::string err;
    int rc = build_elements(el, n, s->base, err);
    if (rc) return set_error(rc, err);
    build_bvh(s->base);
    if (n > kFlatListMax) build_grid(s->base, s->grid);
    s->group = n <= kFlatListMax ? kAccelFlat : (s->grid.valid ? kAccelGrid : kAccelBvh);
    auto put = [&](auto*& dptr, const auto& host, const char* what) {
        const size_t bytes = std::max<size_t>(1, host.size()) * sizeof(host[0]);
        int r = cuda_status(dev_alloc((void**)&dptr, bytes), what);
        if (!r && !host.empty())
            r = cuda_status(cudaMemcpy(dptr, host.data(), host.size() * sizeof(host[0]), cudaMemcpyHostToDevice), what);
        return r;
    };
    rc = put(s->d_topo, s->base.nodes, "upload topology");
    if (!rc) rc = put(s->d_nodes, s->base.nodes, "upload nodes");
    if (!rc) rc = put(s->d_prims, s->base.prims, "upload prims");
    if (!rc) rc = put(s->d_optics, s->base.optics, "upload optics");
    if (!rc) rc = put(s->d_aabbs, s->base.aabbs, "upload aabbs");
    if (!rc && s->grid.valid) rc = put(s->d_cells, s->grid.cell_start, "upload grid cells");
    if (!rc && s->grid.valid) rc = put(s->d_items, s->grid.items, "upload grid items");
    if (!rc && s->grid.valid) rc = put(s->d_global, s->grid.global, "upload grid globals");
    std::lock_guard<std::mutex> lk(mu);
    scenes.push_back(std::move(s));
    if (rc) return rc;
    if (id) *id = (uint32_t)(scenes.size() - 1);
    return CSP_OK;
}

// Arena block of a request, offsets from its start.  Everything the host provides comes first and
// leaves in one upload at admission: the grid descriptor, the flux map and counters (zeros), and
// with per-request poses the element records and the field grid of the poses.  After it, what
// kernels write: the sun frame, the refitted BVH nodes and the sun-ray candidate grid.
struct BlockLayout {
    size_t grid = 0, counts = 0, stats = 0, prims = 0, optics = 0, aabbs = 0, prune = 0, cells = 0, items = 0,
           global = 0, upload = 0, sun = 0, nodes = 0, sgrid = 0, total = 0;
};

static BlockLayout block_layout(const SRequest& r, uint32_t nx, uint32_t ny) {
    const SScene& s = *r.sc;
    const size_t n = s.elements.size();
    BlockLayout L;
    size_t o = 0;
    auto take = [&](size_t& at, size_t bytes) {
        at = o;
        o += align256(bytes);
    };
    take(L.grid, sizeof(GridDesc));
    take(L.counts, (size_t)nx * ny * sizeof(uint32_t));
    take(L.stats, 4 * sizeof(unsigned long long));
    if (!r.poses.empty()) {
        take(L.prims, n * sizeof(Prim));
        take(L.optics, n * sizeof(Optics));
        take(L.aabbs, n * sizeof(Aabb));
        take(L.prune, n * sizeof(Aabb));
        if (r.group == kAccelGrid) {
            take(L.cells, r.grid.cell_start.size() * sizeof(uint32_t));
            take(L.items, r.grid.items.size() * sizeof(Aabb));
            take(L.global, std::max<size_t>(1, r.grid.global.size()) * sizeof(Aabb));
        }
    }
    L.upload = o;
    take(L.sun, sizeof(SunFrame));
    if (!r.poses.empty() && r.group != kAccelGrid) take(L.nodes, s.base.nodes.size() * sizeof(Node));
    if (r.group != kAccelFlat) take(L.sgrid, sungrid_bytes((uint32_t)n));
    L.total = o;
    return L;
}

size_t Server::request_bytes(const SRequest& r) const { return block_layout(r, nx, ny).total; }

int Server::submit(const SRequest& in, uint64_t* id) {
    const SScene* sp = nullptr;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (in.scene < scenes.size()) sp = scenes[in.scene].get();
    }
    if (!sp) return set_error(CSP_ERR_INVALID_ARGUMENT, "no such scene");
    auto r = std::make_unique<SRequest>(in);
    const SScene& s = *sp;
    if (!in.poses.empty()) {
        if (in.poses.size() != s.elements.size())
            return set_error(CSP_ERR_BAD_SCENE, "request poses must have the scene's element count");
        for (size_t k = 0; k < s.elements.size(); ++k)
            if (in.poses[k].surface != s.elements[k].surface || in.poses[k].aperture != s.elements[k].aperture)
                return set_error(CSP_ERR_BAD_SCENE, "request pose " + std::to_string(k) + " changes the surface type");
        // host work of the request, in the submitting thread (the element records of large requests in
        // ranges on the server's host threads): element records and grid of its poses
        std::string err;
        const uint32_t n = (uint32_t)r->poses.size();
        const int rc = n >= 4 * kBuildChunk
                           ? build_elements(r->poses.data(), n, r->hs, err,
                                            [this](size_t tasks, const std::function<void(size_t)>& body) {
                                                pool.run(tasks, body);
                                            })
                           : build_elements(r->poses.data(), n, r->hs, err);
        if (rc) return set_error(rc, err);
        if (s.group != kAccelFlat) build_grid(r->hs, r->grid);
    }
    std::lock_guard<std::mutex> lk(mu);
    if (!fatal.empty()) return set_error(CSP_ERR_CUDA, "server stopped: " + fatal);
    if (!valid_sun_shape(in.shape))
        return set_error(CSP_ERR_INVALID_ARGUMENT, "unknown sun shape");
    if (!(in.param >= 0.0) || in.param > 0.5) return set_error(CSP_ERR_INVALID_ARGUMENT, "sun shape parameter out of range");
    if (in.rays == 0 || in.rays >= (1ull << 40)) return set_error(CSP_ERR_INVALID_ARGUMENT, "bad ray count");
    r->id = next_id++;
    r->out_flags = out_flags;
    r->sc = &s;
    r->group = s.group;
    if (r->group != kAccelFlat && !r->poses.empty()) r->group = r->grid.valid ? kAccelGrid : kAccelBvh;
    r->bytes = request_bytes(*r);
    if (r->bytes > budget) return set_error(CSP_ERR_OUT_OF_MEMORY, "request larger than the server memory budget");
    r->t_submit = Clock::now();
    if (!have_first) {
        have_first = true;
        t_first_submit = r->t_submit;
    }
    if (id) *id = r->id;
    pending.push_back(r.get());
    requests[r->id] = std::move(r);
    cv_work.notify_one();
    return CSP_OK;
}

// Move pending requests into device memory while slots and memory last; queue their uploads,
// refits, sun planes and sun-ray grids on the admission stream.  Called with the lock NOT held.
int Server::admit(std::vector<SRequest*>& admitted, std::string& err) {
    NvtxRange nvtx("csp server admit");
    {
        std::lock_guard<std::mutex> lk(mu);
        while (!hold && !pending.empty() && (int)(active.size() + admitted.size()) < max_active &&
               !free_res_slots.empty()) {
            SRequest* r = pending.front();
            size_t off = 0;
            if (!arena.alloc(r->bytes, off)) break;  // wait for completions to free memory
            pending.pop_front();
            r->off = off;
            r->result_slot = free_res_slots.back();
            free_res_slots.pop_back();
            admitted.push_back(r);
        }
    }
    if (admitted.empty()) return CSP_OK;
    // layout inside each block; the host part of each block is staged (pinned) as it lies in the
    // block and leaves in one upload
    size_t stage = 0;
    std::vector<size_t> stage_off(admitted.size()), upload(admitted.size());
    for (size_t i = 0; i < admitted.size(); ++i) {
        SRequest& r = *admitted[i];
        const BlockLayout L = block_layout(r, nx, ny);
        r.o_grid = r.off + L.grid;
        r.o_counts = r.off + L.counts;
        r.o_stats = r.off + L.stats;
        r.o_prims = r.off + L.prims;
        r.o_optics = r.off + L.optics;
        r.o_aabbs = r.off + L.aabbs;
        r.o_prune = r.off + L.prune;
        r.o_cells = r.off + L.cells;
        r.o_items = r.off + L.items;
        r.o_global = r.off + L.global;
        r.o_sun = r.off + L.sun;
        r.o_nodes = r.off + L.nodes;
        r.o_sgrid = r.off + L.sgrid;
        r.own_records = !r.poses.empty();
        stage_off[i] = stage;
        upload[i] = L.upload;
        stage += align256(L.upload);
    }
    const size_t refit_at = stage;
    stage += align256(admitted.size() * sizeof(RefitJob));
    const size_t sun_at = stage;
    stage += align256(admitted.size() * sizeof(SunJob));
    const size_t sg_at = stage;
    stage += align256(admitted.size() * sizeof(SunGridJob));
    if (stage > adm_cap) {
        // the previous pass's uploads from h_adm finished at the step synchronisation before this call
        if (h_adm) cudaFreeHost(h_adm);
        h_adm = nullptr;
        adm_cap = 0;
        int rc = cuda_status(host_alloc((void**)&h_adm, stage), "cudaHostAlloc admission");
        if (rc == CSP_ERR_OUT_OF_MEMORY) {
            // nothing of this pass is queued yet: its requests fail, the server goes on (the
            // worker releases their blocks and slots after the step)
            std::lock_guard<std::mutex> lk(mu);
            for (SRequest* r : admitted) {
                r->state = kFailed;
                r->error = "no pinned host memory for the request's upload";
                r->error_status = CSP_ERR_OUT_OF_MEMORY;
            }
            return CSP_OK;
        }
        if (rc) return rc;
        adm_cap = stage;
    }
    RefitJob* refits = reinterpret_cast<RefitJob*>(h_adm + refit_at);
    SunJob* suns = reinterpret_cast<SunJob*>(h_adm + sun_at);
    SunGridJob* sgs = reinterpret_cast<SunGridJob*>(h_adm + sg_at);
    int n_refit = 0, n_sun = 0, max_nodes = 0, n_sg = 0, max_sg_n = 0;
    for (size_t i = 0; i < admitted.size(); ++i) {
        SRequest& r = *admitted[i];
        const SScene& s = *r.sc;
        const uint32_t n = (uint32_t)s.elements.size();
        // the block's host part as it lies on the device (offsets relative to the block)
        unsigned char* h = h_adm + stage_off[i];
        auto at = [&](size_t o) { return h + (o - r.off); };
        std::memset(at(r.o_counts), 0, (size_t)nx * ny * sizeof(uint32_t));
        std::memset(at(r.o_stats), 0, 4 * sizeof(unsigned long long));
        const Aabb* d_aabbs = s.d_aabbs;
        if (r.own_records) {
            const HostScene& hs = r.hs;
            std::memcpy(at(r.o_prims), hs.prims.data(), n * sizeof(Prim));
            std::memcpy(at(r.o_optics), hs.optics.data(), n * sizeof(Optics));
            std::memcpy(at(r.o_aabbs), hs.aabbs.data(), n * sizeof(Aabb));
            std::memcpy(at(r.o_prune), hs.prune.data(), n * sizeof(Aabb));
            d_aabbs = reinterpret_cast<const Aabb*>(d_arena + r.o_aabbs);
            if (r.group != kAccelGrid) {
                RefitJob& j = refits[n_refit++];
                j.topo = s.d_topo;
                j.aabbs = d_aabbs;
                j.prune = reinterpret_cast<const Aabb*>(d_arena + r.o_prune);
                j.out = reinterpret_cast<Node*>(d_arena + r.o_nodes);
                j.n_nodes = (int)s.base.nodes.size();
                j.pad = 0;
                max_nodes = std::max(max_nodes, j.n_nodes);
            }
        }
        if (r.group == kAccelGrid) {
            GridDesc g;
            if (r.own_records) {
                const HostGrid& hg = r.grid;
                std::memcpy(at(r.o_cells), hg.cell_start.data(), hg.cell_start.size() * sizeof(uint32_t));
                if (!hg.items.empty()) std::memcpy(at(r.o_items), hg.items.data(), hg.items.size() * sizeof(Aabb));
                if (!hg.global.empty()) std::memcpy(at(r.o_global), hg.global.data(), hg.global.size() * sizeof(Aabb));
                g = grid_desc(hg, reinterpret_cast<const uint32_t*>(d_arena + r.o_cells),
                              reinterpret_cast<const Aabb*>(d_arena + r.o_items),
                              reinterpret_cast<const Aabb*>(d_arena + r.o_global));
            } else {
                g = grid_desc(s.grid, s.d_cells, s.d_items, s.d_global);
            }
            std::memcpy(at(r.o_grid), &g, sizeof g);
        }
        const int rc2 = cuda_status(
            cudaMemcpyAsync(d_arena + r.off, h, upload[i], cudaMemcpyHostToDevice, adm_stream), "upload request");
        if (rc2) return rc2;
        float sv[3];
        sun_vector_f(r.sun, sv);
        SunJob& sj = suns[n_sun++];
        sj.aabbs = d_aabbs;
        sj.n = (int)n;
        sj.sx = sv[0];
        sj.sy = sv[1];
        sj.sz = sv[2];
        sj.tan_pad = tanf((float)sun_pad_angle(r.shape, r.param));
        sj.shape = r.shape;
        sj.param = (float)r.param;
        sj.out = reinterpret_cast<SunFrame*>(d_arena + r.o_sun);
        if (r.group != kAccelFlat) {
            SunGridJob& gj = sgs[n_sg++];
            sungrid_place(d_arena + r.o_sgrid, n, gj);
            gj.sun = sj.out;
            gj.aabbs = d_aabbs;
            max_sg_n = std::max(max_sg_n, (int)n);
        }
        r.t_admit = Clock::now();
    }
    if (n_sun == 0) return CSP_OK;
    // job tables: an arena block released once the stream has passed the kernels that read them
    const size_t job_bytes = stage - refit_at;
    if (job_bytes > jobs_cap) return set_error(CSP_ERR_STATE, "admission job tables exceed their buffer");
    int rc = cuda_status(cudaMemcpyAsync(d_jobs, h_adm + refit_at, job_bytes, cudaMemcpyHostToDevice, adm_stream),
                         "upload admission jobs");
    if (!rc && n_refit)
        rc = cuda_status(launch_refit(reinterpret_cast<const RefitJob*>(d_jobs), n_refit, max_nodes, adm_stream),
                         "refit_kernel");
    if (!rc)
        rc = cuda_status(
            launch_prepare_sun_batch(reinterpret_cast<const SunJob*>(d_jobs + (sun_at - refit_at)), n_sun, adm_stream),
            "prepare_sun_batch_kernel");
    if (!rc && n_sg)
        rc = cuda_status(launch_sungrid_build(reinterpret_cast<const SunGridJob*>(d_jobs + (sg_at - refit_at)), n_sg,
                                              max_sg_n, adm_stream),
                         "sun grid build");
    return rc;
}

// Queue one step over the active requests that have rays left, on stream[par] with the tables of
// parity par; `finishing` receives the requests whose last rays are in it (their results are
// copied behind the launch, and behind the other stream's step when after_other is set: a request
// may have a slice in both).
// Launch parameters of the server's steps per kernel group (element list, BVH, grid): tile/CTA
// size, resident CTAs per SM (0 = occupancy limit), tiles per work grab.  256-ray tiles and 16-tile
// grabs for the element-list and grid groups measured 16 % more served rays/s than 128 / 4 on the
// mixed request workload (fields of 3 to 10,000 heliostats).
constexpr BatchTuning kServeTuning[kBatchGroups] = {{256, 0, 16}, {128, 0, 4}, {256, 0, 16}};

// Smallest slice of an active request in one step (its remaining rays if fewer).  The step's tiles
// run request after request, so with small slices every 16-tile grab of a CTA lands in another
// request than its last one, and each switch drains the CTA's queues in partial batches; a slice
// of 2^24 rays spans ~6 grabs of every resident CTA.  On the mixed request workload (300 requests
// over fields of 3 to 10,000 heliostats, 64 active) it measured 1.86e10 served rays/s at saturation
// against 1.48e10 with 2^20-ray slices, saturation p50 / p99 latency 10.6 / 37 ms against 20.5 /
// 135 ms, and the same latency at 200 requests/s (p50 0.61 ms, p99 6.3 ms), where few requests
// are active and step_rays / active exceeds it anyway.
constexpr uint64_t kMinSlice = 1ull << 24;

int Server::step_launch(int par, bool after_other, std::vector<SRequest*>& finishing, uint64_t& rays) {
    NvtxRange nvtx("csp server step launch");
    rays = 0;
    finishing.clear();
    size_t n_left = 0;
    for (const SRequest* r : active) n_left += r->next_ray < r->rays ? 1 : 0;
    if (n_left == 0) return CSP_OK;
    const uint64_t quantum = std::max<uint64_t>(kMinSlice, step_rays / n_left);
    std::vector<InstanceDesc> desc[kBatchGroups];
    std::vector<uint64_t> tb[kBatchGroups];
    uint64_t tiles[kBatchGroups] = {};
    const size_t desc_stride = align256((size_t)max_active * sizeof(InstanceDesc));
    const size_t tb_base = desc_stride * kBatchGroups;
    const size_t tb_stride = align256((size_t)(max_active + 1) * sizeof(uint64_t));
    for (SRequest* r : active) {
        if (r->next_ray >= r->rays) continue;  // finished in the step still in flight
        const SScene& s = *r->sc;
        const int g = r->group;
        const uint64_t slice = std::min<uint64_t>(quantum, r->rays - r->next_ray);
        if (!r->desc_ready) {
            InstanceDesc& d = r->desc;
            d = InstanceDesc{};
            d.args.nodes = r->own_records && g != kAccelGrid ? reinterpret_cast<const Node*>(d_arena + r->o_nodes)
                                                             : s.d_nodes;
            d.args.prims = r->own_records ? reinterpret_cast<const Prim*>(d_arena + r->o_prims) : s.d_prims;
            d.args.optics = r->own_records ? reinterpret_cast<const Optics*>(d_arena + r->o_optics) : s.d_optics;
            d.args.sun = reinterpret_cast<const SunFrame*>(d_arena + r->o_sun);
            d.args.hits = nullptr;
            d.args.ids = nullptr;
            d.args.seed = r->seed;
            d.args.instance = r->instance;
            d.args.pad = 0;
            d.args.grid = g == kAccelGrid ? reinterpret_cast<const GridDesc*>(d_arena + r->o_grid) : nullptr;
            d.args.h3t12 = h3t12;
            d.args.sgrid = nullptr;
            if (g != kAccelFlat) {
                SunGridJob gj;
                sungrid_place(d_arena + r->o_sgrid, (uint32_t)s.elements.size(), gj);
                d.args.sgrid = gj.desc;
            }
            const csp_element& rcv = (r->poses.empty() ? s.elements : r->poses).back();
            flux_target(rcv, nx, ny, d.flux);
            d.flux.staged = (r->out_flags & CSP_OUT_STAGED) ? 1 : 0;
            d.flux.counts = reinterpret_cast<uint32_t*>(d_arena + r->o_counts);
            d.flux.stats = reinterpret_cast<unsigned long long*>(d_arena + r->o_stats);
            d.n_prims = (int)s.elements.size();
            r->desc_ready = true;
        }
        InstanceDesc d = r->desc;
        d.args.ray_begin = r->next_ray;
        d.args.count = slice;
        d.tile_begin = tiles[g];
        tb[g].push_back(tiles[g]);
        const uint64_t block = (uint64_t)kServeTuning[g].block;
        tiles[g] += (slice + block - 1) / block;
        desc[g].push_back(d);
        r->next_ray += slice;
        rays += slice;
        if (r->next_ray >= r->rays) finishing.push_back(r);
    }
    for (int g = 0; g < kBatchGroups; ++g) {
        tb[g].push_back(tiles[g]);
        if (!desc[g].empty())
            std::memcpy(h_step[par] + desc_stride * g, desc[g].data(), desc[g].size() * sizeof(InstanceDesc));
        std::memcpy(h_step[par] + tb_base + tb_stride * g, tb[g].data(), tb[g].size() * sizeof(uint64_t));
    }
    cudaStream_t st = stream[par];
    int rc = cuda_status(cudaMemcpyAsync(d_step[par], h_step[par], step_bytes, cudaMemcpyHostToDevice, st),
                         "upload step");
    if (!rc)
        rc = cuda_status(cudaMemsetAsync(d_counter[par], 0, kBatchGroups * sizeof(unsigned long long), st), "memset");
    for (int g = 0; g < kBatchGroups && !rc; ++g) {
        if (desc[g].empty()) continue;
        BatchLaunch L;
        L.inst = reinterpret_cast<const InstanceDesc*>(d_step[par] + desc_stride * g);
        L.tile_begin = reinterpret_cast<const uint64_t*>(d_step[par] + tb_base + tb_stride * g);
        L.n_inst = (int)desc[g].size();
        L.chunk = kServeTuning[g].chunk;
        L.total_tiles = tiles[g];
        L.next_tile = d_counter[par] + g;
        rc = cuda_status(launch_trace_batch(L, g, kServeTuning[g], st), "batch_kernel");
    }
    if (!rc && after_other && !finishing.empty())
        rc = cuda_status(cudaStreamWaitEvent(st, step_done[1 - par], 0), "cudaStreamWaitEvent");
    for (SRequest* r : finishing) {
        if (rc) break;
        unsigned char* slot = h_res + res_slot_bytes * r->result_slot;
        rc = cuda_status(cudaMemcpyAsync(slot, d_arena + r->o_counts, (size_t)nx * ny * sizeof(uint32_t),
                                         cudaMemcpyDeviceToHost, st),
                         "D2H flux map");
        if (!rc)
            rc = cuda_status(cudaMemcpyAsync(slot + (size_t)nx * ny * sizeof(uint32_t), d_arena + r->o_stats,
                                             4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st),
                             "D2H stats");
        if (!rc)
            rc = cuda_status(cudaMemcpyAsync(slot + (size_t)nx * ny * sizeof(uint32_t) + 4 * sizeof(unsigned long long),
                                             d_arena + r->o_sun, sizeof(SunFrame), cudaMemcpyDeviceToHost, st),
                             "D2H sun frame");
    }
    return rc;
}

void Server::run_worker() {
    cudaSetDevice(device);
    // the step in flight on the other stream: its finished requests are completed once it ends
    struct InFlight {
        bool valid = false;
        std::vector<SRequest*> finishing;
        uint64_t rays = 0;
    } prev, cur;
    std::vector<SRequest*> admitted;
    bool adm_pending = false;  // an admission pass whose uploads may still be in flight
    int par = 0;
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(mu);
            cv_work.wait(lk, [&] { return stopping || (!pending.empty() && !hold) || !active.empty() || prev.valid; });
            if (stopping && active.empty() && (pending.empty() || hold) && !prev.valid) break;
        }
        std::string err;
        // 1. launch step k on stream[par] over the active requests with rays left; it runs while
        //    step k - 1 (the other stream) finishes
        int rc = step_launch(par, prev.valid, cur.finishing, cur.rays);
        cur.valid = !rc && (cur.rays > 0 || !cur.finishing.empty());
        if (!rc && cur.valid) rc = cuda_status(cudaEventRecord(step_done[par], stream[par]), "cudaEventRecord");
        // 2. admit while it runs (admission stream; its pinned staging is reused only after the last
        //    pass's uploads are done); step k + 1 waits for the admission, so the admitted requests
        //    join it set up
        admitted.clear();
        if (!rc && adm_pending) rc = cuda_status(cudaEventSynchronize(adm_done), "admission");
        adm_pending = false;
        if (!rc) rc = admit(admitted, err);
        if (!rc && !admitted.empty()) {
            rc = cuda_status(cudaEventRecord(adm_done, adm_stream), "cudaEventRecord");
            if (!rc) rc = cuda_status(cudaStreamWaitEvent(stream[1 - par], adm_done, 0), "cudaStreamWaitEvent");
            adm_pending = true;
        }
        if (!rc && !cur.valid && !prev.valid && admitted.empty()) {
            // nothing fits yet (memory) and nothing runs: cannot happen, a request never exceeds
            // the budget; guard against a spin anyway
            std::unique_lock<std::mutex> lk(mu);
            cv_work.wait_for(lk, std::chrono::milliseconds(1));
        }
        // 3. wait for step k - 1 and complete its finished requests
        if (!rc && prev.valid) {
            NvtxRange nvtx("csp server step wait");
            rc = cuda_status(cudaEventSynchronize(step_done[1 - par]), "server step");
        }
        if (!rc && !cur.valid && adm_pending) {
            // nothing launched: let the admission finish before the loop waits for work
            rc = cuda_status(cudaEventSynchronize(adm_done), "admission");
            adm_pending = false;
        }
        const Clock::time_point now = Clock::now();
        std::lock_guard<std::mutex> lk(mu);
        if (rc) {
            fatal = csp_last_error();
            for (SRequest* r : active) {
                r->state = kFailed;
                r->error = fatal;
            }
            for (SRequest* r : admitted) {
                r->state = kFailed;
                r->error = fatal;
            }
            for (SRequest* r : pending) {
                r->state = kFailed;
                r->error = fatal;
            }
            active.clear();
            pending.clear();
            cv_done.notify_all();
            break;
        }
        bool notify = false;
        if (prev.valid) {
            if (prev.rays) ++steps;
            rays_done += prev.rays;
            for (SRequest* r : prev.finishing) {
                const unsigned char* slot = h_res + res_slot_bytes * r->result_slot;
                r->counts.assign(reinterpret_cast<const uint32_t*>(slot),
                                 reinterpret_cast<const uint32_t*>(slot) + (size_t)nx * ny);
                std::memcpy(r->stats, slot + (size_t)nx * ny * sizeof(uint32_t), 4 * sizeof(uint64_t));
                r->stats[0] = r->rays;
                std::memcpy(&r->sunf, slot + (size_t)nx * ny * sizeof(uint32_t) + 4 * sizeof(unsigned long long),
                            sizeof(SunFrame));
                r->state = kDone;
                r->t_done = now;
                t_last_done = now;
                latencies.push_back(std::chrono::duration<double>(r->t_done - r->t_submit).count());
                ++completed;
                arena.release(r->off, r->bytes);
                free_res_slots.push_back(r->result_slot);
                r->result_slot = -1;
                active.erase(std::find(active.begin(), active.end(), r));
                notify = true;
            }
        }
        for (SRequest* r : admitted) {
            if (r->state == kFailed) {
                arena.release(r->off, r->bytes);
                free_res_slots.push_back(r->result_slot);
                notify = true;
                continue;
            }
            r->state = kActive;
            active.push_back(r);
            notify = true;
        }
        peak_active = std::max(peak_active, (int)active.size());
        if (notify) cv_done.notify_all();
        std::swap(prev, cur);
        cur.valid = false;
        cur.finishing.clear();
        cur.rays = 0;
        if (prev.valid) par = 1 - par;
    }
}

}  // namespace csp

using csp::Server;

#define CSP_SGUARD(s)                                                                      \
    do {                                                                                   \
        if (!(s)) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "null server handle");    \
    } while (0)

extern "C" {

int csp_server_create(csp_server* out, int device, uint64_t memory_budget, uint32_t max_active, uint64_t step_rays) {
    if (!out) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "null output handle");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) return csp::cuda_status(e, "cudaGetDeviceCount");
    if (device < 0 || device >= count) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "no such CUDA device");
    Server* s = new (std::nothrow) Server();
    if (!s) return csp::set_error(CSP_ERR_OUT_OF_MEMORY, "host allocation failed");
    const int rc = s->start(device, (size_t)memory_budget, max_active ? (int)max_active : 64,
                            step_rays ? step_rays : (64ull << 20));
    if (rc) {
        delete s;
        return rc;
    }
    *out = reinterpret_cast<csp_server>(s);
    return CSP_OK;
}

int csp_server_destroy(csp_server sh) {
    CSP_SGUARD(sh);
    delete reinterpret_cast<Server*>(sh);
    return CSP_OK;
}

int csp_server_add_scene(csp_server sh, const csp_element* el, uint32_t n, uint32_t* id) {
    CSP_SGUARD(sh);
    if (!el || n == 0) return csp::set_error(CSP_ERR_BAD_SCENE, "scene has no elements");
    return reinterpret_cast<Server*>(sh)->add_scene(el, n, id);
}

int csp_server_submit(csp_server sh, uint32_t scene, const csp_element* poses, const double* sun, int shape,
                      double param, uint64_t rays, uint64_t seed, uint32_t instance, uint64_t* request) {
    CSP_SGUARD(sh);
    if (!sun) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "null sun vector");
    Server* s = reinterpret_cast<Server*>(sh);
    csp::SRequest r;
    r.scene = scene;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (poses && scene < s->scenes.size()) r.poses.assign(poses, poses + s->scenes[scene]->elements.size());
    }
    r.sun[0] = sun[0];
    r.sun[1] = sun[1];
    r.sun[2] = sun[2];
    r.shape = shape;
    r.param = param;
    r.rays = rays;
    r.seed = seed;
    r.instance = instance;
    return s->submit(r, request);
}

int csp_server_set_output(csp_server sh, int flags) {
    CSP_SGUARD(sh);
    if (flags & ~CSP_OUT_STAGED) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "unknown output flags");
    Server* s = reinterpret_cast<Server*>(sh);
    std::lock_guard<std::mutex> lk(s->mu);
    s->out_flags = flags;
    return CSP_OK;
}

int csp_server_hold(csp_server sh, int hold) {
    CSP_SGUARD(sh);
    Server* s = reinterpret_cast<Server*>(sh);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->hold = hold != 0;
    }
    s->cv_work.notify_all();
    return CSP_OK;
}

int csp_server_wait(csp_server sh, uint64_t request, double timeout_s, uint32_t* counts, uint64_t* stats,
                    double* latency_s) {
    CSP_SGUARD(sh);
    Server* s = reinterpret_cast<Server*>(sh);
    std::unique_lock<std::mutex> lk(s->mu);
    // the request is looked up again after every wake-up: another thread waiting on the same id
    // may have taken its results (and freed it) in the meantime
    auto find = [&]() -> csp::SRequest* {
        auto f = s->requests.find(request);
        return f == s->requests.end() ? nullptr : f->second.get();
    };
    if (!find()) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "no such request");
    auto done = [&] {
        const csp::SRequest* q = find();
        return !q || q->state == csp::kDone || q->state == csp::kFailed;
    };
    ++s->waiting;
    bool in_time = true;
    if (timeout_s < 0) s->cv_done.wait(lk, done);
    else in_time = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done);
    if (--s->waiting == 0 && s->stopping) s->cv_done.notify_all();
    if (!in_time) return csp::set_error(CSP_ERR_TIMEOUT, "request not finished within the timeout");
    auto it = s->requests.find(request);
    if (it == s->requests.end())
        return csp::set_error(CSP_ERR_STATE, "the request's results went to another thread waiting on it");
    csp::SRequest* r = it->second.get();
    if (r->state == csp::kFailed) {
        const std::string msg = r->error;
        const int status = r->error_status;
        s->requests.erase(it);
        return csp::set_error(status, "request failed: " + msg);
    }
    if (counts) std::memcpy(counts, r->counts.data(), r->counts.size() * sizeof(uint32_t));
    if (stats) std::memcpy(stats, r->stats, sizeof r->stats);
    if (latency_s) {
        latency_s[0] = std::chrono::duration<double>(r->t_done - r->t_submit).count();
        latency_s[1] = std::chrono::duration<double>(r->t_admit - r->t_submit).count();
    }
    s->requests.erase(it);
    return CSP_OK;
}

int csp_server_stats(csp_server sh, double* out) {
    CSP_SGUARD(sh);
    if (!out) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "null output");
    Server* s = reinterpret_cast<Server*>(sh);
    std::lock_guard<std::mutex> lk(s->mu);
    std::vector<double> l = s->latencies;
    std::sort(l.begin(), l.end());
    auto pct = [&](double p) {
        if (l.empty()) return 0.0;
        const size_t k = (size_t)std::min<double>((double)l.size() - 1, std::ceil(p * l.size()) - 1);
        return l[k];
    };
    const double span = s->completed ? std::chrono::duration<double>(s->t_last_done - s->t_first_submit).count() : 0.0;
    out[0] = (double)s->completed;
    out[1] = (double)s->rays_done;
    out[2] = pct(0.50);
    out[3] = pct(0.99);
    out[4] = span > 0 ? (double)s->rays_done / span : 0.0;
    out[5] = (double)s->peak_active;
    out[6] = (double)s->arena.peak;
    out[7] = (double)s->steps;
    return CSP_OK;
}

}  // extern "C"
