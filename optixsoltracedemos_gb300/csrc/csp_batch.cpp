// csp_batch.cpp -- batched tracing behind csp_batch_* (include/csp_c_api.h).
//
// A run:
//   host    per-instance element builds (the reference's geometry arithmetic, lib/element.cpp and
//           the GeometryDataST constructors, exactly as the single-scene path does it), in
//           parallel threads, written into one pinned staging image of the device arena
//   device  one CUDA graph: upload the image, zero the flux maps and counters, refit every
//           instance's BVH (refit_kernel), compute every instance's sun plane
//           (prepare_sun_batch_kernel) and sun-ray candidate grid (csp_sungrid.cu), trace the
//           small-scene, BVH and grid instances (one persistent batch_kernel launch per group),
//           copy flux maps, counters and sun frames back
// The graph is captured once per batch layout (instances, element counts, ray counts, tuning) and
// re-launched while the layout is unchanged.  Runs are pipelined over two slots (pinned staging and
// result buffers, graph, events): run_async builds the next run on the host while the previous one
// executes, wait completes the oldest run in flight.
//
// Device layout (offsets 16-byte aligned):
//   upload  [per instance: prims | optics | aabbs | prune (| own field grid)] [descs per group]
//           [tile_begin per group] [refit jobs] [sun jobs] [sun grid jobs]
//   nodes   per-instance refitted BVH nodes and sun grid (written on the device)
//   zeroed  [work counters (2)] [stats, 4 x u64 per instance] [counts, nx*ny x u32 per instance]
//   suns    per-instance SunFrame
// The upload region is one copy into the run slot's own device buffer, on the copy stream, so that
// it overlaps the kernels of the run before; the rest is one buffer shared by the runs, whose
// kernels are ordered on the compute stream.  The download region is [stats .. suns end), one copy.
#include "csp_batch.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <tuple>

#include "csp_math.cuh"
#include "csp_system.h"

namespace csp {
namespace {

size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

// Tuned launch parameters per (device model, kernel build, kernel group, ray-count class), shared
// by every batch of the process and, when a cache file is set (csp_set_tune_cache, or the
// CSP_TUNE_CACHE environment variable), by every process that uses that file.  The device model is
// "name ccM.m smN"; the kernel build is a fingerprint of both block sizes' register, shared and
// local memory use, so a rebuilt kernel is tuned afresh.
struct TuneKey {
    std::string device;
    uint32_t build = 0;
    int group = 0, cls = 0;
    bool operator<(const TuneKey& o) const {
        return std::tie(device, build, group, cls) < std::tie(o.device, o.build, o.group, o.cls);
    }
};
std::mutex g_tune_mu;
std::map<TuneKey, BatchTuning> g_tune_cache;
std::string g_tune_path;
bool g_tune_path_set = false;  // set by the API or taken from the environment at first use

// "key": "string" or "key": integer on one line of the cache file.
bool json_str(const char* line, const char* key, std::string& out) {
    const char* p = std::strstr(line, key);
    if (!p) return false;
    p = std::strchr(p + std::strlen(key), '"');
    if (!p) return false;
    const char* q = std::strchr(p + 1, '"');
    if (!q) return false;
    out.assign(p + 1, q);
    return true;
}

bool json_int(const char* line, const char* key, long long& out) {
    const char* p = std::strstr(line, key);
    if (!p) return false;
    p = std::strchr(p + std::strlen(key), ':');
    if (!p) return false;
    char* end = nullptr;
    out = std::strtoll(p + 1, &end, 10);
    return end != p + 1;
}

// Entries of a cache file into g_tune_cache (caller holds g_tune_mu); malformed entries are skipped.
void tune_load_locked(const std::string& path) {
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) return;
    char line[1024];
    while (std::fgets(line, sizeof line, f)) {
        TuneKey k;
        long long build, group, cls, block, ctas, chunk;
        if (!json_str(line, "\"device\"", k.device) || !json_int(line, "\"build\"", build) ||
            !json_int(line, "\"group\"", group) || !json_int(line, "\"ray_class\"", cls) ||
            !json_int(line, "\"block\"", block) || !json_int(line, "\"ctas_per_sm\"", ctas) ||
            !json_int(line, "\"chunk\"", chunk))
            continue;
        if (group < 0 || group >= kBatchGroups || (block != 128 && block != 256) || ctas < 0 || ctas > 64 ||
            chunk < 1 || chunk > 1 << 20)
            continue;
        k.build = (uint32_t)build;
        k.group = (int)group;
        k.cls = (int)cls;
        g_tune_cache[k] = BatchTuning{(int)block, (int)ctas, (int)chunk};
    }
    std::fclose(f);
}

// The whole cache to the file (caller holds g_tune_mu): written to a temporary file next to it and
// renamed over it, so a reader never sees half a file.
void tune_save_locked() {
    if (g_tune_path.empty()) return;
    const std::string tmp = g_tune_path + ".tmp." + std::to_string((unsigned long long)std::hash<std::thread::id>()(
                                                         std::this_thread::get_id()));
    FILE* f = std::fopen(tmp.c_str(), "w");
    if (!f) return;  // an unwritable cache only costs the next process its tuning runs
    std::fprintf(f, "{\"format\": \"csp_gb300 batch tuning cache\", \"version\": 1, \"entries\": [\n");
    size_t i = 0;
    for (const auto& kv : g_tune_cache) {
        std::fprintf(f,
                     "  {\"device\": \"%s\", \"build\": %u, \"group\": %d, \"ray_class\": %d, \"block\": %d, "
                     "\"ctas_per_sm\": %d, \"chunk\": %d}%s\n",
                     kv.first.device.c_str(), kv.first.build, kv.first.group, kv.first.cls, kv.second.block,
                     kv.second.ctas_per_sm, kv.second.chunk, ++i < g_tune_cache.size() ? "," : "");
    }
    std::fprintf(f, "]}\n");
    const bool ok = std::fclose(f) == 0;
    if (!ok || std::rename(tmp.c_str(), g_tune_path.c_str()) != 0) std::remove(tmp.c_str());
}

// First use: the file named by CSP_TUNE_CACHE, unless the API chose one (caller holds g_tune_mu).
void tune_init_locked() {
    if (g_tune_path_set) return;
    g_tune_path_set = true;
    const char* env = std::getenv("CSP_TUNE_CACHE");
    if (env && *env) {
        g_tune_path = env;
        tune_load_locked(g_tune_path);
    }
}

int ray_class(uint64_t mean_rays) {
    int c = 0;
    while (mean_rays > 1 && c < 63) {
        mean_rays >>= 1;
        ++c;
    }
    return c / 2;  // factors of 4
}

}  // namespace

Batch::~Batch() { release(); }

void Batch::release() {
    if (device >= 0) cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);  // runs in flight read the arena and the slots
    flight.clear();
    cur = -1;
    for (RunSlot& S : slot) {
        if (S.graph) cudaGraphExecDestroy(S.graph);
        S.graph = nullptr;
        if (S.h_stage) cudaFreeHost(S.h_stage);
        if (S.h_result) cudaFreeHost(S.h_result);
        S.h_stage = S.h_result = nullptr;
        S.stage_cap = S.result_cap = 0;
        if (S.ev0) cudaEventDestroy(S.ev0);
        if (S.ev1) cudaEventDestroy(S.ev1);
        if (S.done) cudaEventDestroy(S.done);
        if (S.up_done) cudaEventDestroy(S.up_done);
        S.ev0 = S.ev1 = S.done = S.up_done = nullptr;
        cudaFree(S.d_up);
        S.d_up = nullptr;
        S.up_cap = 0;
    }
    d_up = nullptr;
    h_stage = nullptr;
    for (BScene& s : scenes) {
        cudaFree(s.d_topo);
        cudaFree(s.d_cells);
        cudaFree(s.d_items);
        cudaFree(s.d_global);
        s.d_topo = nullptr;
        s.d_cells = nullptr;
        s.d_items = s.d_global = nullptr;
    }
    cudaFree(d_comp);
    d_comp = nullptr;
    comp_cap = 0;
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
    if (copy_stream) cudaStreamDestroy(copy_stream);
    ev0 = ev1 = nullptr;
    stream = copy_stream = nullptr;
}

int Batch::ensure_stream() {
    if (stream) return CSP_OK;
    int rc = cuda_status(cudaSetDevice(device), "cudaSetDevice");
    if (rc) return rc;
    cudaDeviceProp prop;
    if ((rc = cuda_status(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties"))) return rc;
    device_model = std::string(prop.name) + " cc" + std::to_string(prop.major) + "." + std::to_string(prop.minor) +
                   " sm" + std::to_string(prop.multiProcessorCount);
    for (char& c : device_model)
        if (c == '"' || c == '\\') c = '_';
    h3t12 = halton3_table();
    if ((rc = cuda_status(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate"))) return rc;
    if ((rc = cuda_status(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking), "cudaStreamCreate")))
        return rc;
    if ((rc = cuda_status(cudaEventCreate(&ev0), "cudaEventCreate"))) return rc;
    if ((rc = cuda_status(cudaEventCreate(&ev1), "cudaEventCreate"))) return rc;
    for (RunSlot& S : slot) {
        if ((rc = cuda_status(cudaEventCreate(&S.ev0), "cudaEventCreate"))) return rc;
        if ((rc = cuda_status(cudaEventCreate(&S.ev1), "cudaEventCreate"))) return rc;
        if ((rc = cuda_status(cudaEventCreateWithFlags(&S.done, cudaEventDisableTiming), "cudaEventCreate"))) return rc;
        if ((rc = cuda_status(cudaEventCreateWithFlags(&S.up_done, cudaEventDisableTiming), "cudaEventCreate")))
            return rc;
    }
    return CSP_OK;
}

int Batch::add_scene(const csp_element* el, uint32_t n, uint32_t* id) {
    int rc = ensure_stream();
    if (rc) return rc;
    BScene s;
    s.elements.assign(el, el + n);
    std::string err;
    if ((rc = build_elements(el, n, s.base, err))) return set_error(rc, err);
    build_bvh(s.base);
    s.flat = n <= kFlatListMax;
    if (!s.flat) build_grid(s.base, s.grid);
    auto put = [&](auto*& dptr, const auto& host, const char* what) {
        const size_t bytes = std::max<size_t>(1, host.size()) * sizeof(host[0]);
        int r = cuda_status(dev_alloc((void**)&dptr, bytes), what);
        if (!r && !host.empty())
            r = cuda_status(cudaMemcpy(dptr, host.data(), host.size() * sizeof(host[0]), cudaMemcpyHostToDevice), what);
        return r;
    };
    rc = put(s.d_topo, s.base.nodes, "upload topology");
    if (!rc && s.grid.valid) rc = put(s.d_cells, s.grid.cell_start, "upload grid cells");
    if (!rc && s.grid.valid) rc = put(s.d_items, s.grid.items, "upload grid items");
    if (!rc && s.grid.valid) rc = put(s.d_global, s.grid.global, "upload grid globals");
    if (rc) {
        cudaFree(s.d_topo);
        cudaFree(s.d_cells);
        cudaFree(s.d_items);
        cudaFree(s.d_global);
        return rc;
    }
    scenes.push_back(std::move(s));
    if (id) *id = (uint32_t)(scenes.size() - 1);
    return CSP_OK;
}

int Batch::add_instance(const BInst& bi, uint32_t* index) {
    if (bi.scene >= scenes.size()) return set_error(CSP_ERR_INVALID_ARGUMENT, "no such scene");
    const BScene& s = scenes[bi.scene];
    if (!bi.poses.empty()) {
        if (bi.poses.size() != s.elements.size())
            return set_error(CSP_ERR_BAD_SCENE, "instance poses must have the scene's element count");
        for (size_t k = 0; k < s.elements.size(); ++k)
            if (bi.poses[k].surface != s.elements[k].surface || bi.poses[k].aperture != s.elements[k].aperture)
                return set_error(CSP_ERR_BAD_SCENE, "instance pose " + std::to_string(k) + " changes the surface type");
    }
    if (!valid_sun_shape(bi.shape))
        return set_error(CSP_ERR_INVALID_ARGUMENT, "unknown sun shape");
    if (!(bi.param >= 0.0) || bi.param > 0.5) return set_error(CSP_ERR_INVALID_ARGUMENT, "sun shape parameter out of range");
    if (bi.rays >= (1ull << 40)) return set_error(CSP_ERR_INVALID_ARGUMENT, "too many rays for one instance");
    inst.push_back(bi);
    if (index) *index = (uint32_t)(inst.size() - 1);
    return CSP_OK;
}

const csp_element* Batch::elements_of(size_t i) const {
    return inst[i].poses.empty() ? scenes[inst[i].scene].elements.data() : inst[i].poses.data();
}

uint32_t Batch::count_of(size_t i) const { return (uint32_t)scenes[inst[i].scene].elements.size(); }

// Offsets of every region; grows the arena and the pinned buffers when needed.
int Batch::layout(int si) {
    const size_t n = inst.size();
    place.assign(n, Place{});
    for (int g = 0; g < kBatchGroups; ++g) n_group[g] = 0;
    max_nodes = 0;
    n_sg = 0;
    max_sg_n = 0;
    size_t off = 0;
    for (size_t i = 0; i < n; ++i) {
        const BScene& s = scenes[inst[i].scene];
        const size_t ne = s.elements.size();
        Place& p = place[i];
        p.group = s.flat ? kAccelFlat : (grid_of(i).valid ? kAccelGrid : kAccelBvh);
        p.slot = n_group[p.group]++;
        p.prims = off;
        off += align16(ne * sizeof(Prim));
        p.optics = off;
        off += align16(ne * sizeof(Optics));
        p.aabbs = off;
        off += align16(ne * sizeof(Aabb));
        p.prune = off;
        off += align16(ne * sizeof(Aabb));
        if (p.group == kAccelGrid && !inst[i].poses.empty()) {
            const HostGrid& hg = builds[i].grid;
            p.cells = off;
            off += align16(hg.cell_start.size() * sizeof(uint32_t));
            p.items = off;
            off += align16(hg.items.size() * sizeof(Aabb));
            p.global = off;
            off += align16(std::max<size_t>(1, hg.global.size()) * sizeof(Aabb));
        }
        max_nodes = std::max(max_nodes, (int)s.base.nodes.size());
        if (p.group != kAccelFlat) {
            p.sg_slot = n_sg++;
            max_sg_n = std::max(max_sg_n, (int)ne);
        }
    }
    for (int g = 0; g < kBatchGroups; ++g) {
        desc_off[g] = off;
        off += align16(n_group[g] * sizeof(InstanceDesc));
    }
    for (int g = 0; g < kBatchGroups; ++g) {
        tb_off[g] = off;
        off += align16((n_group[g] + 1) * sizeof(uint64_t));
    }
    refit_off = off;
    off += align16(n * sizeof(RefitJob));
    sunjob_off = off;
    off += align16(n * sizeof(SunJob));
    sgjob_off = off;
    off += align16((size_t)n_sg * sizeof(SunGridJob));
    up_bytes = off;
    for (size_t i = 0; i < n; ++i) {
        place[i].nodes = off;
        off += align16(scenes[inst[i].scene].base.nodes.size() * sizeof(Node));
        if (place[i].sg_slot >= 0) {
            place[i].sgrid = off;
            off += align16(sungrid_bytes(count_of(i)));
        }
    }
    zero_off = off;
    counter_off = off;
    off += align16(kBatchGroups * sizeof(unsigned long long));
    res_off = off;
    for (size_t i = 0; i < n; ++i) {
        place[i].stats = off;
        off += 4 * sizeof(unsigned long long);
    }
    const size_t nb = (size_t)nx * ny;
    for (size_t i = 0; i < n; ++i) {
        place[i].counts = off;
        off += align16(nb * sizeof(uint32_t));
    }
    zero_bytes = off - zero_off;
    for (size_t i = 0; i < n; ++i) {
        place[i].sun = off;
        off += align16(sizeof(SunFrame));
    }
    res_bytes = off - res_off;
    const size_t comp = std::max<size_t>(off - up_bytes, 16);

    int rc;
    RunSlot& S = slot[si];
    if (comp > comp_cap) {
        // the runs in flight use the shared region: let them finish (their results stay in their slots)
        if (!flight.empty() && (rc = cuda_status(cudaStreamSynchronize(stream), "batch run"))) return rc;
        for (RunSlot& o : slot) {
            if (o.graph) cudaGraphExecDestroy(o.graph);
            o.graph = nullptr;
        }
        cudaFree(d_comp);
        d_comp = nullptr;
        comp_cap = 0;
        size_t free_b = 0, total_b = 0;
        cudaMemGetInfo(&free_b, &total_b);
        if (comp > free_b) return set_error(CSP_ERR_OUT_OF_MEMORY, "batch does not fit in free device memory");
        if ((rc = cuda_status(dev_alloc((void**)&d_comp, comp), "cudaMalloc batch arena"))) return rc;
        comp_cap = comp;
    }
    if (up_bytes > S.up_cap) {
        // the slot is not in flight: nothing reads its upload region
        if (S.graph) cudaGraphExecDestroy(S.graph);
        S.graph = nullptr;
        cudaFree(S.d_up);
        S.d_up = nullptr;
        S.up_cap = 0;
        size_t free_b = 0, total_b = 0;
        cudaMemGetInfo(&free_b, &total_b);
        if (up_bytes > free_b) return set_error(CSP_ERR_OUT_OF_MEMORY, "batch does not fit in free device memory");
        if ((rc = cuda_status(dev_alloc((void**)&S.d_up, std::max<size_t>(up_bytes, 16)), "cudaMalloc batch upload")))
            return rc;
        S.up_cap = up_bytes;
    }
    d_up = S.d_up;
    // the slot is not in flight; if it holds the current results, this run replaces them
    if (up_bytes > S.stage_cap || res_bytes > S.result_cap) {
        if (S.graph) cudaGraphExecDestroy(S.graph);
        S.graph = nullptr;
        if (si == cur) cur = -1;
    }
    if (up_bytes > S.stage_cap) {
        if (S.h_stage) cudaFreeHost(S.h_stage);
        S.h_stage = nullptr;
        S.stage_cap = 0;
        if ((rc = cuda_status(host_alloc((void**)&S.h_stage, up_bytes), "cudaHostAlloc staging")))
            return rc;
        S.stage_cap = up_bytes;
    }
    if (res_bytes > S.result_cap) {
        if (S.h_result) cudaFreeHost(S.h_result);
        S.h_result = nullptr;
        S.result_cap = 0;
        if ((rc = cuda_status(host_alloc((void**)&S.h_result, std::max<size_t>(res_bytes, 16)), "cudaHostAlloc results")))
            return rc;
        S.result_cap = res_bytes;
    }
    h_stage = S.h_stage;
    return CSP_OK;
}

// Host build of an instance with its own poses: element records (the reference's geometry
// arithmetic) and, for field-like scenes, the grid of those poses.
int Batch::build_instance(size_t i, std::string& err) {
    const BInst& b = inst[i];
    if (b.poses.empty()) return CSP_OK;
    InstBuild& ib = builds[i];
    int rc = build_elements(b.poses.data(), count_of(i), ib.hs, err);
    if (rc) return rc;
    ib.grid = HostGrid{};
    if (!scenes[b.scene].flat) build_grid(ib.hs, ib.grid);
    return CSP_OK;
}

const HostScene& Batch::scene_of(size_t i) const {
    return inst[i].poses.empty() ? scenes[inst[i].scene].base : builds[i].hs;
}

const HostGrid& Batch::grid_of(size_t i) const {
    return inst[i].poses.empty() ? scenes[inst[i].scene].grid : builds[i].grid;
}

// Instance i into the staging image: element records, own grid arrays, refit job, sun job.
void Batch::fill_instance(size_t i) {
    const BInst& b = inst[i];
    const Place& p = place[i];
    const BScene& s = scenes[b.scene];
    const uint32_t ne = count_of(i);
    const HostScene* src = &scene_of(i);
    std::memcpy(h_stage + p.prims, src->prims.data(), ne * sizeof(Prim));
    std::memcpy(h_stage + p.optics, src->optics.data(), ne * sizeof(Optics));
    std::memcpy(h_stage + p.aabbs, src->aabbs.data(), ne * sizeof(Aabb));
    std::memcpy(h_stage + p.prune, src->prune.data(), ne * sizeof(Aabb));
    if (p.group == kAccelGrid && !b.poses.empty()) {
        const HostGrid& hg = builds[i].grid;
        std::memcpy(h_stage + p.cells, hg.cell_start.data(), hg.cell_start.size() * sizeof(uint32_t));
        std::memcpy(h_stage + p.items, hg.items.data(), hg.items.size() * sizeof(Aabb));
        if (!hg.global.empty()) std::memcpy(h_stage + p.global, hg.global.data(), hg.global.size() * sizeof(Aabb));
    }
    RefitJob rj;
    rj.topo = s.d_topo;
    rj.aabbs = reinterpret_cast<const Aabb*>(dev(p.aabbs));
    rj.prune = reinterpret_cast<const Aabb*>(dev(p.prune));
    rj.out = reinterpret_cast<Node*>(dev(p.nodes));
    rj.n_nodes = (int)s.base.nodes.size();
    rj.pad = 0;
    std::memcpy(h_stage + refit_off + i * sizeof(RefitJob), &rj, sizeof rj);
    float sv[3];
    sun_vector_f(b.sun, sv);
    SunJob sj;
    sj.aabbs = rj.aabbs;
    sj.n = (int)ne;
    sj.sx = sv[0];
    sj.sy = sv[1];
    sj.sz = sv[2];
    sj.tan_pad = tanf((float)sun_pad_angle(b.shape, b.param));
    sj.shape = b.shape;
    sj.param = (float)b.param;
    sj.out = reinterpret_cast<SunFrame*>(dev(p.sun));
    std::memcpy(h_stage + sunjob_off + i * sizeof(SunJob), &sj, sizeof sj);
    if (p.sg_slot >= 0) {
        SunGridJob gj;
        sungrid_place(dev(p.sgrid), ne, gj);
        gj.sun = sj.out;
        gj.aabbs = rj.aabbs;
        std::memcpy(h_stage + sgjob_off + (size_t)p.sg_slot * sizeof(SunGridJob), &gj, sizeof gj);
    }
}

// Instance descriptors and tile tables of both groups for the given tile sizes; `sample` (the
// autotuner's): the instances traced whole, the others get no rays; nullptr = all of every instance.
void Batch::fill_descs(const int* block, const std::vector<bool>* sample, std::vector<InstanceDesc>* out_desc,
                       std::vector<uint64_t>* out_tb) {
    const size_t n = inst.size();
    for (int g = 0; g < kBatchGroups; ++g) {
        out_desc[g].assign(n_group[g], InstanceDesc{});
        out_tb[g].assign(n_group[g] + 1, 0);
    }
    uint64_t tiles[kBatchGroups] = {};
    for (size_t i = 0; i < n; ++i) {
        const BInst& b = inst[i];
        const Place& p = place[i];
        const int g = p.group;
        uint64_t rays = b.rays;
        if (sample && !(*sample)[i]) rays = 0;
        InstanceDesc& d = out_desc[g][p.slot];
        d.args.nodes = reinterpret_cast<const Node*>(dev(p.nodes));
        d.args.prims = reinterpret_cast<const Prim*>(dev(p.prims));
        d.args.optics = reinterpret_cast<const Optics*>(dev(p.optics));
        d.args.sun = reinterpret_cast<const SunFrame*>(dev(p.sun));
        d.args.hits = nullptr;
        d.args.ids = nullptr;
        d.args.ray_begin = 0;
        d.args.count = rays;
        d.args.seed = b.seed;
        d.args.instance = b.instance;
        d.args.pad = 0;
        d.args.grid = nullptr;
        d.args.h3t12 = h3t12;
        d.args.sgrid = nullptr;
        if (p.sg_slot >= 0) {
            SunGridJob gj;
            sungrid_place(dev(p.sgrid), count_of(i), gj);
            d.args.sgrid = gj.desc;
        }
        if (g == kAccelGrid) {
            const bool own = !b.poses.empty();
            const BScene& bs = scenes[b.scene];
            d.grid = grid_desc(grid_of(i), own ? reinterpret_cast<const uint32_t*>(dev(p.cells)) : bs.d_cells,
                               own ? reinterpret_cast<const Aabb*>(dev(p.items)) : bs.d_items,
                               own ? reinterpret_cast<const Aabb*>(dev(p.global)) : bs.d_global);
            d.args.grid = reinterpret_cast<const GridDesc*>(dev(desc_off[g] + p.slot * sizeof(InstanceDesc)) +
                                                            offsetof(InstanceDesc, grid));
        }
        flux_target(elements_of(i)[count_of(i) - 1], nx, ny, d.flux);
        d.flux.staged = (out_flags & CSP_OUT_STAGED) ? 1 : 0;
        d.flux.counts = reinterpret_cast<uint32_t*>(dev(p.counts));
        d.flux.stats = reinterpret_cast<unsigned long long*>(dev(p.stats));
        d.tile_begin = tiles[g];
        d.n_prims = (int)count_of(i);
        out_tb[g][p.slot] = tiles[g];
        tiles[g] += (rays + block[g] - 1) / block[g];
    }
    for (int g = 0; g < kBatchGroups; ++g) out_tb[g][n_group[g]] = tiles[g];
}

void Batch::write_descs(const std::vector<InstanceDesc>* desc, const std::vector<uint64_t>* tb, unsigned char* img) {
    for (int g = 0; g < kBatchGroups; ++g) {
        if (!desc[g].empty()) std::memcpy(img + desc_off[g], desc[g].data(), desc[g].size() * sizeof(InstanceDesc));
        std::memcpy(img + tb_off[g], tb[g].data(), tb[g].size() * sizeof(uint64_t));
    }
}

BatchLaunch Batch::launch_of(int g, uint64_t total_tiles, int chunk) const {
    BatchLaunch L;
    L.inst = reinterpret_cast<const InstanceDesc*>(dev(desc_off[g]));
    L.tile_begin = reinterpret_cast<const uint64_t*>(dev(tb_off[g]));
    L.n_inst = n_group[g];
    L.chunk = chunk;
    L.total_tiles = total_tiles;
    L.next_tile = reinterpret_cast<unsigned long long*>(dev(counter_off)) + g;
    return L;
}

// Device work of a run up to (not including) the trace launches.
int Batch::enqueue_upload(cudaStream_t st) {
    return cuda_status(cudaMemcpyAsync(d_up, h_stage, up_bytes, cudaMemcpyHostToDevice, st), "upload batch");
}

int Batch::enqueue_zero(cudaStream_t st) {
    return cuda_status(cudaMemsetAsync(dev(zero_off), 0, zero_bytes, st), "zero flux maps");
}

int Batch::enqueue_scene_setup(cudaStream_t st) {
    int rc;
    if ((rc = cuda_status(launch_refit(reinterpret_cast<const RefitJob*>(dev(refit_off)), (int)inst.size(),
                                       max_nodes, st),
                          "refit_kernel")))
        return rc;
    if ((rc = cuda_status(launch_prepare_sun_batch(reinterpret_cast<const SunJob*>(dev(sunjob_off)),
                                                   (int)inst.size(), st),
                          "prepare_sun_batch_kernel")))
        return rc;
    return cuda_status(launch_sungrid_build(reinterpret_cast<const SunGridJob*>(dev(sgjob_off)), n_sg, max_sg_n, st),
                       "sun grid build");
}

// Time the candidate launch parameters of group g on a sample of its instances and keep the
// fastest.  Needs the scene setup on the device (prefix + refit + sun frames) done.
int Batch::autotune(int g, BatchTuning& best) {
    NvtxRange nvtx("csp batch autotune");
    std::vector<BatchTuning> cands;
    for (int block : {128, 256}) {
        const int occ = batch_occupancy(g, block);
        if (occ <= 0) continue;
        std::vector<int> ctas = {occ};
        if (occ > 1) ctas.push_back(std::max(1, occ * 2 / 3));
        // grabs are guided (they shrink as the work runs out), so their cap is not tuned: 256 tiles
        // measured 2.2 % faster than the best of 1 / 4 / 16 / 64 on the 256-instance field batch,
        // where a sample of whole instances sees too few instance switches to tell them apart
        for (int c : ctas) cands.push_back(BatchTuning{block, c, 256});
    }
    if (cands.empty()) return set_error(CSP_ERR_CUDA, "no launchable configuration of the batch kernel");
    // the sample: whole instances of the group, spread over the batch, until the ray budget of a
    // candidate is reached (whole instances, so that the grabs and instance switches of a candidate
    // are the full run's)
    const double budget = g == kAccelFlat ? 256e6 : (g == kAccelGrid ? 96e6 : 32e6);  // rays per candidate
    std::vector<size_t> members;
    for (size_t i = 0; i < inst.size(); ++i)
        if (place[i].group == g) members.push_back(i);
    std::vector<bool> sample(inst.size(), false);
    {
        // members in bit-reversed order of their position: any prefix is spread over the batch
        std::vector<std::pair<uint32_t, size_t>> order;
        for (size_t k = 0; k < members.size(); ++k) {
            uint32_t r = 0;
            for (int b = 0; b < 32; ++b) r |= (uint32_t)((k >> b) & 1u) << (31 - b);
            order.emplace_back(r, members[k]);
        }
        std::sort(order.begin(), order.end());
        double taken = 0.0;
        for (const auto& o : order) {
            if (taken >= budget) break;
            sample[o.second] = true;
            taken += (double)inst[o.second].rays;
        }
    }
    std::vector<unsigned char> img(up_bytes);
    double best_ms = 1e30;
    int rc = CSP_OK;
    for (const BatchTuning& t : cands) {
        const int block[kBatchGroups] = {t.block, t.block, t.block};
        std::vector<InstanceDesc> desc[kBatchGroups];
        std::vector<uint64_t> tb[kBatchGroups];
        fill_descs(block, &sample, desc, tb);
        // descs and tile tables only: the element records already on the device stay
        const size_t lo = desc_off[0], hi = refit_off;
        write_descs(desc, tb, img.data());
        if ((rc = cuda_status(cudaMemcpyAsync(dev(lo), img.data() + lo, hi - lo, cudaMemcpyHostToDevice, stream),
                              "upload sample descs")))
            break;
        const BatchLaunch L = launch_of(g, tb[g][n_group[g]], t.chunk);
        float ms_best = 1e30f;
        for (int rep = 0; rep < 2 && rc == CSP_OK; ++rep) {
            rc = cuda_status(cudaMemsetAsync(dev(counter_off), 0, kBatchGroups * sizeof(unsigned long long), stream),
                             "zero counters");
            if (!rc) rc = cuda_status(cudaEventRecord(ev0, stream), "cudaEventRecord");
            if (!rc) rc = cuda_status(launch_trace_batch(L, g, t, stream), "batch_kernel");
            if (!rc) rc = cuda_status(cudaEventRecord(ev1, stream), "cudaEventRecord");
            if (!rc) rc = cuda_status(cudaEventSynchronize(ev1), "autotune");
            float ms = 0.f;
            if (!rc) cudaEventElapsedTime(&ms, ev0, ev1);
            ms_best = std::min(ms_best, ms);
        }
        if (rc) break;
        if (ms_best < best_ms) {
            best_ms = ms_best;
            best = t;
        }
    }
    return rc;
}

int Batch::resolve_tuning() {
    uint64_t rays[kBatchGroups] = {};
    for (size_t i = 0; i < inst.size(); ++i) rays[place[i].group] += inst[i].rays;
    bool need_setup = true;
    for (int g = 0; g < kBatchGroups; ++g) {
        if (n_group[g] == 0) {
            used[g] = BatchTuning{128, 0, 4};
            continue;
        }
        if (user.block != 0) {
            if (batch_occupancy(g, user.block) <= 0)
                return set_error(CSP_ERR_INVALID_ARGUMENT, "unsupported batch block size");
            used[g] = user;
            continue;
        }
        TuneKey key;
        key.device = device_model;
        key.build = batch_kernel_build(g);
        key.group = g;
        key.cls = ray_class(rays[g] / (uint64_t)n_group[g]);
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            tune_init_locked();
            auto it = g_tune_cache.find(key);
            if (it != g_tune_cache.end()) {
                used[g] = it->second;
                continue;
            }
        }
        int rc;
        if (need_setup) {
            if ((rc = enqueue_upload(stream)) || (rc = enqueue_zero(stream)) || (rc = enqueue_scene_setup(stream)))
                return rc;
            need_setup = false;
        }
        BatchTuning best{128, 0, 4};
        if ((rc = autotune(g, best))) return rc;
        used[g] = best;
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = best;
        tune_save_locked();
    }
    return CSP_OK;
}

int Batch::run_async() {
    NvtxRange nvtx("csp batch build and launch");
    if (inst.empty()) return set_error(CSP_ERR_STATE, "batch has no instances");
    if (flight.size() >= 2) return set_error(CSP_ERR_STATE, "two runs in flight: wait for one first");
    const auto t0 = std::chrono::steady_clock::now();
    int rc = ensure_stream();
    if (rc) return rc;
    // the slot not in flight (with none in flight, the one without the current results)
    const int si = flight.empty() ? (cur == 0 ? 1 : 0) : 1 - flight.front();
    if (si == cur) cur = -1;  // this run's download replaces those results
    RunSlot& S = slot[si];

    // host builds of the instances with their own poses, then the copies into the staging image,
    // both parallel over instances
    const size_t n = inst.size();
    builds.clear();
    builds.resize(n);
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t workers = std::min<size_t>(std::min<size_t>(hw, 64), n);
    auto parallel = [&](auto&& fn) {
        std::vector<int> wrc(workers, CSP_OK);
        std::vector<std::string> werr(workers);
        auto work = [&](size_t w) {
            for (size_t i = w; i < n; i += workers) {
                const int r = fn(i, werr[w]);
                if (r) {
                    wrc[w] = r;
                    werr[w] = "instance " + std::to_string(i) + ": " + werr[w];
                    return;
                }
            }
        };
        if (workers <= 1) work(0);
        else {
            std::vector<std::thread> th;
            for (size_t w = 0; w < workers; ++w) th.emplace_back(work, w);
            for (auto& t : th) t.join();
        }
        for (size_t w = 0; w < workers; ++w)
            if (wrc[w]) return set_error(wrc[w], werr[w]);
        return (int)CSP_OK;
    };
    if ((rc = parallel([&](size_t i, std::string& err) { return build_instance(i, err); }))) return rc;
    if ((rc = layout(si))) return rc;
    if ((rc = parallel([&](size_t i, std::string&) {
             fill_instance(i);
             return (int)CSP_OK;
         })))
        return rc;

    if ((rc = resolve_tuning())) return rc;
    int block[kBatchGroups];
    for (int g = 0; g < kBatchGroups; ++g) block[g] = used[g].block;
    std::vector<InstanceDesc> desc[kBatchGroups];
    std::vector<uint64_t> tb[kBatchGroups];
    fill_descs(block, nullptr, desc, tb);
    write_descs(desc, tb, h_stage);
    builds.clear();  // everything the device needs is in the staging image now
    builds.shrink_to_fit();
    uint64_t tiles[kBatchGroups];
    for (int g = 0; g < kBatchGroups; ++g) tiles[g] = tb[g][n_group[g]];

    // graph signature: everything the captured launches depend on besides the staged contents
    std::vector<uint64_t> sig = {(uint64_t)(uintptr_t)d_comp, (uint64_t)(uintptr_t)S.d_up, (uint64_t)(uintptr_t)S.h_stage,
                                 (uint64_t)(uintptr_t)S.h_result, up_bytes, zero_bytes, res_bytes, n, nx, ny,
                                 desc_off[0], zero_off, res_off};
    for (int g = 0; g < kBatchGroups; ++g) {
        sig.push_back(tiles[g]);
        sig.push_back((uint64_t)n_group[g]);
        sig.push_back((uint64_t)used[g].block);
        sig.push_back((uint64_t)used[g].ctas_per_sm);
        sig.push_back((uint64_t)used[g].chunk);
    }
    if (!S.graph || sig != S.graph_sig) {
        if (S.graph) cudaGraphExecDestroy(S.graph);
        S.graph = nullptr;
        cudaGraph_t g = nullptr;
        if ((rc = cuda_status(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "begin capture")))
            return rc;
        int crc = enqueue_zero(stream);
        if (!crc) crc = cuda_status(cudaEventRecordWithFlags(S.ev0, stream, cudaEventRecordExternal), "event");
        if (!crc) crc = enqueue_scene_setup(stream);
        for (int gi = 0; gi < kBatchGroups && !crc; ++gi)
            if (n_group[gi] > 0)
                crc = cuda_status(launch_trace_batch(launch_of(gi, tiles[gi], used[gi].chunk), gi, used[gi], stream),
                                  "batch_kernel");
        if (!crc) crc = cuda_status(cudaEventRecordWithFlags(S.ev1, stream, cudaEventRecordExternal), "event");
        if (!crc)
            crc = cuda_status(
                cudaMemcpyAsync(S.h_result, dev(res_off), res_bytes, cudaMemcpyDeviceToHost, stream), "download");
        const int erc = cuda_status(cudaStreamEndCapture(stream, &g), "end capture");
        if (crc || erc) {
            if (g) cudaGraphDestroy(g);
            return crc ? crc : erc;
        }
        rc = cuda_status(cudaGraphInstantiate(&S.graph, g, 0), "cudaGraphInstantiate");
        cudaGraphDestroy(g);
        if (rc) return rc;
        S.graph_sig = sig;
    }
    // what the results of this run need, whatever the instance list holds by then
    S.place = place;
    S.rays.resize(n);
    S.receiver.resize(n);
    for (size_t i = 0; i < n; ++i) {
        S.rays[i] = inst[i].rays;
        S.receiver[i] = elements_of(i)[count_of(i) - 1];
    }
    S.res_off = res_off;
    S.nx = nx;
    S.ny = ny;
    S.time_setup = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    S.up_bytes = up_bytes;
    S.res_bytes = res_bytes;
    // the upload on the copy stream (behind nothing but the uploads before it), the graph behind it
    // and behind the run before on the compute stream
    if ((rc = enqueue_upload(copy_stream))) return rc;
    if ((rc = cuda_status(cudaEventRecord(S.up_done, copy_stream), "cudaEventRecord"))) return rc;
    if ((rc = cuda_status(cudaStreamWaitEvent(stream, S.up_done, 0), "cudaStreamWaitEvent"))) return rc;
    if ((rc = cuda_status(cudaGraphLaunch(S.graph, stream), "cudaGraphLaunch"))) return rc;
    if ((rc = cuda_status(cudaEventRecord(S.done, stream), "cudaEventRecord"))) return rc;
    flight.push_back(si);
    return CSP_OK;
}

int Batch::wait() {
    NvtxRange nvtx("csp batch wait");
    if (flight.empty()) return set_error(CSP_ERR_STATE, "no batch run in flight");
    const int si = flight.front();
    flight.pop_front();
    RunSlot& S = slot[si];
    int rc = cuda_status(cudaEventSynchronize(S.done), "batch run");
    if (rc) return rc;
    float ms = 0.f;
    if ((rc = cuda_status(cudaEventElapsedTime(&ms, S.ev0, S.ev1), "batch timing"))) return rc;
    time_trace = ms * 1e-3;
    time_setup = S.time_setup;
    last_up = S.up_bytes;
    last_res = S.res_bytes;
    cur = si;
    return CSP_OK;
}

int Batch::run() {
    while (!flight.empty()) {
        const int rc = wait();
        if (rc) return rc;
    }
    const int rc = run_async();
    return rc ? rc : wait();
}

int Batch::result(uint32_t index, const uint32_t** counts, const unsigned long long** stats, const SunFrame** sun) const {
    if (cur < 0) return set_error(CSP_ERR_STATE, "no results: run the batch first");
    const RunSlot& S = slot[cur];
    if (index >= S.place.size()) return set_error(CSP_ERR_INVALID_ARGUMENT, "no such instance");
    const Place& p = S.place[index];
    if (counts) *counts = reinterpret_cast<const uint32_t*>(S.h_result + (p.counts - S.res_off));
    if (stats) *stats = reinterpret_cast<const unsigned long long*>(S.h_result + (p.stats - S.res_off));
    if (sun) *sun = reinterpret_cast<const SunFrame*>(S.h_result + (p.sun - S.res_off));
    return CSP_OK;
}

}  // namespace csp

using csp::Batch;

#define CSP_BGUARD(b)                                                                      \
    do {                                                                                   \
        if (!(b)) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "null batch handle");     \
    } while (0)

extern "C" {

int csp_set_tune_cache(const char* path) {
    std::lock_guard<std::mutex> lk(csp::g_tune_mu);
    csp::g_tune_path_set = true;
    csp::g_tune_path = path ? path : "";
    if (!csp::g_tune_path.empty()) csp::tune_load_locked(csp::g_tune_path);
    return CSP_OK;
}

int csp_tune_cache_entries(uint32_t* entries) {
    if (!entries) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "null output");
    std::lock_guard<std::mutex> lk(csp::g_tune_mu);
    csp::tune_init_locked();
    *entries = (uint32_t)csp::g_tune_cache.size();
    return CSP_OK;
}

int csp_batch_create(csp_batch* out, int device) {
    if (!out) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "null output handle");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) return csp::cuda_status(e, "cudaGetDeviceCount");
    if (device < 0 || device >= count) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "no such CUDA device");
    Batch* b = new (std::nothrow) Batch();
    if (!b) return csp::set_error(CSP_ERR_OUT_OF_MEMORY, "host allocation failed");
    b->device = device;
    *out = reinterpret_cast<csp_batch>(b);
    return CSP_OK;
}

int csp_batch_destroy(csp_batch b) {
    CSP_BGUARD(b);
    delete reinterpret_cast<Batch*>(b);
    return CSP_OK;
}

int csp_batch_set_flux_grid(csp_batch bh, uint32_t nx, uint32_t ny) {
    CSP_BGUARD(bh);
    if (nx == 0 || ny == 0 || (uint64_t)nx * ny > (1u << 24)) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "bad flux grid");
    Batch* b = reinterpret_cast<Batch*>(bh);
    b->nx = nx;
    b->ny = ny;
    return CSP_OK;
}

int csp_batch_set_output(csp_batch bh, int flags) {
    CSP_BGUARD(bh);
    if (flags & ~CSP_OUT_STAGED) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "unknown output flags");
    reinterpret_cast<Batch*>(bh)->out_flags = flags;
    return CSP_OK;
}

int csp_batch_add_scene(csp_batch bh, const csp_element* el, uint32_t n, uint32_t* id) {
    CSP_BGUARD(bh);
    if (!el || n == 0) return csp::set_error(CSP_ERR_BAD_SCENE, "scene has no elements");
    return reinterpret_cast<Batch*>(bh)->add_scene(el, n, id);
}

int csp_batch_add_instance(csp_batch bh, uint32_t scene, const csp_element* poses, const double* sun, int shape,
                           double param, uint64_t rays, uint64_t seed, uint32_t instance, uint32_t* index) {
    CSP_BGUARD(bh);
    if (!sun) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "null sun vector");
    Batch* b = reinterpret_cast<Batch*>(bh);
    csp::BInst bi;
    bi.scene = scene;
    if (poses && scene < b->scenes.size()) bi.poses.assign(poses, poses + b->scenes[scene].elements.size());
    bi.sun[0] = sun[0];
    bi.sun[1] = sun[1];
    bi.sun[2] = sun[2];
    bi.shape = shape;
    bi.param = param;
    bi.rays = rays;
    bi.seed = seed;
    bi.instance = instance;
    return b->add_instance(bi, index);
}

int csp_batch_clear_instances(csp_batch bh) {
    CSP_BGUARD(bh);
    Batch* b = reinterpret_cast<Batch*>(bh);
    b->inst.clear();
    return CSP_OK;
}

int csp_batch_num_instances(csp_batch bh, uint32_t* count) {
    CSP_BGUARD(bh);
    if (!count) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "null output");
    *count = (uint32_t)reinterpret_cast<Batch*>(bh)->inst.size();
    return CSP_OK;
}

int csp_batch_set_tuning(csp_batch bh, int block, int ctas_per_sm, int chunk) {
    CSP_BGUARD(bh);
    if (block != 0 && block != 128 && block != 256)
        return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "block must be 0 (autotune), 128 or 256");
    if (block != 0 && (ctas_per_sm < 0 || chunk <= 0))
        return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "bad tuning parameters");
    reinterpret_cast<Batch*>(bh)->user = csp::BatchTuning{block, ctas_per_sm, block ? chunk : 0};
    return CSP_OK;
}

int csp_batch_get_tuning(csp_batch bh, int group, int* block, int* ctas_per_sm, int* chunk) {
    CSP_BGUARD(bh);
    if (group < 0 || group >= csp::kBatchGroups) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "no such group");
    const csp::BatchTuning& t = reinterpret_cast<Batch*>(bh)->used[group];
    if (block) *block = t.block;
    if (ctas_per_sm) *ctas_per_sm = t.ctas_per_sm;
    if (chunk) *chunk = t.chunk;
    return CSP_OK;
}

int csp_batch_run(csp_batch bh) {
    CSP_BGUARD(bh);
    return reinterpret_cast<Batch*>(bh)->run();
}

int csp_batch_run_async(csp_batch bh) {
    CSP_BGUARD(bh);
    return reinterpret_cast<Batch*>(bh)->run_async();
}

int csp_batch_wait(csp_batch bh) {
    CSP_BGUARD(bh);
    return reinterpret_cast<Batch*>(bh)->wait();
}

int csp_batch_get_flux(csp_batch bh, uint32_t index, uint32_t* counts, double dni, double* flux) {
    CSP_BGUARD(bh);
    const Batch* b = reinterpret_cast<Batch*>(bh);
    const uint32_t* c = nullptr;
    const csp::SunFrame* f = nullptr;
    int rc = b->result(index, &c, nullptr, &f);
    if (rc) return rc;
    const csp::RunSlot& S = b->slot[b->cur];
    const size_t nb = (size_t)S.nx * S.ny;
    if (counts) std::memcpy(counts, c, nb * sizeof(uint32_t));
    if (flux)
        csp::counts_to_flux(c, nb, dni, csp::sun_plane_area(*f), S.rays[index],
                            csp::flux_bin_area(S.receiver[index], S.nx, S.ny), flux);
    return CSP_OK;
}

int csp_batch_get_stats(csp_batch bh, uint32_t index, uint64_t* stats) {
    CSP_BGUARD(bh);
    if (!stats) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "null output");
    const Batch* b = reinterpret_cast<Batch*>(bh);
    const unsigned long long* s = nullptr;
    int rc = b->result(index, nullptr, &s, nullptr);
    if (rc) return rc;
    stats[0] = b->slot[b->cur].rays[index];
    for (int k = 1; k < 4; ++k) stats[k] = s[k];
    return CSP_OK;
}

int csp_batch_get_sun_plane(csp_batch bh, uint32_t index, float* out) {
    CSP_BGUARD(bh);
    if (!out) return csp::set_error(CSP_ERR_INVALID_ARGUMENT, "null output");
    const Batch* b = reinterpret_cast<Batch*>(bh);
    const csp::SunFrame* f = nullptr;
    int rc = b->result(index, nullptr, nullptr, &f);
    if (rc) return rc;
    const float v[16] = {f->s_d.x, f->s_d.y, f->s_d.z, f->v0.x, f->v0.y, f->v0.z, f->v1.x, f->v1.y,
                         f->v1.z,  f->v2.x,  f->v2.y,  f->v2.z, f->v3.x, f->v3.y, f->v3.z, f->s_d.w};
    std::memcpy(out, v, sizeof(v));
    return CSP_OK;
}

int csp_batch_get_timing(csp_batch bh, double* setup_s, double* trace_s) {
    CSP_BGUARD(bh);
    const Batch* b = reinterpret_cast<Batch*>(bh);
    if (setup_s) *setup_s = b->time_setup;
    if (trace_s) *trace_s = b->time_trace;
    return CSP_OK;
}

int csp_batch_get_transfer(csp_batch bh, uint64_t* h2d_bytes, uint64_t* d2h_bytes) {
    CSP_BGUARD(bh);
    const Batch* b = reinterpret_cast<Batch*>(bh);
    if (h2d_bytes) *h2d_bytes = b->last_up;
    if (d2h_bytes) *d2h_bytes = b->last_res;
    return CSP_OK;
}

}  // extern "C"
