// csp_batch.h -- state behind one csp_batch handle (batched multi-instance tracing).
#pragma once

#include <cstdint>
#include <deque>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "csp_c_api.h"
#include "csp_kernels.cuh"
#include "csp_scene.h"

namespace csp {

struct BScene {
    std::vector<csp_element> elements;
    HostScene base;         // element records + BVH topology of the scene's own poses
    Node* d_topo = nullptr; // topology on the device (links; boxes of the scene's own poses)
    bool flat = false;      // <= kFlatListMax elements: shared-memory element list kernel
    HostGrid grid;          // field grid of the scene's own poses (valid for field-like scenes)
    uint32_t* d_cells = nullptr;
    Aabb* d_items = nullptr;
    Aabb* d_global = nullptr;
};

// Host build of one instance with its own poses: element records and the grid of those poses.
struct InstBuild {
    HostScene hs;
    HostGrid grid;
};

struct BInst {
    uint32_t scene = 0;
    std::vector<csp_element> poses;  // empty: the scene's own elements
    double sun[3] = {0, 0, 1};
    int shape = CSP_SUN_PILLBOX;
    double param = 0.0;
    uint64_t rays = 0, seed = 0;
    uint32_t instance = 0;
};

// Byte offsets of one instance's arrays in the device arena (and the staging image).
struct Place {
    size_t prims = 0, optics = 0, aabbs = 0, prune = 0, nodes = 0, sun = 0, counts = 0, stats = 0;
    size_t cells = 0, items = 0, global = 0;  // own grid arrays (instances with poses in the grid group)
    size_t sgrid = 0;  // sun-ray candidate grid (BVH and grid groups), built on the device
    int sg_slot = -1;  // index of its build job
    int group = 0;  // kAccelFlat, kAccelBvh or kAccelGrid: the kernel that traces the instance
    int slot = 0;   // index within the group
};

// One run of the pipeline: its pinned buffers and graph, and what its results need (the layout and
// inputs of its instances), so the instance list can change while the run is in flight.  The host
// builds run k + 1 into one slot while run k executes from the other.
struct RunSlot {
    unsigned char* h_stage = nullptr;  // pinned image of the upload region
    size_t stage_cap = 0;
    unsigned char* d_up = nullptr;  // the slot's upload region on the device (see Batch::dev)
    size_t up_cap = 0;
    cudaEvent_t up_done = nullptr;  // the upload of the slot's run, on the copy stream
    unsigned char* h_result = nullptr;  // pinned copy of the download region
    size_t result_cap = 0;
    cudaGraphExec_t graph = nullptr;
    std::vector<uint64_t> graph_sig;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, done = nullptr;
    std::vector<Place> place;
    std::vector<uint64_t> rays;
    std::vector<csp_element> receiver;
    size_t res_off = 0;
    uint32_t nx = 0, ny = 0;
    double time_setup = 0.0;
    size_t up_bytes = 0, res_bytes = 0;  // host-to-device and device-to-host bytes of the run
};

struct Batch {
    int device = -1;
    std::string device_model;  // "name ccM.m smN": the autotuner cache key's device part
    cudaStream_t stream = nullptr;
    // uploads of pipelined runs: run k + 1's upload overlaps run k's kernels on `stream`
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;  // autotuner timing
    const float* h3t12 = nullptr;  // Halton table of the device
    uint32_t nx = 100, ny = 100;
    int out_flags = 0;  // CSP_OUT_* of the instances' flux maps
    std::vector<BScene> scenes;
    std::vector<BInst> inst;
    BatchTuning user{0, 0, 0};  // block 0: autotune
    BatchTuning used[kBatchGroups] = {{128, 0, 4}, {128, 0, 4}, {128, 0, 4}};

    // device memory: the upload region [0, up_bytes) of the layout lives in the run slot's d_up (two
    // runs in flight upload into different memory), the rest, which the device writes, in d_comp
    // (shared: the kernels of runs are ordered on `stream`)
    unsigned char* d_comp = nullptr;
    size_t comp_cap = 0;
    unsigned char* d_up = nullptr;  // upload region of the run being built (its slot's)
    RunSlot slot[2];
    std::deque<int> flight;            // slots of the runs in flight, oldest first
    int cur = -1;                      // slot of the last completed run (its results), -1: none
    unsigned char* h_stage = nullptr;  // staging image of the run being built

    std::vector<Place> place;
    size_t up_bytes = 0, zero_off = 0, zero_bytes = 0, res_off = 0, res_bytes = 0;
    size_t desc_off[kBatchGroups] = {}, tb_off[kBatchGroups] = {}, refit_off = 0, sunjob_off = 0, counter_off = 0;
    size_t sgjob_off = 0;
    int n_group[kBatchGroups] = {};
    int n_sg = 0, max_sg_n = 0;  // sun grid build jobs and their largest element count
    std::vector<InstBuild> builds;  // per instance, during a run (instances with poses)
    int max_nodes = 0;

    double time_setup = 0.0, time_trace = 0.0;  // of the last completed run
    size_t last_up = 0, last_res = 0;            // its transfer sizes

    ~Batch();
    void release();
    int ensure_stream();
    int add_scene(const csp_element* el, uint32_t n, uint32_t* id);
    int add_instance(const BInst& bi, uint32_t* index);
    const csp_element* elements_of(size_t i) const;
    uint32_t count_of(size_t i) const;
    int layout(int s);
    int build_instance(size_t i, std::string& err);
    const HostScene& scene_of(size_t i) const;
    const HostGrid& grid_of(size_t i) const;
    void fill_instance(size_t i);
    void fill_descs(const int* block, const std::vector<bool>* sample, std::vector<InstanceDesc>* desc,
                    std::vector<uint64_t>* tb);
    void write_descs(const std::vector<InstanceDesc>* desc, const std::vector<uint64_t>* tb, unsigned char* img);
    BatchLaunch launch_of(int g, uint64_t total_tiles, int chunk) const;
    // device address of layout offset `off`
    unsigned char* dev(size_t off) const { return off < up_bytes ? d_up + off : d_comp + (off - up_bytes); }
    int enqueue_upload(cudaStream_t st);
    int enqueue_zero(cudaStream_t st);
    int enqueue_scene_setup(cudaStream_t st);
    int autotune(int g, BatchTuning& best);
    int resolve_tuning();
    int run_async();
    int wait();
    int run();
    int result(uint32_t index, const uint32_t** counts, const unsigned long long** stats, const SunFrame** sun) const;
};

}  // namespace csp
