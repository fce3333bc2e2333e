// csp_scene.h -- host scene model: elements -> device records, acceleration structure, refit.
#pragma once

#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "csp_c_api.h"
#include "csp_types.cuh"

namespace csp {

struct HostScene {
    std::vector<Prim> prims;      // per element, element order
    std::vector<Optics> optics;   // per element
    std::vector<Aabb> aabbs;      // exact element AABBs (float), element order; lo.w = element | type << 28 (bits)
    std::vector<Aabb> prune;      // boxes bounding each element's surface (sag, rounding margin)
    std::vector<uint32_t> types;  // EntityType per element
    std::vector<Node> nodes;      // traversal order
    std::vector<int32_t> parent;  // parent node of each node (-1 for the root), for refits
    std::vector<int32_t> leaf_of; // node index of each element's leaf
    float sun[3] = {0, 0, 1};     // normalized sun vector, float
};

// Build prims, optics, AABBs, pruning boxes and entity types.  Returns CSP_OK or an error status
// with `err` filled.  The geometry arithmetic is the reference's (lib/element.cpp, lib/math_util.h,
// cuda/GeometryDataST.h constructors), in the same double/float operation order.
int build_elements(const csp_element* el, uint32_t n, HostScene& s, std::string& err);

// Runs body(k) for every k in [0, tasks), possibly on several threads, and returns when all are
// done.
using ParallelFor = std::function<void(size_t tasks, const std::function<void(size_t)>& body)>;

// build_elements with the elements packed in ranges of kBuildChunk through `pf`: the same records
// (each element's packing reads only that element), and the same error (the lowest failing element).
constexpr uint32_t kBuildChunk = 1024;
int build_elements(const csp_element* el, uint32_t n, HostScene& s, std::string& err, const ParallelFor& pf);

// The records of one element, as build_elements makes them: entity type, exact AABB, Prim, Optics
// and (when `prune` is not null) the pruning box.  Allocates nothing.  Returns CSP_OK, or
// CSP_ERR_BAD_SCENE with `why` pointing to a static message.
int pack_element(const csp_element& e, bool last, uint32_t& type, Aabb& box, Prim& p, Optics& o, Aabb* prune,
                 const char*& why);

// Build the stackless BVH over the pruning boxes (binned SAH, one element per leaf; scenes of up
// to kFlatListMax elements get a plain list of leaves instead).
constexpr uint32_t kFlatListMax = 8;  // = kFlatMax of the trace kernel
void build_bvh(HostScene& s);

// Recompute every node box of an existing topology from the current aabbs/prune boxes (children
// are stored after their parents, so one reverse sweep is a bottom-up refit).
void refit_bvh(HostScene& s);

// Euler angles (yaw, pitch, roll in radians), global-to-local matrix (row-major; rows = local x,
// y, z axes in world space) and exact double AABB of one element.
void element_frame(const csp_element& e, double euler[3], double G[9], double lo[3], double hi[3]);

// Uniform 2D grid of a field-like scene for one set of poses (see GridDesc): every mirror is
// registered in each cell that its pruning box, widened by 2e-5 |coordinate| + 5 cm, overlaps in
// xy; the last element (receiver) and oversized elements form the global list.  Items carry the
// exact AABB (lo.w = element | type << kTypeShift).
struct HostGrid {
    bool valid = false;
    float x0 = 0, y0 = 0, x1 = 0, y1 = 0, cell = 1, inv_cell = 1, zlo = 0, zhi = 0;
    int nx = 0, ny = 0;
    std::vector<uint32_t> cell_start;  // [nx * ny + 1]
    std::vector<Aabb> items;
    std::vector<Aabb> global;
};


// Build the grid of a scene with more than kFlatListMax elements whose mirrors lie in a thin layer
// (at most a quarter of the field's horizontal extent); otherwise leave g.valid false (the BVH is
// used).  Reads s.prune (registration, layer), s.aabbs (items) and s.types.
void build_grid(const HostScene& s, HostGrid& g);

// Device descriptor of a grid whose arrays live at the given device addresses.
GridDesc grid_desc(const HostGrid& g, const uint32_t* cell_start, const Aabb* items, const Aabb* global);

// Flux map target of a receiver element for an nx x ny grid (counts and stats pointers left null),
// and the area of one bin in m^2 (flat: (w/nx)(h/ny); cylinder: (2 pi r/nx)(h/ny)).
void flux_target(const csp_element& rcv, uint32_t nx, uint32_t ny, FluxTarget& F);
double flux_bin_area(const csp_element& rcv, uint32_t nx, uint32_t ny);

// normalized sun vector in double, cast to float (SolTraceSystem::initialize,
// lib/soltrace_system.cpp:81-85)
void sun_vector_f(const double d[3], float out[3]);

}  // namespace csp
