// snk_host.h -- host-side helpers shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <utility>

#include "snk_device.cuh"
#include "snk_pt.h"

namespace snk {

// Owning device allocation (cudaMalloc/cudaFree); grows, never shrinks.
template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DBuf& operator=(DBuf&& o) noexcept { std::swap(p, o.p); std::swap(n, o.n); return *this; }
    ~DBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    cudaError_t reserve(size_t count) {
        if (count <= n && p) return cudaSuccess;
        release();
        if (count == 0) count = 1;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) { p = nullptr; return e; }
        n = count;
        return cudaSuccess;
    }
    T* get() const { return p; }
};

// Error carrying a status code of snk_pt.h and a message.
struct Status {
    int code = 0;
    std::string msg;
    bool ok() const { return code == 0; }
    static Status Ok() { return Status(); }
    static Status Err(int c, std::string m) { Status s; s.code = c; s.msg = std::move(m); return s; }
};

#define SNK_TRY_CUDA(call)                                                                            \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess)                                                                        \
            return ::snk::Status::Err(e_ == cudaErrorMemoryAllocation ? 3 : 2,                        \
                                      std::string(#call) + ": " + cudaGetErrorString(e_));           \
    } while (0)

#define SNK_TRY(expr)              \
    do {                           \
        ::snk::Status s_ = (expr); \
        if (!s_.ok()) return s_;   \
    } while (0)

// ---- BVH builder ---------------------------------------------------------------
struct BuildScratch {
    DBuf<unsigned long long> keys, keys_alt;
    DBuf<uint32_t> vals, vals_alt;
    DBuf<int2> children;
    DBuf<int> parent, flags;
    DBuf<float4> node_lo, node_hi;
    DBuf<uint32_t> leaf_count;
    DBuf<float> cost;             // binary-tree SAH cost per node (treelet restructuring)
    DBuf<uint2> tasks_a, tasks_b;
    DBuf<uint32_t> counters;      // [0] tasks in, [1] tasks out, [2] wide nodes, [3] prims
    DBuf<unsigned> cbounds;       // centroid bounds, order-preserving encoded
    DBuf<uint32_t> sort_hist;     // per-tile digit counts of the multi-CTA radix sort
    DBuf<double> sah;             // SAH accumulator
    DBuf<uint32_t> level_tasks;   // task count per wide level (device-driven collapse)
    DBuf<float> wide_cost;        // 8 per binary internal node: SAH cost of its subtree in 1..8 wide children
    DBuf<uint32_t> wide_split;    // per binary internal node: the split of those children (4-bit fields)
    size_t cap = 0;
};

struct BuildResult {
    uint32_t num_nodes = 0;
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    double sah = 0.0;   // SAH cost of the wide BVH (internal 1, primitive 1, area relative to the root)
};

// Builds an 8-wide compressed BVH over n primitive boxes (prim_lo/prim_hi, xyz used).
// Nodes are written at nodes[node_base + k] (root at node_base) with absolute child
// indices; primitive slots are [prim_base, prim_base + n) and prim_order[k] receives
// the primitive id stored in slot prim_base + k.
Status build_wide_bvh(BuildScratch& sc, const float4* prim_lo, const float4* prim_hi, uint32_t n, WideNode* nodes,
                      uint32_t node_base, uint32_t prim_base, uint32_t* prim_order, cudaStream_t stream,
                      BuildResult* out, int treelet_passes, uint32_t leaf_max, uint32_t leaf_pack,
                      bool sah_collapse = true);

struct SmallBuildOut;
// The same tree without host round trips (for per-frame rebuilds): the collapse
// runs level by level on the device, nothing is read back, and a build error
// (never seen for a correct tree) sets bit 8 of *err_word.  At most n + 1 nodes
// are written.  With out and wide_depth (n + 1 entries) given, the device keeps
// the node count, the deepest level and every node's depth for a later refit.
Status build_wide_bvh_device(BuildScratch& sc, const float4* prim_lo, const float4* prim_hi, uint32_t n,
                             WideNode* nodes, uint32_t node_base, uint32_t prim_base, uint32_t* prim_order,
                             unsigned* err_word, cudaStream_t stream, int treelet_passes, uint32_t leaf_max,
                             uint32_t leaf_pack, SmallBuildOut* out = nullptr, uint32_t* wide_depth = nullptr,
                             bool sah_collapse = true);

// Single-launch build for n <= SMALL_BUILD_MAX primitives (one CTA, shared
// memory, no host synchronisation); same algorithm and output layout as
// build_wide_bvh.  The result record stays on the device.  A build error (never
// seen for a correct tree) sets out->error and bit 8 of *err_word.
constexpr int SMALL_BUILD_MAX = 1024;
struct SmallBuildOut {
    uint32_t num_nodes, prims, error, max_depth;
    double sah;   // not computed by the single-launch build (0)
    float lo[4], hi[4];
};
// wide_box (2 x (n + 1) float4: exact lo, hi per wide node) and wide_depth
// (n + 1) receive what a later refit needs.
Status build_wide_bvh_small(const float4* prim_lo, const float4* prim_hi, uint32_t n, WideNode* nodes,
                            uint32_t node_base, uint32_t prim_base, uint32_t* prim_order, int treelet_passes,
                            SmallBuildOut* out, unsigned* err_word, float4* wide_box, uint32_t* wide_depth,
                            cudaStream_t stream, uint32_t leaf_max, bool sah_collapse = true);
// Refit of a tree made by build_wide_bvh_small or build_wide_bvh_device (with its
// record and depths) for the same n primitives in new boxes (prim_order as that
// build wrote it; wide_box: 2 x (n + 1) float4 of scratch that receives every
// node's exact box; everything stays on the device).
Status refit_wide_bvh(const float4* prim_lo, const float4* prim_hi, uint32_t n, WideNode* nodes, uint32_t node_base,
                      uint32_t prim_base, const uint32_t* prim_order, const SmallBuildOut* info, float4* wide_box,
                      const uint32_t* wide_depth, unsigned* err_word, cudaStream_t stream);

// Per-triangle padded boxes of one mesh (object space).
Status launch_triangle_boxes(const float* positions, const uint32_t* indices, uint32_t vertex_offset,
                             uint32_t index_offset, uint32_t num_tris, float4* lo, float4* hi, cudaStream_t s);
// Triangle records of one mesh from the build's primitive order.
Status launch_fill_triangles(const uint32_t* prim_order, uint32_t n, const float* positions, const uint32_t* indices,
                             uint32_t vertex_offset, uint32_t index_offset, TriRecord* out, cudaStream_t s);
// World boxes of the listed instances (transform of the mesh bounds) for the instance BVH.
Status launch_instance_boxes(const uint32_t* inst_list, uint32_t n, const InstShade* inst, const MeshInfo* meshes,
                             float4* lo, float4* hi, cudaStream_t s);
// ---- per-frame scene tables (scene_tables.cu) ---------------------------------
struct LightCdfScratch {
    DBuf<unsigned long long> acc, wmax, tile_sums, q;   // prefix sums, max weight, tile sums, quantised weights
};
// traversal and shading records of n instances from their raw records
Status launch_instance_records(const snk_instance* raw, uint32_t n, const MeshInfo* meshes, InstTrace* it,
                               InstShade* is, cudaStream_t st);
// ReSTIR candidate records of the emissive instances em_list[0..n_em) (after their instance records)
Status launch_emissive_records(const uint32_t* em_list, uint32_t n_em, const InstShade* is, const MeshInfo* meshes,
                               const MaterialDev* mats, EmissiveRec* recs, cudaStream_t st);
// NEE records and weights of the n_tri triangles of the emissive instances em_list[0..n_em)
// (em_first: prefix sums of their triangle counts)
Status launch_emissive_lights(const snk_instance* raw, const uint32_t* em_list, const uint32_t* em_first, uint32_t n_em,
                              uint32_t n_tri, const MeshInfo* meshes, const float* pos, const uint32_t* idx,
                              const MaterialDev* mats, LocalLight* lights, double* w, cudaStream_t st);
// light-selection CDF and PMF of n weights (quantised to integers, exact prefix sums)
Status launch_light_cdf(const double* w, uint32_t n, LightCdfScratch& sc, float* cdf, float* pmf, cudaStream_t st);
// the same table computed on the host (for tables whose weights are all known there)
void light_cdf_host(const double* w, uint32_t n, float* cdf, float* pmf);

// tlas_prims[k] = inst_list[prim_order[k]]
Status launch_map_prims(const uint32_t* prim_order, const uint32_t* inst_list, uint32_t n, uint32_t* out,
                        cudaStream_t s);

}  // namespace snk
