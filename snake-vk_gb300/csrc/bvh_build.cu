// bvh_build.cu -- GPU construction of 8-wide compressed BVHs.
//
// Replaces the driver-built acceleration structures of the reference:
//   BLAS::GenerateFromMeshData   Core/src/resources/TLAS.cpp:109-186 (per submesh, at load)
//   TLAS::BuildFromInstances     Core/src/resources/TLAS.cpp:10-87   (full rebuild every frame,
//                                Core/src/scene/TlasSystem.cpp:16-20,27-49)
//
// Pipeline (all on the device, one stream):
//   1. centroid bounds (block reduction + order-preserving atomics)
//   2. 63-bit Morton codes of the centroids (21 bits per axis)
//   3. radix sort of (code, primitive) pairs (CUB DeviceRadixSort)
//   4. binary radix tree (Karras, HPG 2012): one thread per internal node
//   5. bottom-up boxes and leaf counts (atomic arrival flags)
//   6. top-down collapse to 8-wide nodes, one thread per output node, level by
//      level: a node's children start as its binary children; the internal child
//      with the largest surface area and more than 3 leaves is replaced by its two
//      children until 8 children exist or none can be opened.  Children with <= 3
//      leaves become leaves.  Children are assigned to the 8 slots greedily by how
//      well their centroid offset matches each octant corner, so that visiting
//      slot ^ ray_octant in increasing order is roughly front to back.  Child boxes
//      are quantised outwards to 8 bits per plane.
//   7. SAH cost of the result (for quality reporting).
#include <cub/device/device_radix_sort.cuh>

#include "snk_host.h"

namespace snk {
namespace {

constexpr int BLK = 256;

__device__ __forceinline__ unsigned enc_f(float f) {
    unsigned b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float dec_f(unsigned u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

__global__ void k_init_bounds(unsigned* cb) {
    if (threadIdx.x < 3) { cb[threadIdx.x] = 0xFFFFFFFFu; cb[3 + threadIdx.x] = 0u; }
}

__global__ void k_centroid_bounds(const float4* __restrict__ lo, const float4* __restrict__ hi, uint32_t n,
                                  unsigned* cb) {
    __shared__ unsigned smin[3][BLK], smax[3][BLK];
    unsigned mn[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu}, mx[3] = {0u, 0u, 0u};
    for (uint32_t i = blockIdx.x * BLK + threadIdx.x; i < n; i += gridDim.x * BLK) {
        float4 a = lo[i], b = hi[i];
        float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
        for (int k = 0; k < 3; k++) { unsigned e = enc_f(c[k]); mn[k] = min(mn[k], e); mx[k] = max(mx[k], e); }
    }
    for (int k = 0; k < 3; k++) { smin[k][threadIdx.x] = mn[k]; smax[k][threadIdx.x] = mx[k]; }
    __syncthreads();
    for (int s = BLK / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s)
            for (int k = 0; k < 3; k++) {
                smin[k][threadIdx.x] = min(smin[k][threadIdx.x], smin[k][threadIdx.x + s]);
                smax[k][threadIdx.x] = max(smax[k][threadIdx.x], smax[k][threadIdx.x + s]);
            }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 3; k++) { atomicMin(&cb[k], smin[k][0]); atomicMax(&cb[3 + k], smax[k][0]); }
}

__device__ __forceinline__ unsigned long long spread21(unsigned long long x) {
    x &= 0x1FFFFFull;
    x = (x | (x << 32)) & 0x1F00000000FFFFull;
    x = (x | (x << 16)) & 0x1F0000FF0000FFull;
    x = (x | (x << 8)) & 0x100F00F00F00F00Full;
    x = (x | (x << 4)) & 0x10C30C30C30C30C3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

__global__ void k_morton(const float4* __restrict__ lo, const float4* __restrict__ hi, uint32_t n,
                         const unsigned* cb, unsigned long long* keys, uint32_t* vals) {
    uint32_t i = blockIdx.x * BLK + threadIdx.x;
    if (i >= n) return;
    float4 a = lo[i], b = hi[i];
    float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
    unsigned long long q[3];
    for (int k = 0; k < 3; k++) {
        float mn = dec_f(cb[k]), mx = dec_f(cb[3 + k]);
        float ext = mx - mn;
        float f = ext > 0.0f ? (c[k] - mn) / ext : 0.5f;
        f = fminf(fmaxf(f, 0.0f), 1.0f);
        q[k] = (unsigned long long)fminf(f * 2097152.0f, 2097151.0f);
    }
    keys[i] = (spread21(q[0]) << 2) | (spread21(q[1]) << 1) | spread21(q[2]);
    vals[i] = i;
}

__device__ __forceinline__ int delta(const unsigned long long* __restrict__ k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    unsigned long long a = k[i], b = k[j];
    if (a == b) return 64 + __clz((unsigned)(i ^ j));
    return __clzll(a ^ b);
}

__global__ void k_karras(const unsigned long long* __restrict__ keys, int n, int2* children, int* parent) {
    int i = blockIdx.x * BLK + threadIdx.x;
    if (i >= n - 1) return;
    int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = delta(keys, n, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int gamma = i + s * d + min(d, 0);
    int left = (min(i, j) == gamma) ? (n - 1 + gamma) : gamma;
    int right = (max(i, j) == gamma + 1) ? (n - 1 + gamma + 1) : gamma + 1;
    children[i] = make_int2(left, right);
    parent[left] = i;
    parent[right] = i;
}

__global__ void k_bottom_up(const uint32_t* __restrict__ sorted, const float4* __restrict__ plo,
                            const float4* __restrict__ phi, int n, const int2* __restrict__ children,
                            const int* __restrict__ parent, int* flags, float4* node_lo, float4* node_hi,
                            uint32_t* leaf_count) {
    int j = blockIdx.x * BLK + threadIdx.x;
    if (j >= n) return;
    int node = n - 1 + j;
    uint32_t prim = sorted[j];
    float4 lo = plo[prim], hi = phi[prim];
    node_lo[node] = lo;
    node_hi[node] = hi;
    leaf_count[node] = 1;
    if (n == 1) return;
    int p = parent[node];
    while (p >= 0) {
        __threadfence();
        if (atomicAdd(&flags[p], 1) == 0) return;
        __threadfence();
        int2 ch = children[p];
        float4 al = __ldcg(&node_lo[ch.x]), ah = __ldcg(&node_hi[ch.x]);
        float4 bl = __ldcg(&node_lo[ch.y]), bh = __ldcg(&node_hi[ch.y]);
        uint32_t ca = __ldcg(&leaf_count[ch.x]), cb = __ldcg(&leaf_count[ch.y]);
        node_lo[p] = make_float4(fminf(al.x, bl.x), fminf(al.y, bl.y), fminf(al.z, bl.z), 0.0f);
        node_hi[p] = make_float4(fmaxf(ah.x, bh.x), fmaxf(ah.y, bh.y), fmaxf(ah.z, bh.z), 0.0f);
        leaf_count[p] = ca + cb;
        p = parent[p];
    }
}

__device__ __forceinline__ float half_area(float4 lo, float4 hi) {
    float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    return dx * dy + dy * dz + dz * dx;
}

// smallest power-of-two exponent (biased) with 2^(e-127) >= x; at least 1
__device__ __forceinline__ uint32_t ceil_exp_biased(float x) {
    uint32_t b = __float_as_uint(x);
    uint32_t e = (b >> 23) & 0xFFu;
    if (e == 0) return 1u;
    if (b & 0x7FFFFFu) e += 1;
    return e > 254u ? 254u : e;
}

__global__ void k_collapse(const uint2* __restrict__ tasks_in, uint32_t* counters, uint2* tasks_out, int n,
                           const int2* __restrict__ children, const float4* __restrict__ node_lo,
                           const float4* __restrict__ node_hi, const uint32_t* __restrict__ leaf_count,
                           const uint32_t* __restrict__ sorted, WideNode* nodes, uint32_t node_base,
                           uint32_t prim_base, uint32_t* prim_order, double* sah, float root_half_area) {
    uint32_t ti = blockIdx.x * BLK + threadIdx.x;
    if (ti >= counters[0]) return;
    uint2 task = tasks_in[ti];
    int b = (int)task.x;
    uint32_t w = task.y;
    const int nl = n - 1;  // first leaf id
    int C[8];
    int nc;
    if (b >= nl) { C[0] = b; nc = 1; }
    else { int2 ch = children[b]; C[0] = ch.x; C[1] = ch.y; nc = 2; }
    while (nc < 8) {
        int best = -1;
        float best_a = -1.0f;
        for (int k = 0; k < nc; k++) {
            int c = C[k];
            if (c < nl && leaf_count[c] > 3u) {
                float a = half_area(node_lo[c], node_hi[c]);
                if (a > best_a) { best_a = a; best = k; }
            }
        }
        if (best < 0) break;
        int2 ch = children[C[best]];
        C[best] = ch.x;
        C[nc++] = ch.y;
    }
    // parent box and child centroids
    float4 plo = node_lo[C[0]], phi = node_hi[C[0]];
    for (int k = 1; k < nc; k++) {
        float4 a = node_lo[C[k]], z = node_hi[C[k]];
        plo.x = fminf(plo.x, a.x); plo.y = fminf(plo.y, a.y); plo.z = fminf(plo.z, a.z);
        phi.x = fmaxf(phi.x, z.x); phi.y = fmaxf(phi.y, z.y); phi.z = fmaxf(phi.z, z.z);
    }
    float pcx = 0.5f * (plo.x + phi.x), pcy = 0.5f * (plo.y + phi.y), pcz = 0.5f * (plo.z + phi.z);
    float ccx[8], ccy[8], ccz[8];
    for (int k = 0; k < nc; k++) {
        float4 a = node_lo[C[k]], z = node_hi[C[k]];
        ccx[k] = 0.5f * (a.x + z.x) - pcx; ccy[k] = 0.5f * (a.y + z.y) - pcy; ccz[k] = 0.5f * (a.z + z.z) - pcz;
    }
    // greedy slot assignment: slot bit i set <=> the child lies on the + side of axis i
    int slot_child[8];
    for (int s = 0; s < 8; s++) slot_child[s] = -1;
    uint32_t used_c = 0, used_s = 0;
    for (int it = 0; it < nc; it++) {
        float best = -3.4e38f;
        int bk = -1, bs = -1;
        for (int k = 0; k < nc; k++) {
            if (used_c & (1u << k)) continue;
            for (int s = 0; s < 8; s++) {
                if (used_s & (1u << s)) continue;
                float sc = ((s & 1) ? ccx[k] : -ccx[k]) + ((s & 2) ? ccy[k] : -ccy[k]) + ((s & 4) ? ccz[k] : -ccz[k]);
                if (sc > best) { best = sc; bk = k; bs = s; }
            }
        }
        used_c |= 1u << bk;
        used_s |= 1u << bs;
        slot_child[bs] = C[bk];
    }
    // classify and allocate
    uint32_t n_int = 0, n_prims = 0;
    for (int s = 0; s < 8; s++) {
        int c = slot_child[s];
        if (c < 0) continue;
        if (c < nl && leaf_count[c] > 3u) n_int++;
        else n_prims += leaf_count[c];
    }
    uint32_t child_local = n_int ? atomicAdd(&counters[2], n_int) : 0u;
    uint32_t prim_local = n_prims ? atomicAdd(&counters[3], n_prims) : 0u;
    // capacity checks: n wide nodes, n primitive slots, n tasks (never exceeded by a
    // correct tree; a violation is recorded and the node is not written)
    if (child_local + n_int > (uint32_t)n + 1u || prim_local + n_prims > (uint32_t)n || w - node_base > (uint32_t)n) {
        atomicOr(&counters[4], 1u);
        return;
    }
    // quantisation frame
    float ex_[3] = {__fsub_ru(phi.x, plo.x), __fsub_ru(phi.y, plo.y), __fsub_ru(phi.z, plo.z)};
    uint32_t eb[3];
    float inv_scale[3];
    for (int a = 0; a < 3; a++) {
        eb[a] = ceil_exp_biased(__fdiv_ru(ex_[a], 255.0f));
        inv_scale[a] = __uint_as_float((254u - eb[a]) << 23);   // 2^(127 - (eb - 127))
    }
    WideNode node;
    node.px = plo.x; node.py = plo.y; node.pz = plo.z;
    node.ex = (uint8_t)eb[0]; node.ey = (uint8_t)eb[1]; node.ez = (uint8_t)eb[2];
    node.imask = 0;
    node.child_base = node_base + child_local;
    node.prim_base = prim_base + prim_local;
    uint32_t rank = 0, off = 0;
    float p3[3] = {plo.x, plo.y, plo.z};
    double local_sah = 0.0;
    for (int s = 0; s < 8; s++) {
        int c = slot_child[s];
        if (c < 0) {
            node.meta[s] = 0;
            for (int a = 0; a < 3; a++) { node.qlo[a][s] = 0; node.qhi[a][s] = 0; }
            continue;
        }
        float4 a4 = node_lo[c], z4 = node_hi[c];
        float clo[3] = {a4.x, a4.y, a4.z}, chi[3] = {z4.x, z4.y, z4.z};
        for (int a = 0; a < 3; a++) {
            float ql = floorf(__fmul_rd(__fsub_rd(clo[a], p3[a]), inv_scale[a]));
            float qh = ceilf(__fmul_ru(__fsub_ru(chi[a], p3[a]), inv_scale[a]));
            node.qlo[a][s] = (uint8_t)fminf(fmaxf(ql, 0.0f), 255.0f);
            node.qhi[a][s] = (uint8_t)fminf(fmaxf(qh, 0.0f), 255.0f);
        }
        float ha = half_area(a4, z4) / root_half_area;
        if (c < nl && leaf_count[c] > 3u) {
            node.meta[s] = 0x80u;
            node.imask |= (uint8_t)(1u << s);
            uint32_t slot_out = atomicAdd(&counters[1], 1u);
            if (slot_out < (uint32_t)n) tasks_out[slot_out] = make_uint2((uint32_t)c, node.child_base + rank);
            else atomicOr(&counters[4], 2u);
            rank++;
            local_sah += (double)ha;   // one traversal step into the child
        } else {
            uint32_t cnt = leaf_count[c];
            node.meta[s] = (uint8_t)((cnt << 5) | off);
            // collect the (<= 3) leaves of subtree c in order
            int stk[4];
            int sp = 0;
            stk[sp++] = c;
            uint32_t k = 0;
            while (sp > 0) {
                int x = stk[--sp];
                if (x >= nl) {
                    if (k < cnt) prim_order[prim_local + off + k] = sorted[x - nl];
                    k++;
                } else if (sp < 3) {
                    int2 ch = children[x];
                    stk[sp++] = ch.y;
                    stk[sp++] = ch.x;
                }
            }
            off += cnt;
            local_sah += (double)ha * (double)cnt;   // primitive tests
        }
    }
    atomicAdd(sah, local_sah);
    uint4* dst = reinterpret_cast<uint4*>(nodes + w);
    const uint4* src = reinterpret_cast<const uint4*>(&node);
    for (int k = 0; k < 5; k++) dst[k] = src[k];
}

__global__ void k_triangle_boxes(const float* __restrict__ pos, const uint32_t* __restrict__ idx, uint32_t vo,
                                 uint32_t io, uint32_t nt, float4* lo, float4* hi) {
    uint32_t t = blockIdx.x * BLK + threadIdx.x;
    if (t >= nt) return;
    float l[3] = {3.4e38f, 3.4e38f, 3.4e38f}, h[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    for (int k = 0; k < 3; k++) {
        const float* p = pos + 3ull * (vo + idx[io + 3ull * t + k]);
        for (int a = 0; a < 3; a++) { l[a] = fminf(l[a], p[a]); h[a] = fmaxf(h[a], p[a]); }
    }
    float ext = fmaxf(fmaxf(h[0] - l[0], h[1] - l[1]), h[2] - l[2]);
    for (int a = 0; a < 3; a++) {
        float pad = 1e-5f * (ext + fabsf(l[a]) + fabsf(h[a])) + 1e-7f;
        l[a] -= pad;
        h[a] += pad;
    }
    lo[t] = make_float4(l[0], l[1], l[2], 0.0f);
    hi[t] = make_float4(h[0], h[1], h[2], 0.0f);
}

__global__ void k_fill_triangles(const uint32_t* __restrict__ order, uint32_t n, const float* __restrict__ pos,
                                 const uint32_t* __restrict__ idx, uint32_t vo, uint32_t io, TriRecord* out) {
    uint32_t i = blockIdx.x * BLK + threadIdx.x;
    if (i >= n) return;
    uint32_t t = order[i];
    TriRecord r;
    float* v[3] = {r.v0, r.v1, r.v2};
    for (int k = 0; k < 3; k++) {
        const float* p = pos + 3ull * (vo + idx[io + 3ull * t + k]);
        v[k][0] = p[0]; v[k][1] = p[1]; v[k][2] = p[2]; v[k][3] = 0.0f;
    }
    r.v0[3] = __uint_as_float(t);
    out[i] = r;
}

__global__ void k_instance_boxes(const uint32_t* __restrict__ list, uint32_t n, const InstShade* __restrict__ inst,
                                 const MeshInfo* __restrict__ meshes, float4* lo, float4* hi) {
    uint32_t i = blockIdx.x * BLK + threadIdx.x;
    if (i >= n) return;
    const InstShade& I = inst[list[i]];
    const MeshInfo& M = meshes[I.mesh_id];
    float l[3] = {3.4e38f, 3.4e38f, 3.4e38f}, h[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    for (int c = 0; c < 8; c++) {
        V3 p = v3((c & 1) ? M.hi[0] : M.lo[0], (c & 2) ? M.hi[1] : M.lo[1], (c & 4) ? M.hi[2] : M.lo[2]);
        V3 q = xform_point(I.m, p);
        l[0] = fminf(l[0], q.x); l[1] = fminf(l[1], q.y); l[2] = fminf(l[2], q.z);
        h[0] = fmaxf(h[0], q.x); h[1] = fmaxf(h[1], q.y); h[2] = fmaxf(h[2], q.z);
    }
    float ext = fmaxf(fmaxf(h[0] - l[0], h[1] - l[1]), h[2] - l[2]);
    for (int a = 0; a < 3; a++) {
        float pad = 1e-5f * (ext + fabsf(l[a]) + fabsf(h[a])) + 1e-6f;
        l[a] -= pad;
        h[a] += pad;
    }
    lo[i] = make_float4(l[0], l[1], l[2], 0.0f);
    hi[i] = make_float4(h[0], h[1], h[2], 0.0f);
}

__global__ void k_map_prims(const uint32_t* __restrict__ order, const uint32_t* __restrict__ list, uint32_t n,
                            uint32_t* out) {
    uint32_t i = blockIdx.x * BLK + threadIdx.x;
    if (i < n) out[i] = list[order[i]];
}

inline unsigned grid_for(uint32_t n) { return (n + BLK - 1) / BLK; }

}  // namespace

Status build_wide_bvh(BuildScratch& sc, const float4* prim_lo, const float4* prim_hi, uint32_t n, WideNode* nodes,
                      uint32_t node_base, uint32_t prim_base, uint32_t* prim_order, cudaStream_t st,
                      BuildResult* out) {
    if (n == 0) return Status::Err(1, "build_wide_bvh: no primitives");
    if (n > (1u << 30)) return Status::Err(1, "build_wide_bvh: too many primitives");
    SNK_TRY_CUDA(sc.keys.reserve(n));
    SNK_TRY_CUDA(sc.keys_alt.reserve(n));
    SNK_TRY_CUDA(sc.vals.reserve(n));
    SNK_TRY_CUDA(sc.vals_alt.reserve(n));
    SNK_TRY_CUDA(sc.children.reserve(n));
    SNK_TRY_CUDA(sc.parent.reserve(2 * (size_t)n));
    SNK_TRY_CUDA(sc.flags.reserve(n));
    SNK_TRY_CUDA(sc.node_lo.reserve(2 * (size_t)n));
    SNK_TRY_CUDA(sc.node_hi.reserve(2 * (size_t)n));
    SNK_TRY_CUDA(sc.leaf_count.reserve(2 * (size_t)n));
    SNK_TRY_CUDA(sc.tasks_a.reserve(n));
    SNK_TRY_CUDA(sc.tasks_b.reserve(n));
    SNK_TRY_CUDA(sc.counters.reserve(5));
    SNK_TRY_CUDA(sc.cbounds.reserve(6));
    SNK_TRY_CUDA(sc.sah.reserve(1));

    k_init_bounds<<<1, 32, 0, st>>>(sc.cbounds.p);
    unsigned g = grid_for(n);
    k_centroid_bounds<<<g < 1024u ? g : 1024u, BLK, 0, st>>>(prim_lo, prim_hi, n, sc.cbounds.p);
    k_morton<<<g, BLK, 0, st>>>(prim_lo, prim_hi, n, sc.cbounds.p, sc.keys.p, sc.vals.p);
    SNK_TRY_CUDA(cudaGetLastError());

    cub::DoubleBuffer<unsigned long long> dk(sc.keys.p, sc.keys_alt.p);
    cub::DoubleBuffer<uint32_t> dv(sc.vals.p, sc.vals_alt.p);
    size_t tmp_bytes = 0;
    SNK_TRY_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, dk, dv, (int)n, 0, 63, st));
    SNK_TRY_CUDA(sc.cub_tmp.reserve(tmp_bytes));
    SNK_TRY_CUDA(cub::DeviceRadixSort::SortPairs(sc.cub_tmp.p, tmp_bytes, dk, dv, (int)n, 0, 63, st));
    const unsigned long long* keys = dk.Current();
    const uint32_t* sorted = dv.Current();

    SNK_TRY_CUDA(cudaMemsetAsync(sc.flags.p, 0, sizeof(int) * n, st));
    int minus1 = -1;
    SNK_TRY_CUDA(cudaMemcpyAsync(sc.parent.p, &minus1, sizeof(int), cudaMemcpyHostToDevice, st));
    if (n > 1) k_karras<<<grid_for(n - 1), BLK, 0, st>>>(keys, (int)n, sc.children.p, sc.parent.p);
    k_bottom_up<<<g, BLK, 0, st>>>(sorted, prim_lo, prim_hi, (int)n, sc.children.p, sc.parent.p, sc.flags.p,
                                   sc.node_lo.p, sc.node_hi.p, sc.leaf_count.p);
    SNK_TRY_CUDA(cudaGetLastError());

    float4 rlo, rhi;
    SNK_TRY_CUDA(cudaMemcpyAsync(&rlo, sc.node_lo.p, sizeof(float4), cudaMemcpyDeviceToHost, st));
    SNK_TRY_CUDA(cudaMemcpyAsync(&rhi, sc.node_hi.p, sizeof(float4), cudaMemcpyDeviceToHost, st));
    uint2 root_task = make_uint2(0u, node_base);
    uint32_t init_ctr[5] = {1u, 0u, 1u, 0u, 0u};
    SNK_TRY_CUDA(cudaMemcpyAsync(sc.tasks_a.p, &root_task, sizeof(uint2), cudaMemcpyHostToDevice, st));
    SNK_TRY_CUDA(cudaMemcpyAsync(sc.counters.p, init_ctr, sizeof(init_ctr), cudaMemcpyHostToDevice, st));
    SNK_TRY_CUDA(cudaMemsetAsync(sc.sah.p, 0, sizeof(double), st));
    SNK_TRY_CUDA(cudaStreamSynchronize(st));
    float rha = (rhi.x - rlo.x) * (rhi.y - rlo.y) + (rhi.y - rlo.y) * (rhi.z - rlo.z) + (rhi.z - rlo.z) * (rhi.x - rlo.x);
    if (!(rha > 0.0f)) rha = 1.0f;

    uint32_t ntasks = 1;
    uint2* tin = sc.tasks_a.p;
    uint2* tout = sc.tasks_b.p;
    for (int level = 0; ntasks > 0; level++) {
        if (level > 4096) return Status::Err(5, "build_wide_bvh: collapse did not terminate");
        k_collapse<<<grid_for(ntasks), BLK, 0, st>>>(tin, sc.counters.p, tout, (int)n, sc.children.p, sc.node_lo.p,
                                                     sc.node_hi.p, sc.leaf_count.p, sorted, nodes, node_base,
                                                     prim_base, prim_order, sc.sah.p, rha);
        SNK_TRY_CUDA(cudaGetLastError());
        uint32_t ctr[5];
        SNK_TRY_CUDA(cudaMemcpyAsync(ctr, sc.counters.p, sizeof(ctr), cudaMemcpyDeviceToHost, st));
        SNK_TRY_CUDA(cudaStreamSynchronize(st));
        if (ctr[4]) return Status::Err(5, "build_wide_bvh: collapse exceeded its capacity");
        ntasks = ctr[1];
        uint32_t next[2] = {ntasks, 0u};
        SNK_TRY_CUDA(cudaMemcpyAsync(sc.counters.p, next, sizeof(next), cudaMemcpyHostToDevice, st));
        std::swap(tin, tout);
        if (ntasks == 0) {
            if (ctr[3] != n) return Status::Err(2, "build_wide_bvh: primitive count mismatch");
            out->num_nodes = ctr[2];
        }
    }
    double sah = 0.0;
    SNK_TRY_CUDA(cudaMemcpyAsync(&sah, sc.sah.p, sizeof(double), cudaMemcpyDeviceToHost, st));
    SNK_TRY_CUDA(cudaStreamSynchronize(st));
    out->sah = 1.0 + sah;
    out->lo[0] = rlo.x; out->lo[1] = rlo.y; out->lo[2] = rlo.z;
    out->hi[0] = rhi.x; out->hi[1] = rhi.y; out->hi[2] = rhi.z;
    return Status::Ok();
}

Status launch_triangle_boxes(const float* positions, const uint32_t* indices, uint32_t vo, uint32_t io,
                             uint32_t nt, float4* lo, float4* hi, cudaStream_t s) {
    if (nt) k_triangle_boxes<<<grid_for(nt), BLK, 0, s>>>(positions, indices, vo, io, nt, lo, hi);
    SNK_TRY_CUDA(cudaGetLastError());
    return Status::Ok();
}

Status launch_fill_triangles(const uint32_t* order, uint32_t n, const float* positions, const uint32_t* indices,
                             uint32_t vo, uint32_t io, TriRecord* out, cudaStream_t s) {
    if (n) k_fill_triangles<<<grid_for(n), BLK, 0, s>>>(order, n, positions, indices, vo, io, out);
    SNK_TRY_CUDA(cudaGetLastError());
    return Status::Ok();
}

Status launch_instance_boxes(const uint32_t* list, uint32_t n, const InstShade* inst, const MeshInfo* meshes,
                             float4* lo, float4* hi, cudaStream_t s) {
    if (n) k_instance_boxes<<<grid_for(n), BLK, 0, s>>>(list, n, inst, meshes, lo, hi);
    SNK_TRY_CUDA(cudaGetLastError());
    return Status::Ok();
}

Status launch_map_prims(const uint32_t* order, const uint32_t* list, uint32_t n, uint32_t* out, cudaStream_t s) {
    if (n) k_map_prims<<<grid_for(n), BLK, 0, s>>>(order, list, n, out);
    SNK_TRY_CUDA(cudaGetLastError());
    return Status::Ok();
}

}  // namespace snk
