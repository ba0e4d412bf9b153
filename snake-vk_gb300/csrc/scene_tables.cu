// scene_tables.cu -- per-frame scene tables built on the device.
//
// Replaces the host packing of the reference's per-frame instance buffer
// (RaytracingBufferSystem, Core/src/scene/RaytracingBufferSystem.cpp:105-130:
// InstanceData per instance plus the emissive index list) and adds the
// path tracer's light-selection table.  From the caller's raw instance records
// (uploaded as they are) one launch per table writes
//   * the traversal record (world->object 3x4, BLAS root) and the shading
//     record (transforms, normal matrix, determinant) of every instance;
//   * one NEE record per emissive triangle (world-space vertices, unit normal,
//     radiance, area) with its selection weight 2 pi A lum(Le);
// and the weights become a CDF: each weight is quantised to an integer
// (w / w_max * 2^40, at least 1 for a positive weight), the integers are
// summed by an exact prefix scan, and cdf[k] = acc[k] / total, pmf[k] = q[k] /
// total in double rounded to float.  Integer sums do not depend on the order
// of summation, so the parallel scan and the oracle's sequential loop agree
// bit for bit.  This unit is compiled without contraction (--fmad=false): the
// float and double expressions round exactly as the oracle's.

#include <algorithm>
#include <cmath>
#include <vector>

#include "snk_host.h"

namespace snk {
namespace {

constexpr double LIGHT_Q_SCALE = 1099511627776.0;   // 2^40

// inverse of a row-major 3x4 affine transform in double rounded to float, the
// normal matrix transpose(inverse(mat3)) and determinant(mat3)
__device__ void invert_affine(const float* mf, float* inv_out, float* nmat_out, float* det_out) {
    double a[3][3], t[3];
    for (int r = 0; r < 3; r++) {
        for (int c = 0; c < 3; c++) a[r][c] = mf[4 * r + c];
        t[r] = mf[4 * r + 3];
    }
    const double c00 = a[1][1] * a[2][2] - a[1][2] * a[2][1];
    const double c01 = a[1][2] * a[2][0] - a[1][0] * a[2][2];
    const double c02 = a[1][0] * a[2][1] - a[1][1] * a[2][0];
    const double det = (a[0][0] * c00 + a[0][1] * c01) + a[0][2] * c02;
    double inv[3][3];
    inv[0][0] = c00 / det;
    inv[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) / det;
    inv[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) / det;
    inv[1][0] = c01 / det;
    inv[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) / det;
    inv[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) / det;
    inv[2][0] = c02 / det;
    inv[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) / det;
    inv[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) / det;
    for (int r = 0; r < 3; r++) {
        const double it = -((inv[r][0] * t[0] + inv[r][1] * t[1]) + inv[r][2] * t[2]);
        for (int c = 0; c < 3; c++) inv_out[4 * r + c] = (float)inv[r][c];
        inv_out[4 * r + 3] = (float)it;
    }
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) nmat_out[3 * r + c] = (float)inv[c][r];
    *det_out = (float)det;
}

__global__ void k_instance_records(const snk_instance* __restrict__ raw, uint32_t n, const MeshInfo* __restrict__ meshes,
                                   InstTrace* __restrict__ it, InstShade* __restrict__ is) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const snk_instance& in = raw[i];
    InstShade S;
    InstTrace T;
    for (int k = 0; k < 12; k++) {
        S.m[k] = in.transform[k];
        S.pm[k] = in.prev_transform[k];
    }
    invert_affine(S.m, T.inv, S.nmat, &S.det3);
    S.mesh_id = in.mesh_id;
    S.material_id = in.material_id;
    T.blas_root = meshes[in.mesh_id].blas_root;
    T.mesh_id = in.mesh_id;
    T.material_id = in.material_id;
    T.pad = 0;
    it[i] = T;
    is[i] = S;
}

__global__ void k_emissive_records(const uint32_t* __restrict__ em_list, uint32_t n_em,
                                   const InstShade* __restrict__ is, const MeshInfo* __restrict__ meshes,
                                   const MaterialDev* __restrict__ mats, EmissiveRec* __restrict__ recs) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_em) return;
    const uint32_t ii = em_list[e];
    const InstShade& I = is[ii];
    const MeshInfo& M = meshes[I.mesh_id];
    EmissiveRec r;
    for (int k = 0; k < 12; k++) r.m[k] = I.m[k];
    r.det3 = I.det3;
    r.inst = ii;
    r.ntri = M.num_triangles;
    r.index_offset = M.index_offset;
    r.vertex_offset = M.vertex_offset;
    for (int k = 0; k < 3; k++) r.albedo[k] = mats[I.material_id].albedo[k];
    recs[e] = r;
}

// one thread per emissive triangle j: emissive instance e = the last with
// first[e] <= j, triangle j - first[e] of its mesh
__global__ void k_emissive_lights(const snk_instance* __restrict__ raw, const uint32_t* __restrict__ em_list,
                                  const uint32_t* __restrict__ em_first, uint32_t n_em, uint32_t n_tri,
                                  const MeshInfo* __restrict__ meshes, const float* __restrict__ pos,
                                  const uint32_t* __restrict__ idx, const MaterialDev* __restrict__ mats,
                                  LocalLight* __restrict__ lights, double* __restrict__ w) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_tri) return;
    uint32_t lo = 0, hi = n_em - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (em_first[mid] <= j) lo = mid; else hi = mid - 1;
    }
    const uint32_t ii = em_list[lo];
    const uint32_t t = j - em_first[lo];
    const snk_instance& in = raw[ii];
    const MeshInfo& M = meshes[in.mesh_id];
    const uint32_t* tri = idx + M.index_offset + 3ull * t;
    LocalLight L;
    L.kind = 1;
    L.index = ii;
    L.pad0 = 0;
    L.pad1 = 0;
    const V3 p0 = xform_point(in.transform, load3(pos + 3ull * (M.vertex_offset + tri[0])));
    const V3 p1 = xform_point(in.transform, load3(pos + 3ull * (M.vertex_offset + tri[1])));
    const V3 p2 = xform_point(in.transform, load3(pos + 3ull * (M.vertex_offset + tri[2])));
    const V3 nl = cross(sub(p1, p0), sub(p2, p0));
    const float len = length(nl);
    const float area = 0.5f * len;
    const V3 nn = len > 0.0f ? divs(nl, len) : v3(0.0f, 1.0f, 0.0f);
    const V3 Le = load3(mats[in.material_id].albedo);
    L.p0[0] = p0.x; L.p0[1] = p0.y; L.p0[2] = p0.z; L.p0[3] = 0.0f;
    L.p1[0] = p1.x; L.p1[1] = p1.y; L.p1[2] = p1.z; L.p1[3] = 0.0f;
    L.p2[0] = p2.x; L.p2[1] = p2.y; L.p2[2] = p2.z; L.p2[3] = 0.0f;
    L.n[0] = nn.x; L.n[1] = nn.y; L.n[2] = nn.z; L.n[3] = 0.0f;
    L.L[0] = Le.x; L.L[1] = Le.y; L.L[2] = Le.z; L.L[3] = area;
    lights[j] = L;
    w[j] = 2.0 * M_PI * (double)area * (0.2126 * Le.x + 0.7152 * Le.y + 0.0722 * Le.z);
}

// largest positive weight, as the bits of a positive double (which order like
// the values); *wmax starts at 0
__global__ void k_weight_max(const double* __restrict__ w, uint32_t n, unsigned long long* wmax) {
    unsigned long long m = 0ull;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const double x = w[k];
        if (x > 0.0) m = max(m, (unsigned long long)__double_as_longlong(x));
    }
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
    if ((threadIdx.x & 31u) == 0 && m) atomicMax(wmax, m);
}

// integer weight of w[k], read by the prefix scan
struct QuantisedWeight {
    const double* w;
    const unsigned long long* wmax;
    __device__ __forceinline__ unsigned long long operator()(uint32_t k) const {
        const double wm = __longlong_as_double((long long)*wmax);
        const double x = w[k];
        return (x > 0.0 && wm > 0.0) ? max(1ull, __double2ull_rn(x / wm * LIGHT_Q_SCALE)) : 0ull;
    }
};

// the quantised weight of every light, once, over the whole grid (the double
// division is slow on this GPU, so the scan reads these instead of recomputing them)
__global__ void k_quantise(QuantisedWeight qw, uint32_t n, unsigned long long* q) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) q[k] = qw(k);
}

// Inclusive prefix sums of the quantised weights.  The sums are exact integers,
// so any order of summation gives the same bits: k_scan_tiles sums each tile of
// `tile` weights, k_scan_apply scans each tile (a contiguous run per thread, then
// the runs' totals across the block) starting from the sum of the tiles before it.
constexpr int SCAN_THREADS = 1024;

// inclusive scan of one value per thread across the block; *block_total = the sum
__device__ __forceinline__ unsigned long long block_scan_incl(unsigned long long v, unsigned long long* warp_tot,
                                                              unsigned long long* block_total) {
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    unsigned long long incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long u = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    unsigned long long off = 0ull, all = 0ull;
    for (int w = 0; w < SCAN_THREADS / 32; w++) {
        if (w < warp) off += warp_tot[w];
        all += warp_tot[w];
    }
    *block_total = all;
    return off + incl;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tiles(const unsigned long long* __restrict__ q, uint32_t n,
                                                             uint32_t tile, unsigned long long* tile_sums) {
    __shared__ unsigned long long warp_tot[SCAN_THREADS / 32];
    const uint32_t b0 = blockIdx.x * tile, b1 = min(b0 + tile, n);
    unsigned long long s = 0ull;
    for (uint32_t k = b0 + threadIdx.x; k < b1; k += SCAN_THREADS) s += q[k];
    unsigned long long total;
    block_scan_incl(s, warp_tot, &total);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(const unsigned long long* __restrict__ q, uint32_t n,
                                                             uint32_t tile,
                                                             const unsigned long long* __restrict__ tile_sums,
                                                             unsigned long long* acc) {
    __shared__ unsigned long long warp_tot[SCAN_THREADS / 32];
    __shared__ unsigned long long before;
    if (threadIdx.x == 0) {
        unsigned long long b = 0ull;
        for (uint32_t j = 0; j < blockIdx.x; j++) b += tile_sums[j];
        before = b;
    }
    const uint32_t b0 = blockIdx.x * tile, b1 = min(b0 + tile, n);
    const uint32_t per = (tile + SCAN_THREADS - 1) / SCAN_THREADS;
    const uint32_t r0 = min(b0 + threadIdx.x * per, b1), r1 = min(r0 + per, b1);
    unsigned long long s = 0ull;
    for (uint32_t k = r0; k < r1; k++) s += q[k];
    unsigned long long total;
    const unsigned long long incl = block_scan_incl(s, warp_tot, &total);   // (its barrier orders `before`)
    unsigned long long run = before + incl - s;
    for (uint32_t k = r0; k < r1; k++) {
        run += q[k];
        acc[k] = run;
    }
}

__global__ void k_light_cdf(const unsigned long long* __restrict__ acc, uint32_t n, float* __restrict__ cdf,
                            float* __restrict__ pmf) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const unsigned long long total = acc[n - 1];
    if (total == 0ull) {
        cdf[k] = 0.0f;
        pmf[k] = 0.0f;
        return;
    }
    const double tot = __ull2double_rn(total);
    const unsigned long long q = acc[k] - (k ? acc[k - 1] : 0ull);
    cdf[k] = k == n - 1 ? 1.0f : (float)(__ull2double_rn(acc[k]) / tot);
    pmf[k] = (float)(__ull2double_rn(q) / tot);
}

uint32_t blocks_for(uint32_t n, uint32_t b) { return (n + b - 1) / b; }

}  // namespace

Status launch_instance_records(const snk_instance* raw, uint32_t n, const MeshInfo* meshes, InstTrace* it,
                               InstShade* is, cudaStream_t st) {
    if (n == 0) return Status::Ok();
    k_instance_records<<<blocks_for(n, 128), 128, 0, st>>>(raw, n, meshes, it, is);
    SNK_TRY_CUDA(cudaGetLastError());
    return Status::Ok();
}

Status launch_emissive_records(const uint32_t* em_list, uint32_t n_em, const InstShade* is, const MeshInfo* meshes,
                               const MaterialDev* mats, EmissiveRec* recs, cudaStream_t st) {
    if (n_em == 0) return Status::Ok();
    k_emissive_records<<<blocks_for(n_em, 128), 128, 0, st>>>(em_list, n_em, is, meshes, mats, recs);
    SNK_TRY_CUDA(cudaGetLastError());
    return Status::Ok();
}

Status launch_emissive_lights(const snk_instance* raw, const uint32_t* em_list, const uint32_t* em_first, uint32_t n_em,
                              uint32_t n_tri, const MeshInfo* meshes, const float* pos, const uint32_t* idx,
                              const MaterialDev* mats, LocalLight* lights, double* w, cudaStream_t st) {
    if (n_tri == 0 || n_em == 0) return Status::Ok();
    k_emissive_lights<<<blocks_for(n_tri, 128), 128, 0, st>>>(raw, em_list, em_first, n_em, n_tri, meshes, pos, idx,
                                                              mats, lights, w);
    SNK_TRY_CUDA(cudaGetLastError());
    return Status::Ok();
}

Status launch_light_cdf(const double* w, uint32_t n, LightCdfScratch& sc, float* cdf, float* pmf, cudaStream_t st) {
    if (n == 0) return Status::Ok();
    // tiles of one weight per thread, or more when that would make over 1024 tiles
    const uint32_t per_thread = std::max<uint32_t>(1u, (uint32_t)((n + 1024ull * SCAN_THREADS - 1) /
                                                                  (1024ull * SCAN_THREADS)));
    const uint32_t tile = per_thread * SCAN_THREADS;
    const uint32_t tiles = (n + tile - 1) / tile;
    SNK_TRY_CUDA(sc.acc.reserve(n));
    SNK_TRY_CUDA(sc.q.reserve(n));
    SNK_TRY_CUDA(sc.wmax.reserve(1));
    SNK_TRY_CUDA(sc.tile_sums.reserve(tiles));
    const QuantisedWeight qw{w, sc.wmax.p};
    SNK_TRY_CUDA(cudaMemsetAsync(sc.wmax.p, 0, sizeof(unsigned long long), st));
    k_weight_max<<<std::min<uint32_t>(blocks_for(n, 256), 1024), 256, 0, st>>>(w, n, sc.wmax.p);
    k_quantise<<<std::min<uint32_t>(blocks_for(n, 256), 4096), 256, 0, st>>>(qw, n, sc.q.p);
    k_scan_tiles<<<tiles, SCAN_THREADS, 0, st>>>(sc.q.p, n, tile, sc.tile_sums.p);
    k_scan_apply<<<tiles, SCAN_THREADS, 0, st>>>(sc.q.p, n, tile, sc.tile_sums.p, sc.acc.p);
    SNK_TRY_CUDA(cudaGetLastError());
    k_light_cdf<<<blocks_for(n, 256), 256, 0, st>>>(sc.acc.p, n, cdf, pmf);
    SNK_TRY_CUDA(cudaGetLastError());
    return Status::Ok();
}

void light_cdf_host(const double* w, uint32_t n, float* cdf, float* pmf) {
    double wmax = 0.0;
    for (uint32_t k = 0; k < n; k++)
        if (w[k] > 0.0 && w[k] > wmax) wmax = w[k];
    std::vector<unsigned long long> q(n);
    unsigned long long total = 0ull;
    for (uint32_t k = 0; k < n; k++) {
        q[k] = (w[k] > 0.0 && wmax > 0.0)
                   ? std::max<unsigned long long>(1ull, (unsigned long long)std::llrint(w[k] / wmax * LIGHT_Q_SCALE))
                   : 0ull;
        total += q[k];
    }
    unsigned long long acc = 0ull;
    for (uint32_t k = 0; k < n; k++) {
        acc += q[k];
        cdf[k] = total ? (k + 1 == n ? 1.0f : (float)((double)acc / (double)total)) : 0.0f;
        pmf[k] = total ? (float)((double)q[k] / (double)total) : 0.0f;
    }
}

}  // namespace snk
