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
//   3. sort of (code, primitive) pairs (project kernels below: a bitonic network
//      in one CTA's shared memory up to 8192 pairs, an LSD radix sort in one CTA
//      up to 65,536, three kernels per radix digit beyond)
//   4. binary radix tree (Karras, HPG 2012): one thread per internal node
//   5. bottom-up boxes and leaf counts (atomic arrival flags)
//   5b. treelet restructuring (Karras & Aila, HPG 2013): bottom-up over the binary
//      tree, every node whose subtree holds >= 7 primitives roots a treelet of 7
//      leaves (grown by opening the largest-area treelet leaf); one warp finds the
//      SAH-optimal binary topology of those 7 leaves by dynamic programming over
//      all 127 leaf subsets and every 2-partition of each, and rewrites the
//      treelet's 6 internal nodes in place.  Subtrees of <= 3 primitives are
//      costed as the leaves the collapse will make of them.  Repeated for a few
//      passes; the result is deterministic (each treelet depends only on its
//      finished subtrees, ties break on the lowest subset index).
//   6. top-down collapse to 8-wide nodes, one thread per output node, level by
//      level: a node's children start as its binary children; the internal child
//      with the largest surface area and more than leaf_max primitives is replaced
//      by its two children until 8 children exist or none can be opened.  Children
//      with <= leaf_pack primitives (leaf_max <= leaf_pack <= 4) become leaves: a
//      full node keeps small subtrees as multi-primitive leaves instead of
//      spending a sparsely filled child node on them.  Children are assigned to the 8 slots greedily by how
//      well their centroid offset matches each octant corner, so that visiting
//      slot ^ ray_octant in increasing order is roughly front to back.  Child boxes
//      are quantised outwards to 8 bits per plane.
//   7. SAH cost of the result (for quality reporting).
//
// Mesh BVHs (built once, at load) take the multi-launch pipeline above.  The
// per-frame instance BVH of up to 1024 instances is built by one single-CTA
// launch instead (k_build_small: clustering in shared memory, then treelet passes
// and the same collapse), so that a frame's rebuild costs no host round trip.

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

// loads of tree data written by other threads during the build: through L2 for
// global memory (G), plain for shared memory (the single-CTA builder)
template <bool G, class T>
__device__ __forceinline__ T ldx(const T* p) {
    if constexpr (G) return __ldcg(p);
    else return *p;
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

// cb: encoded centroid bounds (min xyz, max xyz)
__device__ __forceinline__ unsigned long long morton_of(float4 a, float4 b, const unsigned* cb) {
    float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
    unsigned long long q[3];
    for (int k = 0; k < 3; k++) {
        float mn = dec_f(cb[k]), mx = dec_f(cb[3 + k]);
        float ext = mx - mn;
        float f = ext > 0.0f ? (c[k] - mn) / ext : 0.5f;
        f = fminf(fmaxf(f, 0.0f), 1.0f);
        q[k] = (unsigned long long)fminf(f * 2097152.0f, 2097151.0f);
    }
    return (spread21(q[0]) << 2) | (spread21(q[1]) << 1) | spread21(q[2]);
}

__global__ void k_morton(const float4* __restrict__ lo, const float4* __restrict__ hi, uint32_t n,
                         const unsigned* cb, unsigned long long* keys, uint32_t* vals) {
    uint32_t i = blockIdx.x * BLK + threadIdx.x;
    if (i >= n) return;
    keys[i] = morton_of(lo[i], hi[i], cb);
    vals[i] = i;
}

__device__ __forceinline__ int delta(const unsigned long long* __restrict__ k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    unsigned long long a = k[i], b = k[j];
    if (a == b) return 64 + __clz((unsigned)(i ^ j));
    return __clzll(a ^ b);
}

__device__ void karras_node(int i, const unsigned long long* __restrict__ keys, int n, int2* children, int* parent) {
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

// ---- radix sort of (63-bit Morton code, primitive) pairs ------------------------------
// LSD radix sort with 8-bit digits.  Every pass is stable: the elements of one
// digit keep their current order.  A CTA ranks a chunk of 1024 consecutive
// elements at a time: lanes holding the same digit find each other with
// __match_any_sync (their order within the warp is their lane order), every warp
// counts its digits in shared memory, and an exclusive scan of those counts over
// the warps gives each warp its start within the digit.  Up to SORT_SMALL_MAX
// elements (sets above the bitonic sort's 8192) one CTA runs all passes in
// one launch and skips the passes whose digit is the same for every key; larger
// sets (mesh BVHs, at load time) take three launches per pass (per-tile digit
// counts, their exclusive scan in digit-major order, the stable scatter).  The
// result is always back in the first buffer pair.
constexpr int SORT_THREADS = 1024;
constexpr int SORT_WARPS = SORT_THREADS / 32;
constexpr int SORT_RADIX = 256;
constexpr int SORT_PASSES = 8;                      // 64 bits (the codes use 63)
constexpr uint32_t SORT_SMALL_MAX = 1u << 16;
constexpr uint32_t SORT_TILE = 4u * SORT_THREADS;  // elements per CTA and pass (multi-CTA sort)

struct SortSmem {
    uint32_t wcnt[SORT_WARPS][SORT_RADIX];   // per-warp digit counts, then their exclusive scan
    uint32_t base[SORT_RADIX];               // next output position of each digit
    uint32_t total[SORT_RADIX];              // the current chunk's count of each digit
    uint32_t warp_sum[SORT_RADIX / 32];
};

__device__ __forceinline__ uint32_t sort_digit(unsigned long long k, int shift) {
    return (uint32_t)(k >> shift) & (SORT_RADIX - 1u);
}

// threads 0..255: base[d] = sum of in[0..d) (in may alias base)
__device__ __forceinline__ void scan_radix(SortSmem& S, const uint32_t* in) {
    const int t = threadIdx.x, lane = t & 31;
    uint32_t v = 0, incl = 0;
    if (t < SORT_RADIX) {
        v = in[t];
        incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += u;
        }
        if (lane == 31) S.warp_sum[t >> 5] = incl;
    }
    __syncthreads();
    if (t < SORT_RADIX) {
        uint32_t off = 0;
        for (int w = 0; w < (t >> 5); w++) off += S.warp_sum[w];
        S.base[t] = off + incl - v;
    }
    __syncthreads();
}

// Output position of this thread's element (valid, digit d) in a chunk of one
// element per thread, in thread order; then base advances past the chunk.
__device__ __forceinline__ uint32_t rank_chunk(SortSmem& S, bool valid, uint32_t d) {
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    for (int i = t; i < SORT_WARPS * SORT_RADIX; i += SORT_THREADS) (&S.wcnt[0][0])[i] = 0u;
    __syncthreads();
    const uint32_t key = valid ? d : (uint32_t)(SORT_RADIX + lane);   // lanes without an element match nobody
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, key);
    const uint32_t before = (uint32_t)__popc(peers & ((1u << lane) - 1u));
    if (valid && before == 0u) S.wcnt[warp][d] = (uint32_t)__popc(peers);
    __syncthreads();
    if (t < SORT_RADIX) {
        uint32_t run = 0;
        for (int w = 0; w < SORT_WARPS; w++) {
            const uint32_t c = S.wcnt[w][t];
            S.wcnt[w][t] = run;
            run += c;
        }
        S.total[t] = run;
    }
    __syncthreads();
    const uint32_t pos = valid ? S.base[d] + S.wcnt[warp][d] + before : 0u;
    __syncthreads();
    if (t < SORT_RADIX) S.base[t] += S.total[t];
    return pos;   // (the next chunk's first barrier orders the base update)
}

__global__ void __launch_bounds__(SORT_THREADS, 1) k_sort_small(unsigned long long* keys, uint32_t* vals,
                                                              unsigned long long* keys_alt, uint32_t* vals_alt,
                                                              uint32_t n) {
    __shared__ SortSmem S;
    __shared__ uint32_t hist[SORT_RADIX];
    __shared__ int skip;
    const int t = threadIdx.x;
    unsigned long long* sk = keys;
    uint32_t* sv = vals;
    unsigned long long* dk = keys_alt;
    uint32_t* dv = vals_alt;
    for (int pass = 0; pass < SORT_PASSES; pass++) {
        const int shift = 8 * pass;
        if (t < SORT_RADIX) hist[t] = 0u;
        __syncthreads();
        for (uint32_t i = t; i < n; i += SORT_THREADS) atomicAdd(&hist[sort_digit(sk[i], shift)], 1u);
        __syncthreads();
        if (t == 0) skip = hist[sort_digit(sk[0], shift)] == n;   // every key has this digit
        scan_radix(S, hist);
        if (skip) continue;
        for (uint32_t c = 0; c < n; c += SORT_THREADS) {
            const uint32_t i = c + (uint32_t)t;
            const bool valid = i < n;
            const unsigned long long k = valid ? sk[i] : 0ull;
            const uint32_t v = valid ? sv[i] : 0u;
            const uint32_t pos = rank_chunk(S, valid, sort_digit(k, shift));
            if (valid) { dk[pos] = k; dv[pos] = v; }
        }
        __syncthreads();
        unsigned long long* tk = sk; sk = dk; dk = tk;
        uint32_t* tv = sv; sv = dv; dv = tv;
    }
    if (sk != keys) {   // an odd number of passes ran: the result goes back to the first pair
        for (uint32_t i = t; i < n; i += SORT_THREADS) { keys[i] = sk[i]; vals[i] = sv[i]; }
    }
}

// Up to SORT_BITONIC_MAX pairs (the per-frame instance sets) one CTA sorts in shared
// memory with a bitonic network: 91 barrier-separated compare-exchange stages for
// 8192 entries instead of 8 radix passes over global memory.  The network is not
// stable by itself, so it orders by (key, value): the values are the primitives'
// indices 0..n-1 in their input order, which makes the result the stable order.
// Entries past n are padded with the largest pair.
constexpr uint32_t SORT_BITONIC_MAX = 8192;

__global__ void __launch_bounds__(SORT_THREADS, 1) k_sort_bitonic(unsigned long long* keys, uint32_t* vals,
                                                                uint32_t n) {
    extern __shared__ __align__(16) unsigned char sort_smem[];
    uint32_t N = 2;
    while (N < n) N <<= 1;
    unsigned long long* sk = reinterpret_cast<unsigned long long*>(sort_smem);
    uint32_t* sv = reinterpret_cast<uint32_t*>(sk + N);
    for (uint32_t i = threadIdx.x; i < N; i += SORT_THREADS) {
        sk[i] = i < n ? keys[i] : ~0ull;
        sv[i] = i < n ? vals[i] : ~0u;
    }
    __syncthreads();
    for (uint32_t k = 2; k <= N; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < N / 2; i += SORT_THREADS) {
                const uint32_t lo = ((i & ~(j - 1u)) << 1) | (i & (j - 1u)), hi = lo + j;
                const unsigned long long ka = sk[lo], kb = sk[hi];
                const uint32_t va = sv[lo], vb = sv[hi];
                const bool a_greater = ka > kb || (ka == kb && va > vb);
                if (a_greater == ((lo & k) == 0u)) {   // ascending blocks put the smaller first
                    sk[lo] = kb; sk[hi] = ka;
                    sv[lo] = vb; sv[hi] = va;
                }
            }
            __syncthreads();
        }
    }
    for (uint32_t i = threadIdx.x; i < n; i += SORT_THREADS) {
        keys[i] = sk[i];
        vals[i] = sv[i];
    }
}

// multi-CTA pass, step 1: digit counts of each tile, digit-major (hist[d * tiles + tile])
__global__ void __launch_bounds__(SORT_THREADS) k_sort_hist(const unsigned long long* __restrict__ keys, uint32_t n,
                                                            int shift, uint32_t* hist, uint32_t tiles) {
    __shared__ uint32_t h[SORT_RADIX];
    const int t = threadIdx.x;
    if (t < SORT_RADIX) h[t] = 0u;
    __syncthreads();
    const uint32_t b0 = blockIdx.x * SORT_TILE, b1 = min(b0 + SORT_TILE, n);
    for (uint32_t i = b0 + t; i < b1; i += SORT_THREADS) atomicAdd(&h[sort_digit(keys[i], shift)], 1u);
    __syncthreads();
    if (t < SORT_RADIX) hist[(size_t)t * tiles + blockIdx.x] = h[t];
}

// step 2: exclusive scan of the m = 256 x tiles counts in place (one CTA; each
// thread scans a contiguous run, the runs' totals are scanned across the block)
__global__ void __launch_bounds__(SORT_THREADS) k_sort_scan(uint32_t* hist, uint32_t m) {
    __shared__ uint32_t warp_tot[SORT_WARPS];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t per = (m + SORT_THREADS - 1) / SORT_THREADS;
    const uint32_t b0 = min((uint32_t)t * per, m), b1 = min(b0 + per, m);
    uint32_t sum = 0;
    for (uint32_t i = b0; i < b1; i++) sum += hist[i];
    uint32_t incl = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    uint32_t off = 0;
    for (int w = 0; w < warp; w++) off += warp_tot[w];
    uint32_t run = off + incl - sum;
    for (uint32_t i = b0; i < b1; i++) {
        const uint32_t c = hist[i];
        hist[i] = run;
        run += c;
    }
}

// step 3: stable scatter of each tile from its digits' scanned starts
__global__ void __launch_bounds__(SORT_THREADS, 1) k_sort_scatter(const unsigned long long* __restrict__ sk,
                                                                const uint32_t* __restrict__ sv, uint32_t n, int shift,
                                                                const uint32_t* __restrict__ hist, uint32_t tiles,
                                                                unsigned long long* dk, uint32_t* dv) {
    __shared__ SortSmem S;
    const int t = threadIdx.x;
    if (t < SORT_RADIX) S.base[t] = hist[(size_t)t * tiles + blockIdx.x];
    const uint32_t b0 = blockIdx.x * SORT_TILE, b1 = min(b0 + SORT_TILE, n);
    for (uint32_t c = b0; c < b1; c += SORT_THREADS) {
        const uint32_t i = c + (uint32_t)t;
        const bool valid = i < b1;
        const unsigned long long k = valid ? sk[i] : 0ull;
        const uint32_t v = valid ? sv[i] : 0u;
        const uint32_t pos = rank_chunk(S, valid, sort_digit(k, shift));
        if (valid) { dk[pos] = k; dv[pos] = v; }
    }
}

__global__ void k_karras(const unsigned long long* __restrict__ keys, int n, int2* children, int* parent) {
    int i = blockIdx.x * BLK + threadIdx.x;
    if (i < n - 1) karras_node(i, keys, n, children, parent);
}

template <bool G>
__device__ __forceinline__ void mem_fence() {
    if constexpr (G) __threadfence();
    else __threadfence_block();
}

// boxes and primitive counts from leaf j to the root (the second thread to
// arrive at a node completes it)
template <bool G>
__device__ void bottom_up_leaf(int j, const uint32_t* __restrict__ sorted, const float4* __restrict__ plo,
                               const float4* __restrict__ phi, int n, const int2* children, const int* parent,
                               int* flags, float4* node_lo, float4* node_hi, uint32_t* leaf_count) {
    int node = n - 1 + j;
    uint32_t prim = sorted[j];
    node_lo[node] = plo[prim];
    node_hi[node] = phi[prim];
    leaf_count[node] = 1;
    if (n == 1) return;
    int p = parent[node];
    while (p >= 0) {
        mem_fence<G>();
        if (atomicAdd(&flags[p], 1) == 0) return;
        mem_fence<G>();
        int2 ch = children[p];
        float4 al = ldx<G>(&node_lo[ch.x]), ah = ldx<G>(&node_hi[ch.x]);
        float4 bl = ldx<G>(&node_lo[ch.y]), bh = ldx<G>(&node_hi[ch.y]);
        uint32_t ca = ldx<G>(&leaf_count[ch.x]), cb = ldx<G>(&leaf_count[ch.y]);
        node_lo[p] = make_float4(fminf(al.x, bl.x), fminf(al.y, bl.y), fminf(al.z, bl.z), 0.0f);
        node_hi[p] = make_float4(fmaxf(ah.x, bh.x), fmaxf(ah.y, bh.y), fmaxf(ah.z, bh.z), 0.0f);
        leaf_count[p] = ca + cb;
        p = parent[p];
    }
}

__global__ void k_bottom_up(const uint32_t* __restrict__ sorted, const float4* __restrict__ plo,
                            const float4* __restrict__ phi, int n, const int2* __restrict__ children,
                            const int* __restrict__ parent, int* flags, float4* node_lo, float4* node_hi,
                            uint32_t* leaf_count) {
    int j = blockIdx.x * BLK + threadIdx.x;
    if (j < n) bottom_up_leaf<true>(j, sorted, plo, phi, n, children, parent, flags, node_lo, node_hi, leaf_count);
}

__device__ __forceinline__ float half_area(float4 lo, float4 hi) {
    float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    return dx * dy + dy * dz + dz * dx;
}

// ---- treelet restructuring -----------------------------------------------------
constexpr int TL_LEAVES = 7;
constexpr int TL_SUBSETS = 1 << TL_LEAVES;
constexpr int TL_WARPS = BLK / 32;
constexpr float SAH_CI = 1.2f;   // binary internal node
constexpr float SAH_CT = 1.0f;   // primitive

struct TreeletSmem {
    float area[TL_SUBSETS];
    float cost[TL_SUBSETS];
    uint32_t count[TL_SUBSETS];
    uint8_t part[TL_SUBSETS];
    float4 lo[TL_LEAVES], hi[TL_LEAVES];
    float leaf_cost[TL_LEAVES];
    uint32_t leaf_cnt[TL_LEAVES];
    int leaf[TL_LEAVES];
    int inner[TL_LEAVES - 1];
};

// subtrees of at most leaf_max primitives become leaves of the wide BVH
__device__ __forceinline__ float node_cost(float area, uint32_t cnt, float split_cost, uint32_t leaf_max) {
    return cnt <= leaf_max ? SAH_CT * area * (float)cnt : SAH_CI * area + split_cost;
}

// Optimises the treelet rooted at `root` (all 32 lanes of the warp call this).
template <bool G>
__device__ void treelet_optimise(int root, int nl, int2* children, int* parent, float4* node_lo, float4* node_hi,
                                 uint32_t* leaf_count, float* cost, TreeletSmem& T, uint32_t leaf_max) {
    const int lane = threadIdx.x & 31;
    const uint32_t total = ldx<G>(&leaf_count[root]);
    if (total < (uint32_t)TL_LEAVES) {
        // small subtree: only its cost (boxes and counts are already final)
        if (lane == 0) {
            int2 ch = ldx<G>(&children[root]);
            float c = ldx<G>(&cost[ch.x]) + ldx<G>(&cost[ch.y]);
            cost[root] = node_cost(half_area(ldx<G>(&node_lo[root]), ldx<G>(&node_hi[root])), total, c, leaf_max);
        }
        __syncwarp();
        return;
    }
    if (lane == 0) {
        int2 ch = ldx<G>(&children[root]);
        int L[TL_LEAVES];
        float A[TL_LEAVES];
        L[0] = ch.x; L[1] = ch.y;
        A[0] = half_area(ldx<G>(&node_lo[ch.x]), ldx<G>(&node_hi[ch.x]));
        A[1] = half_area(ldx<G>(&node_lo[ch.y]), ldx<G>(&node_hi[ch.y]));
        T.inner[0] = root;
        int nleaf = 2, ninner = 1;
        while (nleaf < TL_LEAVES) {
            int best = -1;
            float ba = -1.0f;
            for (int k = 0; k < nleaf; k++)
                if (L[k] < nl && A[k] > ba) { ba = A[k]; best = k; }
            // (a subtree of >= 7 primitives always has an internal node to open)
            int2 c2 = ldx<G>(&children[L[best]]);
            T.inner[ninner++] = L[best];
            L[best] = c2.x;
            A[best] = half_area(ldx<G>(&node_lo[c2.x]), ldx<G>(&node_hi[c2.x]));
            L[nleaf] = c2.y;
            A[nleaf] = half_area(ldx<G>(&node_lo[c2.y]), ldx<G>(&node_hi[c2.y]));
            nleaf++;
        }
        for (int k = 0; k < TL_LEAVES; k++) {
            T.leaf[k] = L[k];
            T.lo[k] = ldx<G>(&node_lo[L[k]]);
            T.hi[k] = ldx<G>(&node_hi[L[k]]);
            T.leaf_cost[k] = ldx<G>(&cost[L[k]]);
            T.leaf_cnt[k] = ldx<G>(&leaf_count[L[k]]);
        }
    }
    __syncwarp();
    // subset areas and primitive counts
    for (int sub = lane + 1; sub < TL_SUBSETS; sub += 32) {
        float4 lo = make_float4(3.4e38f, 3.4e38f, 3.4e38f, 0.0f), hi = make_float4(-3.4e38f, -3.4e38f, -3.4e38f, 0.0f);
        uint32_t cnt = 0;
        for (int k = 0; k < TL_LEAVES; k++) {
            if (!(sub & (1 << k))) continue;
            float4 a = T.lo[k], b = T.hi[k];
            lo.x = fminf(lo.x, a.x); lo.y = fminf(lo.y, a.y); lo.z = fminf(lo.z, a.z);
            hi.x = fmaxf(hi.x, b.x); hi.y = fmaxf(hi.y, b.y); hi.z = fmaxf(hi.z, b.z);
            cnt += T.leaf_cnt[k];
        }
        T.area[sub] = half_area(lo, hi);
        T.count[sub] = cnt;
        if (__popc(sub) == 1) { T.cost[sub] = T.leaf_cost[__ffs(sub) - 1]; T.part[sub] = 0; }
    }
    __syncwarp();
    // subsets of 2..6 leaves, by size; every unordered 2-partition (the part that
    // holds the lowest leaf is enumerated)
    for (int size = 2; size < TL_LEAVES; size++) {
        for (int sub = lane + 1; sub < TL_SUBSETS; sub += 32) {
            if (__popc(sub) != size) continue;
            const int low = sub & -sub, rest = sub ^ low;
            float best = 3.4e38f;
            int bp = 0;
            // P = low | q over the proper subsets q of rest (q = rest would be all of sub)
            for (int q = (rest - 1) & rest;; q = (q - 1) & rest) {
                const int P = low | q;
                float c = T.cost[P] + T.cost[sub ^ P];
                if (c < best || (c == best && P < bp)) { best = c; bp = P; }
                if (q == 0) break;
            }
            T.cost[sub] = node_cost(T.area[sub], T.count[sub], best, leaf_max);
            T.part[sub] = (uint8_t)bp;
        }
        __syncwarp();
    }
    // the full set: 63 partitions across the warp
    {
        const int full = TL_SUBSETS - 1;
        float best = 3.4e38f;
        int bp = 0;
        for (int q = lane; q < (TL_SUBSETS >> 1) - 1; q += 32) {
            int P = 1 | (q << 1);
            float c = T.cost[P] + T.cost[full ^ P];
            if (c < best || (c == best && P < bp)) { best = c; bp = P; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            float ob = __shfl_xor_sync(0xFFFFFFFFu, best, o);
            int op = __shfl_xor_sync(0xFFFFFFFFu, bp, o);
            if (ob < best || (ob == best && op < bp)) { best = ob; bp = op; }
        }
        if (lane == 0) {
            T.cost[full] = node_cost(T.area[full], T.count[full], best, leaf_max);
            T.part[full] = (uint8_t)bp;
        }
    }
    __syncwarp();
    // rewrite the treelet's internal nodes (lane 0; 6 nodes)
    if (lane == 0) {
        int stk_sub[TL_LEAVES], stk_node[TL_LEAVES];
        int sp = 0, next = 1;
        stk_sub[sp] = TL_SUBSETS - 1; stk_node[sp] = T.inner[0]; sp++;
        while (sp > 0) {
            --sp;
            const int sub = stk_sub[sp], node = stk_node[sp];
            const int P = T.part[sub], Q = sub ^ P;
            int cidx[2];
            const int halves[2] = {P, Q};
            for (int h = 0; h < 2; h++) {
                const int hs = halves[h];
                if (__popc(hs) == 1) {
                    cidx[h] = T.leaf[__ffs(hs) - 1];
                } else {
                    cidx[h] = T.inner[next++];
                    stk_sub[sp] = hs; stk_node[sp] = cidx[h]; sp++;
                }
                parent[cidx[h]] = node;
            }
            children[node] = make_int2(cidx[0], cidx[1]);
            float4 lo = make_float4(3.4e38f, 3.4e38f, 3.4e38f, 0.0f), hi = make_float4(-3.4e38f, -3.4e38f, -3.4e38f, 0.0f);
            for (int k = 0; k < TL_LEAVES; k++) {
                if (!(sub & (1 << k))) continue;
                float4 a = T.lo[k], b = T.hi[k];
                lo.x = fminf(lo.x, a.x); lo.y = fminf(lo.y, a.y); lo.z = fminf(lo.z, a.z);
                hi.x = fmaxf(hi.x, b.x); hi.y = fmaxf(hi.y, b.y); hi.z = fmaxf(hi.z, b.z);
            }
            node_lo[node] = lo;
            node_hi[node] = hi;
            leaf_count[node] = T.count[sub];
            cost[node] = T.cost[sub];
        }
    }
    __syncwarp();
}

// One restructuring pass, leaf j of this thread (every lane of the warp calls
// it): each thread climbs towards the root; the second thread to reach a node
// hands that node's treelet to its whole warp.
template <bool G>
__device__ void treelet_climb(int j, int n, int2* children, int* parent, int* flags, float4* node_lo,
                              float4* node_hi, uint32_t* leaf_count, float* cost, TreeletSmem& T, uint32_t leaf_max) {
    const int nl = n - 1;
    bool active = j < n;
    int cur = nl + j;
    if (active) cost[cur] = SAH_CT * half_area(node_lo[cur], node_hi[cur]);
    while (true) {
        int p = -1;
        bool ready = false;
        if (active) {
            p = ldx<G>(&parent[cur]);
            if (p < 0) {
                active = false;
            } else {
                mem_fence<G>();
                if (atomicAdd(&flags[p], 1) == 0) active = false;
                else ready = true;
                mem_fence<G>();
            }
        }
        unsigned m = __ballot_sync(0xFFFFFFFFu, ready);
        while (m) {
            const int l = __ffs(m) - 1;
            m &= m - 1;
            const int root = __shfl_sync(0xFFFFFFFFu, p, l);
            treelet_optimise<G>(root, nl, children, parent, node_lo, node_hi, leaf_count, cost, T, leaf_max);
        }
        mem_fence<G>();
        if (ready) cur = p;
        if (!__any_sync(0xFFFFFFFFu, active)) break;
    }
}

__global__ void __launch_bounds__(BLK) k_treelet_pass(int n, int2* children, int* parent, int* flags,
                                                      float4* node_lo, float4* node_hi, uint32_t* leaf_count,
                                                      float* cost, uint32_t leaf_max) {
    __shared__ TreeletSmem smem[TL_WARPS];
    treelet_climb<true>(blockIdx.x * BLK + threadIdx.x, n, children, parent, flags, node_lo, node_hi, leaf_count,
                        cost, smem[threadIdx.x >> 5], leaf_max);
}

// smallest power-of-two exponent (biased) with 2^(e-127) >= x; at least 1
__device__ __forceinline__ uint32_t ceil_exp_biased(float x) {
    uint32_t b = __float_as_uint(x);
    uint32_t e = (b >> 23) & 0xFFu;
    if (e == 0) return 1u;
    if (b & 0x7FFFFFu) e += 1;
    return e > 254u ? 254u : e;
}

// 8-bit child-box quantisation of a wide node: a power-of-two scale per axis
// (the smallest with 255 steps covering the parent box, rounded up) and child
// planes rounded outwards, so the decoded boxes always contain the exact ones.
struct QuantFrame {
    float p[3], inv_scale[3];
    uint32_t eb[3];
};
__device__ __forceinline__ QuantFrame quant_frame(float4 plo, float4 phi) {
    QuantFrame F;
    const float ex_[3] = {__fsub_ru(phi.x, plo.x), __fsub_ru(phi.y, plo.y), __fsub_ru(phi.z, plo.z)};
    F.p[0] = plo.x; F.p[1] = plo.y; F.p[2] = plo.z;
    for (int a = 0; a < 3; a++) {
        F.eb[a] = ceil_exp_biased(__fdiv_ru(ex_[a], 255.0f));
        F.inv_scale[a] = __uint_as_float((254u - F.eb[a]) << 23);   // 2^(127 - (eb - 127))
    }
    return F;
}
__device__ __forceinline__ void quant_child(const QuantFrame& F, float4 a4, float4 z4, WideNode& node, int s) {
    const float clo[3] = {a4.x, a4.y, a4.z}, chi[3] = {z4.x, z4.y, z4.z};
    for (int a = 0; a < 3; a++) {
        const float ql = floorf(__fmul_rd(__fsub_rd(clo[a], F.p[a]), F.inv_scale[a]));
        const float qh = ceilf(__fmul_ru(__fsub_ru(chi[a], F.p[a]), F.inv_scale[a]));
        node.qlo[a][s] = (uint8_t)fminf(fmaxf(ql, 0.0f), 255.0f);
        node.qhi[a][s] = (uint8_t)fminf(fmaxf(qh, 0.0f), 255.0f);
    }
}

// ---- SAH-optimal 8-wide collapse ------------------------------------------------
// Dynamic programming over the binary tree (Ylitie, Karras, Laine, HPG 2017): for
// every internal node x and every i in 1..8, D(x, i) is the least SAH cost of the
// subtree of x represented by at most i children of a wide node.  A child is x
// itself (a wide node of cost WIDE_CN A(x) plus the best distribution of x's
// subtree over 8 children, or a leaf of WIDE_CT A(x) per primitive when x holds at
// most leaf_pack primitives), or the children of a split of the i slots between
// x's two binary children.  wide_split[x] packs the argmins in 4-bit fields: field
// 0 the split of a wide node rooted at x (8 slots), field i - 1 (i = 2..8) the
// choice for D(x, i): 0 keeps x as one child, k > 0 gives k slots to the left child
// and i - k to the right one.
constexpr float WIDE_CN = 1.0f;   // one 8-wide node test
constexpr float WIDE_CT = 1.0f;   // one primitive test (0.3 and 0.6 gave the same trees on the test scenes)

template <bool G>
__device__ __forceinline__ void wide_costs(int c, int nl, const float4* node_lo, const float4* node_hi,
                                           const float* wide_cost, float d[8]) {
    if (c >= nl) {
        const float v = WIDE_CT * half_area(ldx<G>(&node_lo[c]), ldx<G>(&node_hi[c]));
#pragma unroll
        for (int i = 0; i < 8; i++) d[i] = v;
    } else {
        const float4* src = reinterpret_cast<const float4*>(wide_cost + 8 * (size_t)c);
        const float4 a = ldx<G>(src), b = ldx<G>(src + 1);
        d[0] = a.x; d[1] = a.y; d[2] = a.z; d[3] = a.w; d[4] = b.x; d[5] = b.y; d[6] = b.z; d[7] = b.w;
    }
}

// D(p, 1..8) and wide_split[p] of internal node p from its two children's entries
template <bool G>
__device__ __forceinline__ void wide_cost_node(int p, int nl, const int2* children, const float4* node_lo,
                                               const float4* node_hi, const uint32_t* leaf_count, float* wide_cost,
                                               uint32_t* wide_split, uint32_t leaf_max, uint32_t leaf_pack) {
    const int2 ch = ldx<G>(&children[p]);
    float a[8], b[8];
    wide_costs<G>(ch.x, nl, node_lo, node_hi, wide_cost, a);
    wide_costs<G>(ch.y, nl, node_lo, node_hi, wide_cost, b);
    float e[9];
    uint32_t ek[9];
#pragma unroll
    for (int i = 2; i <= 8; i++) {
        float best = a[0] + b[i - 2];
        uint32_t bk = 1;
#pragma unroll
        for (int k = 2; k < i; k++) {
            const float c = a[k - 1] + b[i - k - 1];
            if (c < best) { best = c; bk = (uint32_t)k; }
        }
        e[i] = best;
        ek[i] = bk;
    }
    const float area = half_area(ldx<G>(&node_lo[p]), ldx<G>(&node_hi[p]));
    const uint32_t cnt = ldx<G>(&leaf_count[p]);
    const float d1 = cnt <= leaf_pack ? WIDE_CT * area * (float)cnt : WIDE_CN * area + e[8];
    float d[8];
    uint32_t split = ek[8];
    d[0] = d1;
#pragma unroll
    for (int i = 2; i <= 8; i++) {
        const bool open = cnt > leaf_max && e[i] < d1;   // subtrees of at most leaf_max primitives stay leaves
        d[i - 1] = open ? e[i] : d1;
        split |= (open ? ek[i] : 0u) << (4 * (i - 1));
    }
    float4* dst = reinterpret_cast<float4*>(wide_cost + 8 * (size_t)p);
    dst[0] = make_float4(d[0], d[1], d[2], d[3]);
    dst[1] = make_float4(d[4], d[5], d[6], d[7]);
    wide_split[p] = split;
}

// bottom-up from leaf j of n (the second thread to arrive at a node completes it)
template <bool G>
__device__ void wide_cost_climb(int j, int n, const int2* children, const int* parent, int* flags,
                                const float4* node_lo, const float4* node_hi, const uint32_t* leaf_count,
                                float* wide_cost, uint32_t* wide_split, uint32_t leaf_max, uint32_t leaf_pack) {
    if (n == 1) return;
    const int nl = n - 1;
    int p = parent[nl + j];
    while (p >= 0) {
        mem_fence<G>();
        if (atomicAdd(&flags[p], 1) == 0) return;
        mem_fence<G>();
        wide_cost_node<G>(p, nl, children, node_lo, node_hi, leaf_count, wide_cost, wide_split, leaf_max, leaf_pack);
        p = parent[p];
    }
}

__global__ void k_collapse_cost(int n, const int2* __restrict__ children, const int* __restrict__ parent, int* flags,
                                const float4* __restrict__ node_lo, const float4* __restrict__ node_hi,
                                const uint32_t* __restrict__ leaf_count, float* wide_cost, uint32_t* wide_split,
                                uint32_t leaf_max, uint32_t leaf_pack) {
    const int j = blockIdx.x * BLK + threadIdx.x;
    if (j < n)
        wide_cost_climb<true>(j, n, children, parent, flags, node_lo, node_hi, leaf_count, wide_cost, wide_split,
                              leaf_max, leaf_pack);
}

// the children of the wide node rooted at internal node b chosen by wide_split
// (the least-SAH distribution of b's subtree over 8 slots); returns their number
__device__ __forceinline__ int wide_children(int b, int nl, const int2* children, const uint32_t* wide_split,
                                             int C[8]) {
    int sn[8], ss[8], sp = 0, nc = 0;
    const int2 ch = children[b];
    const int k8 = (int)(wide_split[b] & 15u);
    sn[sp] = ch.y; ss[sp++] = 8 - k8;
    sn[sp] = ch.x; ss[sp++] = k8;
    while (sp > 0 && nc < 8) {
        const int y = sn[--sp], slots = ss[sp];
        const int k = (y >= nl || slots <= 1) ? 0 : (int)((wide_split[y] >> (4 * (slots - 1))) & 15u);
        if (k == 0 || k >= slots || sp > 6) {
            C[nc++] = y;
        } else {
            const int2 cy = children[y];
            sn[sp] = cy.y; ss[sp++] = slots - k;
            sn[sp] = cy.x; ss[sp++] = k;
        }
    }
    return sp > 0 ? -1 : nc;   // -1: more than 8 children (never with a consistent table)
}

// One output node: task = (binary node, wide node slot).  counters: [1] tasks
// out, [2] wide nodes, [3] primitive slots, [4] capacity error bits.
__device__ void collapse_task(uint2 task, uint32_t* counters, uint2* tasks_out, int n,
                              const int2* __restrict__ children, const float4* __restrict__ node_lo,
                              const float4* __restrict__ node_hi, const uint32_t* __restrict__ leaf_count,
                              const uint32_t* __restrict__ sorted, WideNode* nodes, uint32_t node_base,
                              uint32_t prim_base, uint32_t* prim_order, double* sah, float root_half_area,
                              uint32_t leaf_max, uint32_t leaf_pack, const uint32_t* __restrict__ wide_split) {
    int b = (int)task.x;
    uint32_t w = task.y;
    const int nl = n - 1;  // first leaf id
    int C[8];
    int nc;
    if (b >= nl) { C[0] = b; nc = 1; }
    else if (wide_split) {
        nc = wide_children(b, nl, children, wide_split, C);
        if (nc < 0) { atomicOr(&counters[4], 8u); return; }
    }
    else { int2 ch = children[b]; C[0] = ch.x; C[1] = ch.y; nc = 2; }
    while (!wide_split && nc < 8) {
        int best = -1;
        float best_a = -1.0f;
        for (int k = 0; k < nc; k++) {
            int c = C[k];
            if (c < nl && leaf_count[c] > leaf_max) {
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
        if (c < nl && leaf_count[c] > leaf_pack) n_int++;
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
    const QuantFrame F = quant_frame(plo, phi);
    WideNode node;
    node.px = plo.x; node.py = plo.y; node.pz = plo.z;
    node.ex = (uint8_t)F.eb[0]; node.ey = (uint8_t)F.eb[1]; node.ez = (uint8_t)F.eb[2];
    node.imask = 0;
    node.child_base = node_base + child_local;
    node.prim_base = prim_base + prim_local;
    uint32_t rank = 0, off = 0;
    double local_sah = 0.0;
    for (int s = 0; s < 8; s++) {
        int c = slot_child[s];
        if (c < 0) {
            node.meta[s] = 0;
            for (int a = 0; a < 3; a++) { node.qlo[a][s] = 0; node.qhi[a][s] = 0; }
            continue;
        }
        float4 a4 = node_lo[c], z4 = node_hi[c];
        quant_child(F, a4, z4, node, s);
        const float ha = sah ? half_area(a4, z4) / root_half_area : 0.0f;
        if (c < nl && leaf_count[c] > leaf_pack) {
            node.meta[s] = (uint8_t)META_INTERNAL;
            node.imask |= (uint8_t)(1u << s);
            uint32_t slot_out = atomicAdd(&counters[1], 1u);
            if (slot_out < (uint32_t)n) tasks_out[slot_out] = make_uint2((uint32_t)c, node.child_base + rank);
            else atomicOr(&counters[4], 2u);
            rank++;
            local_sah += (double)ha;   // one traversal step into the child
        } else {
            uint32_t cnt = leaf_count[c];
            node.meta[s] = (uint8_t)((cnt << 5) | off);
            // collect the (<= leaf_pack) leaves of subtree c in order
            int stk[8];
            int sp = 0;
            stk[sp++] = c;
            uint32_t k = 0;
            while (sp > 0) {
                int x = stk[--sp];
                if (x >= nl) {
                    if (k < cnt) prim_order[prim_local + off + k] = sorted[x - nl];
                    k++;
                } else if (sp < 7) {
                    int2 ch = children[x];
                    stk[sp++] = ch.y;
                    stk[sp++] = ch.x;
                } else {
                    atomicOr(&counters[4], 4u);   // deeper than a subtree of leaf_pack leaves can be
                }
            }
            off += cnt;
            local_sah += (double)ha * (double)cnt;   // primitive tests
        }
    }
    if (sah) atomicAdd(sah, local_sah);
    uint4* dst = reinterpret_cast<uint4*>(nodes + w);
    const uint4* src = reinterpret_cast<const uint4*>(&node);
    for (int k = 0; k < 5; k++) dst[k] = src[k];
}

__global__ void k_collapse(const uint2* __restrict__ tasks_in, uint32_t* counters, uint2* tasks_out, int n,
                           const int2* __restrict__ children, const float4* __restrict__ node_lo,
                           const float4* __restrict__ node_hi, const uint32_t* __restrict__ leaf_count,
                           const uint32_t* __restrict__ sorted, WideNode* nodes, uint32_t node_base,
                           uint32_t prim_base, uint32_t* prim_order, double* sah, float root_half_area,
                           uint32_t leaf_max, uint32_t leaf_pack, const uint32_t* __restrict__ wide_split) {
    uint32_t ti = blockIdx.x * BLK + threadIdx.x;
    if (ti >= counters[0]) return;
    collapse_task(tasks_in[ti], counters, tasks_out, n, children, node_lo, node_hi, leaf_count, sorted, nodes,
                  node_base, prim_base, prim_order, sah, root_half_area, leaf_max, leaf_pack, wide_split);
}

// ---- single-CTA agglomerative builder for small primitive sets -----------------
// The per-frame instance BVH (<= 1024 instances): one block of 1024 threads, every
// array in shared memory, one launch, no host synchronisation.  Locally-ordered
// clustering (PLOC, Meister & Bittner, TVCG 2018): clusters start as the
// primitives in Morton order; every round, each cluster finds the neighbour
// within PLOC_RADIUS positions whose merged box has the least surface area (ties:
// the lower position), mutual nearest neighbours merge into a new binary node, and
// the cluster list is compacted in order.  The globally closest pair is always
// mutual, so every round merges at least once.  Large boxes (a ground plane that
// spans the scene) are nobody's nearest neighbour and end up near the root.
// Internal node ids count down from n-2 as merges happen (the last merge is the
// root, node 0); leaves are n-1 + their Morton position, so the 8-wide collapse
// above applies unchanged.
constexpr int SMALL_THREADS = 1024;
constexpr int PLOC_RADIUS = 16;
static_assert(SMALL_BUILD_MAX == SMALL_THREADS, "one cluster per thread");

struct SmallSmem {
    unsigned long long keys[SMALL_BUILD_MAX];
    uint32_t vals[SMALL_BUILD_MAX];            // primitive at Morton position k
    int clusters[2][SMALL_BUILD_MAX];          // node ids of the live clusters, in order
    int2 children[SMALL_BUILD_MAX];
    float4 node_lo[2 * SMALL_BUILD_MAX], node_hi[2 * SMALL_BUILD_MAX];
    uint32_t leaf_count[2 * SMALL_BUILD_MAX];
    uint2 tasks[2][SMALL_BUILD_MAX];
    int parent[2 * SMALL_BUILD_MAX];           // treelet passes
    int flags[SMALL_BUILD_MAX];
    float cost[2 * SMALL_BUILD_MAX];
    uint32_t warp_sums[32];
    uint32_t counters[8];
    unsigned cb[6];
    double sah;
    union {
        TreeletSmem tl[SMALL_THREADS / 32];    // treelet passes
        struct {                               // then the least-SAH collapse table
            float wide_cost[8 * SMALL_BUILD_MAX];
            uint32_t wide_split[SMALL_BUILD_MAX];
        } dp;
    };
    WideNode stage[SMALL_THREADS / 32];        // per-warp staging of collapsed nodes
};
static_assert(sizeof(SmallSmem) <= 227 * 1024, "single-CTA builder exceeds shared memory");

__device__ __forceinline__ float4 f4min(float4 a, float4 b) {
    return make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), 0.0f);
}
__device__ __forceinline__ float4 f4max(float4 a, float4 b) {
    return make_float4(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z), 0.0f);
}

// inclusive block-wide sum of v (all SMALL_THREADS threads); *total = block sum
__device__ __forceinline__ uint32_t block_scan(uint32_t v, uint32_t* warp_sums, uint32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) warp_sums[warp] = v;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_sums[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= o) w += t;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    const uint32_t r = v + (warp ? warp_sums[warp - 1] : 0u);
    *total = warp_sums[31];
    __syncthreads();
    return r;
}

// float -> unsigned with the same order (for warp max reductions)
__device__ __forceinline__ unsigned order_f(float f) {
    const unsigned b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// collapse_task for a whole warp (every lane passes the same task): the same
// greedy choices, made with warp reductions instead of one thread's loops.
// counters: [2] wide nodes, [3] primitive slots, [4] capacity error bits;
// next_tasks counts the child tasks queued in tasks_out.
// Lane k < nc holds candidate child k while the node is opened; the 64 (child,
// slot) pairs p = 8k + s of the slot assignment are spread two per lane; lane s
// < 8 then builds slot s.  Ties go to the lowest child / pair index, as in the
// sequential loops.  stage: this warp's 80-byte staging node in shared memory.
__device__ void collapse_task_warp(uint2 task, uint32_t* counters, uint32_t* next_tasks, uint2* tasks_out, int n,
                                   const int2* children,
                                   const float4* node_lo, const float4* node_hi, const uint32_t* leaf_count,
                                   const uint32_t* sorted, WideNode* nodes, WideNode* stage, uint32_t node_base,
                                   uint32_t prim_base, uint32_t* prim_order, uint32_t leaf_max, uint32_t leaf_pack,
                                   const uint32_t* wide_split) {
    constexpr unsigned FULL = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    const int b = (int)task.x;
    const uint32_t w = task.y;
    const int nl = n - 1;   // first leaf id
    int c = -1, nc;
    if (b >= nl) {
        nc = 1;
        if (lane == 0) c = b;
    } else if (wide_split) {
        // the least-SAH children (lane 0 expands the split table, lane k takes child k)
        int C[8];
        int m = 0;
        if (lane == 0) m = wide_children(b, nl, children, wide_split, C);
        m = __shfl_sync(FULL, m, 0);
        if (m < 0) {
            if (lane == 0) atomicOr(&counters[4], 8u);
            return;
        }
        nc = m;
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const int v = __shfl_sync(FULL, (lane == 0 && k < m) ? C[k] : -1, 0);
            if (lane == k) c = v;
        }
    } else {
        const int2 ch = children[b];
        nc = 2;
        c = lane == 0 ? ch.x : (lane == 1 ? ch.y : -1);
    }
    // greedy: open the largest internal candidate (more than leaf_max primitives) until 8 children
    while (!wide_split && nc < 8) {
        const bool elig = lane < nc && c < nl && leaf_count[c] > leaf_max;
        const unsigned key = elig ? __float_as_uint(half_area(node_lo[c], node_hi[c])) + 1u : 0u;   // areas >= 0
        const unsigned mx = __reduce_max_sync(FULL, key);
        if (mx == 0u) break;
        const int best = __ffs(__ballot_sync(FULL, key == mx)) - 1;
        const int cb = __shfl_sync(FULL, c, best);
        const int2 ch = children[cb];
        if (lane == best) c = ch.x;
        if (lane == nc) c = ch.y;
        nc++;
    }
    // parent box (min / max are exact, so the reduction order does not matter)
    float4 lo = make_float4(3.4e38f, 3.4e38f, 3.4e38f, 0.0f), hi = make_float4(-3.4e38f, -3.4e38f, -3.4e38f, 0.0f);
    float4 clo = lo, chi = hi;
    if (lane < nc) { clo = node_lo[c]; chi = node_hi[c]; lo = clo; hi = chi; }
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
        lo.x = fminf(lo.x, __shfl_xor_sync(FULL, lo.x, o)); lo.y = fminf(lo.y, __shfl_xor_sync(FULL, lo.y, o));
        lo.z = fminf(lo.z, __shfl_xor_sync(FULL, lo.z, o));
        hi.x = fmaxf(hi.x, __shfl_xor_sync(FULL, hi.x, o)); hi.y = fmaxf(hi.y, __shfl_xor_sync(FULL, hi.y, o));
        hi.z = fmaxf(hi.z, __shfl_xor_sync(FULL, hi.z, o));
    }
    const float4 plo = make_float4(__shfl_sync(FULL, lo.x, 0), __shfl_sync(FULL, lo.y, 0), __shfl_sync(FULL, lo.z, 0), 0.0f);
    const float4 phi = make_float4(__shfl_sync(FULL, hi.x, 0), __shfl_sync(FULL, hi.y, 0), __shfl_sync(FULL, hi.z, 0), 0.0f);
    const float pcx = 0.5f * (plo.x + phi.x), pcy = 0.5f * (plo.y + phi.y), pcz = 0.5f * (plo.z + phi.z);
    const float cx = 0.5f * (clo.x + chi.x) - pcx, cy = 0.5f * (clo.y + chi.y) - pcy, cz = 0.5f * (clo.z + chi.z) - pcz;
    // greedy slot assignment over the pairs p0 = lane, p1 = lane + 32 (child p >> 3, slot p & 7)
    const int s_ = lane & 7, k0 = lane >> 3, k1 = 4 + (lane >> 3);
    float sc[2];
    {
        const float x0 = __shfl_sync(FULL, cx, k0), y0 = __shfl_sync(FULL, cy, k0), z0 = __shfl_sync(FULL, cz, k0);
        const float x1 = __shfl_sync(FULL, cx, k1), y1 = __shfl_sync(FULL, cy, k1), z1 = __shfl_sync(FULL, cz, k1);
        sc[0] = ((s_ & 1) ? x0 : -x0) + ((s_ & 2) ? y0 : -y0) + ((s_ & 4) ? z0 : -z0);
        sc[1] = ((s_ & 1) ? x1 : -x1) + ((s_ & 2) ? y1 : -y1) + ((s_ & 4) ? z1 : -z1);
    }
    uint32_t used_c = 0, used_s = 0;
    int slot_c = -1;   // lane s < 8: the child in slot s
    for (int it = 0; it < nc; it++) {
        const bool v0 = k0 < nc && !((used_c >> k0) & 1u) && !((used_s >> s_) & 1u);
        const bool v1 = k1 < nc && !((used_c >> k1) & 1u) && !((used_s >> s_) & 1u);
        const bool take1 = v1 && (!v0 || sc[1] > sc[0]);
        const bool has = v0 || v1;
        const unsigned key = has ? order_f(take1 ? sc[1] : sc[0]) : 0u;
        const uint32_t p = take1 ? (uint32_t)lane + 32u : (uint32_t)lane;
        const unsigned mx = __reduce_max_sync(FULL, key);
        const uint32_t pm = __reduce_min_sync(FULL, (has && key == mx) ? p : 0xFFFFFFFFu);
        const int bk = (int)(pm >> 3), bs = (int)(pm & 7u);
        used_c |= 1u << bk;
        used_s |= 1u << bs;
        const int cb = __shfl_sync(FULL, c, bk);
        if (lane == bs) slot_c = cb;
    }
    // classify and allocate
    const bool mine = lane < 8 && slot_c >= 0;
    const bool is_int = mine && slot_c < nl && leaf_count[slot_c] > leaf_pack;
    const uint32_t cnt = (mine && !is_int) ? leaf_count[slot_c] : 0u;
    const unsigned int_mask = __ballot_sync(FULL, is_int);
    const uint32_t n_int = (uint32_t)__popc(int_mask);
    uint32_t off = cnt;   // inclusive scan of the leaf counts over the slots, then exclusive
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
        const uint32_t t = __shfl_up_sync(FULL, off, o);
        if (lane >= o) off += t;
    }
    const uint32_t n_prims = __shfl_sync(FULL, off, 7);
    off -= cnt;
    uint32_t child_local = 0, prim_local = 0, task_base = 0;
    if (lane == 0) {
        child_local = n_int ? atomicAdd(&counters[2], n_int) : 0u;
        prim_local = n_prims ? atomicAdd(&counters[3], n_prims) : 0u;
    }
    child_local = __shfl_sync(FULL, child_local, 0);
    prim_local = __shfl_sync(FULL, prim_local, 0);
    // capacity checks (never exceeded by a correct tree; a violation is recorded,
    // the node is not written and no child task is queued)
    if (child_local + n_int > (uint32_t)n + 1u || prim_local + n_prims > (uint32_t)n || w - node_base > (uint32_t)n) {
        if (lane == 0) atomicOr(&counters[4], 1u);
        return;
    }
    if (lane == 0 && n_int) task_base = atomicAdd(next_tasks, n_int);
    task_base = __shfl_sync(FULL, task_base, 0);
    const QuantFrame F = quant_frame(plo, phi);
    if (lane == 0) {
        stage->px = plo.x; stage->py = plo.y; stage->pz = plo.z;
        stage->ex = (uint8_t)F.eb[0]; stage->ey = (uint8_t)F.eb[1]; stage->ez = (uint8_t)F.eb[2];
        stage->imask = (uint8_t)(int_mask & 0xFFu);
        stage->child_base = node_base + child_local;
        stage->prim_base = prim_base + prim_local;
    }
    if (lane < 8) {
        const int s = lane;
        if (slot_c < 0) {
            stage->meta[s] = 0;
            for (int a = 0; a < 3; a++) { stage->qlo[a][s] = 0; stage->qhi[a][s] = 0; }
        } else {
            quant_child(F, node_lo[slot_c], node_hi[slot_c], *stage, s);
            if (is_int) {
                const uint32_t rank = (uint32_t)__popc(int_mask & ((1u << s) - 1u));
                stage->meta[s] = (uint8_t)META_INTERNAL;
                const uint32_t slot_out = task_base + rank;
                if (slot_out < (uint32_t)n) tasks_out[slot_out] = make_uint2((uint32_t)slot_c, node_base + child_local + rank);
                else atomicOr(&counters[4], 2u);
            } else {
                stage->meta[s] = (uint8_t)((cnt << 5) | off);
                // the (<= leaf_pack) leaves of subtree slot_c, in order
                int stk[8];
                int sp = 0;
                stk[sp++] = slot_c;
                uint32_t k = 0;
                while (sp > 0) {
                    const int x = stk[--sp];
                    if (x >= nl) {
                        if (k < cnt) prim_order[prim_local + off + k] = sorted[x - nl];
                        k++;
                    } else if (sp < 7) {
                        const int2 ch = children[x];
                        stk[sp++] = ch.y;
                        stk[sp++] = ch.x;
                    } else {
                        atomicOr(&counters[4], 4u);
                    }
                }
            }
        }
    }
    __syncwarp();
    if (lane < 5) reinterpret_cast<uint4*>(nodes + w)[lane] = reinterpret_cast<const uint4*>(stage)[lane];
    __syncwarp();
}

__global__ void __launch_bounds__(SMALL_THREADS, 1)
k_build_small(const float4* __restrict__ plo, const float4* __restrict__ phi, int n, int passes, WideNode* nodes,
              uint32_t node_base, uint32_t prim_base, uint32_t* prim_order, SmallBuildOut* out, unsigned* err_word,
              float4* wide_box, uint32_t* wide_depth, uint32_t leaf_max, bool sah_collapse) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmallSmem& S = *reinterpret_cast<SmallSmem*>(smem_raw);
    const int tid = threadIdx.x, nt = blockDim.x;
    // 1. centroid bounds
    if (tid < 6) S.cb[tid] = tid < 3 ? 0xFFFFFFFFu : 0u;
    __syncthreads();
    {
        unsigned mn[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu}, mx[3] = {0u, 0u, 0u};
        if (tid < n) {
            const float4 a = plo[tid], b = phi[tid];
            const float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
            for (int k = 0; k < 3; k++) { mn[k] = enc_f(c[k]); mx[k] = mn[k]; }
        }
        for (int k = 0; k < 3; k++) {
            const unsigned a = __reduce_min_sync(0xFFFFFFFFu, mn[k]), b = __reduce_max_sync(0xFFFFFFFFu, mx[k]);
            if ((tid & 31) == 0) { atomicMin(&S.cb[k], a); atomicMax(&S.cb[3 + k], b); }
        }
    }
    __syncthreads();
    // 2. Morton codes, padded to a power of two with keys that sort last
    int n2 = 1;
    while (n2 < n) n2 <<= 1;
    for (int i = tid; i < n2; i += nt) {
        S.keys[i] = i < n ? morton_of(plo[i], phi[i], S.cb) : ~0ull;
        S.vals[i] = (uint32_t)i;
    }
    __syncthreads();
    // 3. bitonic sort by (code, index): the order of a stable radix sort
    for (int k = 2; k <= n2; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = tid; i < n2; i += nt) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const unsigned long long ka = S.keys[i], kb = S.keys[ixj];
                    const uint32_t va = S.vals[i], vb = S.vals[ixj];
                    const bool gt = ka > kb || (ka == kb && va > vb);
                    if (gt == ((i & k) == 0)) {
                        S.keys[i] = kb; S.keys[ixj] = ka;
                        S.vals[i] = vb; S.vals[ixj] = va;
                    }
                }
            }
            __syncthreads();
        }
    }
    // 4. leaves and the initial cluster list
    const int nl = n - 1;
    if (tid < n) {
        const uint32_t p = S.vals[tid];
        S.node_lo[nl + tid] = plo[p];
        S.node_hi[nl + tid] = phi[p];
        S.leaf_count[nl + tid] = 1;
        S.clusters[0][tid] = nl + tid;
    }
    if (tid == 0) { S.counters[5] = (uint32_t)n; S.counters[6] = 0u; }
    __syncthreads();
    // 5. clustering rounds (thread i owns cluster position i) while more than 32
    // clusters remain; the last 32 finish inside warp 0 (every cluster sees every
    // other one, rounds synchronise through shuffles instead of block barriers)
    int cur = 0, rounds = 0;
    uint32_t m = (uint32_t)n;
    uint32_t next_id = n > 1 ? (uint32_t)(n - 2) : 0u;
    while (m > 32 && rounds < SMALL_BUILD_MAX) {
        // nearest neighbour of every position within PLOC_RADIUS: a group of tpc
        // threads per position splits the 2 * PLOC_RADIUS candidates, then takes
        // the minimum of (area, position), so ties keep the lower position
        {
            int tpc = 2 * PLOC_RADIUS;
            while (tpc > 1 && (uint32_t)tpc * m > (uint32_t)SMALL_THREADS) tpc >>= 1;
            const int g = tid / tpc, sub = tid % tpc;
            float best = 3.4e38f;
            uint32_t nn = 0xFFFFFFFFu;
            if (g < (int)m) {
                const int cg = S.clusters[cur][g];
                const float4 glo = S.node_lo[cg], ghi = S.node_hi[cg];
                for (int u = sub; u < 2 * PLOC_RADIUS; u += tpc) {
                    const int j = g + (u < PLOC_RADIUS ? u - PLOC_RADIUS : u - PLOC_RADIUS + 1);
                    if (j < 0 || j >= (int)m) continue;
                    const int cj = S.clusters[cur][j];
                    const float a = half_area(f4min(glo, S.node_lo[cj]), f4max(ghi, S.node_hi[cj]));
                    if (a < best) { best = a; nn = (uint32_t)j; }   // increasing j within the thread
                }
            }
            for (int o = 1; o < tpc; o <<= 1) {
                const float ob = __shfl_xor_sync(0xFFFFFFFFu, best, o);
                const uint32_t on = __shfl_xor_sync(0xFFFFFFFFu, nn, o);
                if (ob < best || (ob == best && on < nn)) { best = ob; nn = on; }
            }
            if (sub == 0 && g < (int)m) S.tasks[0][g].x = nn;   // scratch: nearest neighbour per position
        }
        __syncthreads();
        const int i = tid;
        int nn = -1;
        float4 mylo = make_float4(0.f, 0.f, 0.f, 0.f), myhi = mylo;
        if (i < (int)m) {
            const int ci = S.clusters[cur][i];
            mylo = S.node_lo[ci];
            myhi = S.node_hi[ci];
            nn = (int)S.tasks[0][i].x;
        }
        bool merge = false, keep = false;
        if (i < (int)m) {
            const bool mutual = nn >= 0 && (int)S.tasks[0][nn].x == i;
            merge = mutual && i < nn;
            keep = !mutual || i < nn;
        }
        // one scan of both counts: kept clusters in the low half, merges in the high half
        uint32_t totals;
        const uint32_t v = (keep ? 1u : 0u) | (merge ? 0x10000u : 0u);
        const uint32_t incl = block_scan(v, S.warp_sums, &totals);
        const uint32_t kpos = (incl & 0xFFFFu) - (keep ? 1u : 0u), mrank = (incl >> 16) - (merge ? 1u : 0u);
        const uint32_t total_keep = totals & 0xFFFFu, total_merge = totals >> 16;
        if (keep) {
            int id = S.clusters[cur][i];
            if (merge) {
                const int cj = S.clusters[cur][nn];
                id = (int)(next_id - mrank);
                S.children[id] = make_int2(S.clusters[cur][i], cj);
                S.node_lo[id] = f4min(mylo, S.node_lo[cj]);
                S.node_hi[id] = f4max(myhi, S.node_hi[cj]);
                S.leaf_count[id] = S.leaf_count[S.clusters[cur][i]] + S.leaf_count[cj];
            }
            S.clusters[cur ^ 1][kpos] = id;
        }
        if (total_merge == 0 && tid == 0) S.counters[6] |= 16u;   // no progress (cannot happen)
        next_id -= total_merge;
        m = total_keep;
        cur ^= 1;
        rounds++;
        __syncthreads();
        if (total_merge == 0) break;
    }
    if (tid < 32 && m > 1 && m <= 32) {
        const int lane = tid;
        const bool live0 = lane < (int)m;
        int id = live0 ? S.clusters[cur][lane] : -1;
        float4 lo = live0 ? S.node_lo[id] : make_float4(0.f, 0.f, 0.f, 0.f);
        float4 hi = live0 ? S.node_hi[id] : lo;
        uint32_t cnt = live0 ? S.leaf_count[id] : 0u;
        for (int r = 0; m > 1 && r < 64; r++) {
            const bool live = lane < (int)m;
            float best = 3.4e38f;
            int nn = -1;
            // every live cluster's box is stored at its node id (merges write it before
            // the __syncwarp that ends a round)
            for (int j = 0; j < (int)m; j++) {
                const int idj = __shfl_sync(0xFFFFFFFFu, id, j);
                if (j == lane || !live) continue;
                const float a = half_area(f4min(lo, S.node_lo[idj]), f4max(hi, S.node_hi[idj]));
                if (a < best) { best = a; nn = j; }
            }
            const int nn_of_nn = __shfl_sync(0xFFFFFFFFu, nn, nn < 0 ? lane : nn);
            const bool mutual = live && nn >= 0 && nn_of_nn == lane;
            const bool merge = mutual && lane < nn;
            const bool keep = live && (!mutual || lane < nn);
            const unsigned mm = __ballot_sync(0xFFFFFFFFu, merge), km = __ballot_sync(0xFFFFFFFFu, keep);
            const unsigned below = (1u << lane) - 1u;
            // partner data (for the merging lane)
            const int pid = __shfl_sync(0xFFFFFFFFu, id, nn < 0 ? lane : nn);
            const float4 pl = make_float4(__shfl_sync(0xFFFFFFFFu, lo.x, nn < 0 ? lane : nn),
                                          __shfl_sync(0xFFFFFFFFu, lo.y, nn < 0 ? lane : nn),
                                          __shfl_sync(0xFFFFFFFFu, lo.z, nn < 0 ? lane : nn), 0.0f);
            const float4 ph = make_float4(__shfl_sync(0xFFFFFFFFu, hi.x, nn < 0 ? lane : nn),
                                          __shfl_sync(0xFFFFFFFFu, hi.y, nn < 0 ? lane : nn),
                                          __shfl_sync(0xFFFFFFFFu, hi.z, nn < 0 ? lane : nn), 0.0f);
            const uint32_t pc = __shfl_sync(0xFFFFFFFFu, cnt, nn < 0 ? lane : nn);
            if (merge) {
                const int nid = (int)(next_id - (uint32_t)__popc(mm & below));
                S.children[nid] = make_int2(id, pid);
                lo = f4min(lo, pl);
                hi = f4max(hi, ph);
                cnt += pc;
                S.node_lo[nid] = lo;
                S.node_hi[nid] = hi;
                S.leaf_count[nid] = cnt;
                id = nid;
            }
            if (mm == 0u) { if (lane == 0) S.counters[6] |= 16u; break; }
            next_id -= (uint32_t)__popc(mm);
            // compact: lane k takes the k-th kept cluster
            const int k = lane < __popc(km) ? (int)__fns(km, 0, lane + 1) : lane;
            id = __shfl_sync(0xFFFFFFFFu, id, k);
            lo = make_float4(__shfl_sync(0xFFFFFFFFu, lo.x, k), __shfl_sync(0xFFFFFFFFu, lo.y, k),
                             __shfl_sync(0xFFFFFFFFu, lo.z, k), 0.0f);
            hi = make_float4(__shfl_sync(0xFFFFFFFFu, hi.x, k), __shfl_sync(0xFFFFFFFFu, hi.y, k),
                             __shfl_sync(0xFFFFFFFFu, hi.z, k), 0.0f);
            cnt = __shfl_sync(0xFFFFFFFFu, cnt, k);
            m = (uint32_t)__popc(km);
            __syncwarp();
        }
        if (lane == 0) S.clusters[cur][0] = id;
        if (lane == 0 && m != 1u) S.counters[6] |= 16u;
        __syncwarp();
    }
    __syncthreads();
    if (tid == 0 && n > 1 && (next_id != 0xFFFFFFFFu || S.clusters[cur][0] != 0)) S.counters[6] |= 16u;
    __syncthreads();
    // 5b. optional treelet restructuring of the clustered tree (leaves dealt
    // round-robin over the 32 warps so that treelets that become ready together
    // run in different warps)
    if (passes > 0 && n >= TL_LEAVES + 1 && S.counters[6] == 0u) {
        if (tid == 0) S.parent[0] = -1;
        if (tid < n - 1) {
            const int2 ch = S.children[tid];
            S.parent[ch.x] = tid;
            S.parent[ch.y] = tid;
        }
        for (int pass = 0; pass < passes; pass++) {
            if (tid < n) S.flags[tid] = 0;
            __syncthreads();
            treelet_climb<false>((tid & 31) * 32 + (tid >> 5), n, S.children, S.parent, S.flags, S.node_lo,
                                 S.node_hi, S.leaf_count, S.cost, S.tl[tid >> 5], leaf_max);
            __syncthreads();
        }
    }
    // 5c. least-SAH choice of every wide node's children (bottom-up, in shared memory)
    const bool dp = sah_collapse && n > 1 && S.counters[6] == 0u;
    if (dp) {
        if (tid == 0) S.parent[0] = -1;
        if (tid < n - 1) {
            const int2 ch = S.children[tid];
            S.parent[ch.x] = tid;
            S.parent[ch.y] = tid;
        }
        if (tid < n) S.flags[tid] = 0;
        __syncthreads();
        if (tid < n)
            wide_cost_climb<false>(tid, n, S.children, S.parent, S.flags, S.node_lo, S.node_hi, S.leaf_count,
                                   S.dp.wide_cost, S.dp.wide_split, leaf_max, leaf_max);
        __syncthreads();
    }
    // 6. collapse, level by level
    const float4 rlo = S.node_lo[0], rhi = S.node_hi[0];
    float rha = half_area(rlo, rhi);
    if (!(rha > 0.0f)) rha = 1.0f;
    if (tid == 0) {
        S.tasks[0][0] = make_uint2(0u, node_base);
        S.counters[0] = 1u; S.counters[1] = 0u; S.counters[2] = 1u; S.counters[3] = 0u; S.counters[4] = 0u;
        S.sah = 0.0;
    }
    __syncthreads();
    int cc = 0, level = 0;
    for (; level < 4096; level++) {
        const uint32_t nin = min(S.counters[0], (uint32_t)n);   // the task arrays hold n entries
        if (nin == 0 || S.counters[4] != 0u) break;               // done, or a capacity error
        // one warp per wide node (no SAH statistic: the per-frame build skips it)
        for (uint32_t t = (uint32_t)(tid >> 5); t < nin; t += (uint32_t)(nt >> 5)) {
            const uint2 task = S.tasks[cc][t];
            // refit data: exact box and depth of every wide node
            const uint32_t local = task.y - node_base;
            if ((tid & 31) == 0 && local <= (uint32_t)n) {
                wide_box[2 * local] = S.node_lo[task.x];
                wide_box[2 * local + 1] = S.node_hi[task.x];
                wide_depth[local] = (uint32_t)level;
            }
            collapse_task_warp(task, S.counters, &S.counters[1], S.tasks[cc ^ 1], n, S.children, S.node_lo, S.node_hi,
                               S.leaf_count, S.vals, nodes, &S.stage[tid >> 5], node_base, prim_base, prim_order,
                               leaf_max, leaf_max, dp ? S.dp.wide_split : nullptr);
        }
        __syncthreads();
        if (tid == 0) { S.counters[0] = S.counters[1]; S.counters[1] = 0u; }
        cc ^= 1;
        __syncthreads();
    }
    if (tid == 0) {
        uint32_t e = S.counters[4] | S.counters[6];
        if (S.counters[3] != (uint32_t)n) e |= 4u;
        if (level >= 4096) e |= 8u;
        out->num_nodes = S.counters[2];
        out->prims = S.counters[3];
        out->error = e;
        out->max_depth = level > 0 ? (uint32_t)(level - 1) : 0u;
        out->sah = 0.0;
        out->lo[0] = rlo.x; out->lo[1] = rlo.y; out->lo[2] = rlo.z; out->lo[3] = 0.0f;
        out->hi[0] = rhi.x; out->hi[1] = rhi.y; out->hi[2] = rhi.z; out->hi[3] = 0.0f;
        if (e && err_word) atomicOr(err_word, 8u);
    }
}

// ---- collapse without host round trips (multi-launch builds of per-frame trees) ----------
// level_tasks[l] counts the tasks of wide level l (tasks of even levels in
// tasks_a, odd levels in tasks_b); counters: [2] wide nodes, [3] primitive
// slots, [4] capacity error bits.  A few launches of k_collapse_level take the
// usual depths with every SM; k_collapse_finish takes whatever is left in one
// block, so no level count has to come back to the host.
constexpr int COLLAPSE_MAX_LEVELS = 128;
constexpr int COLLAPSE_FAST_LEVELS = 8;
constexpr int LEVEL_WARPS = 8;

__global__ void k_collapse_init(uint2* tasks_a, uint32_t* counters, uint32_t* level_tasks, uint32_t node_base) {
    for (int l = threadIdx.x; l <= COLLAPSE_MAX_LEVELS; l += blockDim.x) level_tasks[l] = l == 0 ? 1u : 0u;
    if (threadIdx.x == 0) {
        tasks_a[0] = make_uint2(0u, node_base);
        counters[2] = 1u;
        counters[3] = 0u;
        counters[4] = 0u;
    }
}

// the depth of the wide node a task writes (for a later refit), by lane 0 of its warp
__device__ __forceinline__ void note_depth(uint32_t* wide_depth, uint2 task, uint32_t node_base, int n, int level) {
    const uint32_t local = task.y - node_base;
    if (wide_depth && (threadIdx.x & 31) == 0 && local <= (uint32_t)n) wide_depth[local] = (uint32_t)level;
}

__global__ void __launch_bounds__(32 * LEVEL_WARPS) k_collapse_level(
    int level, uint2* tasks_a, uint2* tasks_b, uint32_t* level_tasks, uint32_t* counters, int n, const int2* children,
    const float4* node_lo, const float4* node_hi, const uint32_t* leaf_count, const uint32_t* sorted, WideNode* nodes,
    uint32_t node_base, uint32_t prim_base, uint32_t* prim_order, uint32_t leaf_max, uint32_t leaf_pack,
    uint32_t* wide_depth, const uint32_t* wide_split) {
    __shared__ WideNode stage[LEVEL_WARPS];
    const uint32_t nin = min(level_tasks[level], (uint32_t)n);   // the task arrays hold n entries
    if (nin == 0 || counters[4] != 0u) return;
    const uint2* tin = (level & 1) ? tasks_b : tasks_a;
    uint2* tout = (level & 1) ? tasks_a : tasks_b;
    const uint32_t w = threadIdx.x >> 5;
    for (uint32_t t = blockIdx.x * LEVEL_WARPS + w; t < nin; t += gridDim.x * LEVEL_WARPS) {
        const uint2 task = tin[t];
        note_depth(wide_depth, task, node_base, n, level);
        collapse_task_warp(task, counters, &level_tasks[level + 1], tout, n, children, node_lo, node_hi, leaf_count,
                           sorted, nodes, &stage[w], node_base, prim_base, prim_order, leaf_max, leaf_pack,
                           wide_split);
    }
}

__global__ void __launch_bounds__(1024) k_collapse_finish(
    int first_level, uint2* tasks_a, uint2* tasks_b, uint32_t* level_tasks, uint32_t* counters, int n,
    const int2* children, const float4* node_lo, const float4* node_hi, const uint32_t* leaf_count,
    const uint32_t* sorted, WideNode* nodes, uint32_t node_base, uint32_t prim_base, uint32_t* prim_order,
    uint32_t leaf_max, uint32_t leaf_pack, unsigned* err_word, uint32_t* wide_depth, SmallBuildOut* out,
    const uint32_t* wide_split) {
    __shared__ WideNode stage[32];
    const uint32_t w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int level = first_level;
    for (; level < COLLAPSE_MAX_LEVELS; level++) {
        const uint32_t nin = min(level_tasks[level], (uint32_t)n);
        if (nin == 0 || counters[4] != 0u) break;
        const uint2* tin = (level & 1) ? tasks_b : tasks_a;
        uint2* tout = (level & 1) ? tasks_a : tasks_b;
        for (uint32_t t = w; t < nin; t += nw) {
            const uint2 task = tin[t];
            note_depth(wide_depth, task, node_base, n, level);
            collapse_task_warp(task, counters, &level_tasks[level + 1], tout, n, children, node_lo, node_hi,
                               leaf_count, sorted, nodes, &stage[w], node_base, prim_base, prim_order, leaf_max,
                               leaf_pack, wide_split);
        }
        __syncthreads();   // this level's child tasks and their count are complete
    }
    if (threadIdx.x == 0) {
        const bool unfinished = level >= COLLAPSE_MAX_LEVELS && level_tasks[COLLAPSE_MAX_LEVELS] != 0u;
        const bool bad = counters[4] != 0u || unfinished || counters[3] != (uint32_t)n;
        if (bad && err_word) atomicOr(err_word, 8u);
        if (out) {   // the record a refit reads: node count and deepest level
            uint32_t deepest = 0;
            for (int l = 0; l < COLLAPSE_MAX_LEVELS; l++)
                if (level_tasks[l] != 0u) deepest = (uint32_t)l;
            out->num_nodes = counters[2];
            out->prims = counters[3];
            out->error = bad ? 8u : 0u;
            out->max_depth = deepest;
            out->sah = 0.0;
        }
    }
}

// Refit of a per-frame wide BVH (made by k_build_small or by the device-driven
// multi-launch build) for moved primitives: the topology (child and primitive
// slots) stays, every node's exact box and quantised child planes are
// recomputed, deepest level first (one block, a barrier per level; the tree of
// n primitives has at most n + 1 nodes, each visited once per refit).
__global__ void __launch_bounds__(SMALL_THREADS, 1)
k_refit_small(WideNode* nodes, uint32_t node_base, uint32_t prim_base, const SmallBuildOut* info,
              float4* wide_box, const uint32_t* wide_depth, const uint32_t* prim_order,
              const float4* __restrict__ plo, const float4* __restrict__ phi, int n, unsigned* err_word) {
    const uint32_t nn = info->num_nodes;
    if (info->error || nn == 0 || nn > (uint32_t)n + 1u) return;
    const int max_depth = (int)min(info->max_depth, 4095u);
    for (int level = max_depth; level >= 0; level--) {
        for (uint32_t k = threadIdx.x; k < nn; k += blockDim.x) {
            if (wide_depth[k] != (uint32_t)level) continue;
            WideNode node;
            const uint4* src = reinterpret_cast<const uint4*>(nodes + node_base + k);
            uint4* dst4 = reinterpret_cast<uint4*>(&node);
            for (int q = 0; q < 5; q++) dst4[q] = src[q];
            float4 clo[8], chi[8];
            float4 lo = make_float4(3.4e38f, 3.4e38f, 3.4e38f, 0.0f), hi = make_float4(-3.4e38f, -3.4e38f, -3.4e38f, 0.0f);
            bool bad = false;
            for (int s = 0; s < 8; s++) {
                const uint32_t meta = node.meta[s];
                clo[s] = make_float4(3.4e38f, 3.4e38f, 3.4e38f, 0.0f);
                chi[s] = make_float4(-3.4e38f, -3.4e38f, -3.4e38f, 0.0f);
                if (meta == 0u) continue;
                if (meta == META_INTERNAL) {
                    const uint32_t child = node.child_base + (uint32_t)__popc(node.imask & ((1u << s) - 1u)) - node_base;
                    if (child >= nn) { bad = true; continue; }
                    clo[s] = wide_box[2 * child];
                    chi[s] = wide_box[2 * child + 1];
                } else {
                    const uint32_t cnt = meta >> 5, off = meta & 31u;
                    for (uint32_t j = 0; j < cnt; j++) {
                        const uint32_t slot = node.prim_base + off + j - prim_base;
                        if (slot >= (uint32_t)n) { bad = true; continue; }
                        const uint32_t li = prim_order[slot];
                        if (li >= (uint32_t)n) { bad = true; continue; }
                        clo[s] = f4min(clo[s], plo[li]);
                        chi[s] = f4max(chi[s], phi[li]);
                    }
                }
                lo = f4min(lo, clo[s]);
                hi = f4max(hi, chi[s]);
            }
            if (bad) { atomicOr(err_word, 8u); continue; }
            const QuantFrame F = quant_frame(lo, hi);
            node.px = lo.x; node.py = lo.y; node.pz = lo.z;
            node.ex = (uint8_t)F.eb[0]; node.ey = (uint8_t)F.eb[1]; node.ez = (uint8_t)F.eb[2];
            for (int s = 0; s < 8; s++) {
                if (node.meta[s] == 0u) continue;
                quant_child(F, clo[s], chi[s], node, s);
            }
            uint4* out4 = reinterpret_cast<uint4*>(nodes + node_base + k);
            for (int q = 0; q < 5; q++) out4[q] = dst4[q];
            wide_box[2 * k] = lo;
            wide_box[2 * k + 1] = hi;
        }
        __syncthreads();
    }
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

namespace {
// sorts (sc.keys, sc.vals) by key, stably (sc.keys_alt / sc.vals_alt: scratch)
Status sort_pairs(BuildScratch& sc, uint32_t n, cudaStream_t st) {
    if (n <= SORT_BITONIC_MAX) {
        uint32_t N = 2;
        while (N < n) N <<= 1;
        const int bytes = (int)(N * (sizeof(unsigned long long) + sizeof(uint32_t)));
        SNK_TRY_CUDA(cudaFuncSetAttribute(k_sort_bitonic, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        k_sort_bitonic<<<1, SORT_THREADS, bytes, st>>>(sc.keys.p, sc.vals.p, n);
        SNK_TRY_CUDA(cudaGetLastError());
        return Status::Ok();
    }
    if (n <= SORT_SMALL_MAX) {
        k_sort_small<<<1, SORT_THREADS, 0, st>>>(sc.keys.p, sc.vals.p, sc.keys_alt.p, sc.vals_alt.p, n);
        SNK_TRY_CUDA(cudaGetLastError());
        return Status::Ok();
    }
    const uint32_t tiles = (n + SORT_TILE - 1) / SORT_TILE;
    SNK_TRY_CUDA(sc.sort_hist.reserve((size_t)SORT_RADIX * tiles));
    unsigned long long *sk = sc.keys.p, *dk = sc.keys_alt.p;
    uint32_t *sv = sc.vals.p, *dv = sc.vals_alt.p;
    for (int pass = 0; pass < SORT_PASSES; pass++) {   // an even number: the result ends in sc.keys / sc.vals
        const int shift = 8 * pass;
        k_sort_hist<<<tiles, SORT_THREADS, 0, st>>>(sk, n, shift, sc.sort_hist.p, tiles);
        k_sort_scan<<<1, SORT_THREADS, 0, st>>>(sc.sort_hist.p, (uint32_t)SORT_RADIX * tiles);
        k_sort_scatter<<<tiles, SORT_THREADS, 0, st>>>(sk, sv, n, shift, sc.sort_hist.p, tiles, dk, dv);
        SNK_TRY_CUDA(cudaGetLastError());
        std::swap(sk, dk);
        std::swap(sv, dv);
    }
    static_assert(SORT_PASSES % 2 == 0, "the multi-CTA sort ends in the first buffer pair");
    return Status::Ok();
}

// the binary tree of build_wide_bvh and build_wide_bvh_device (Morton codes, radix
// sort, Karras hierarchy, bottom-up boxes, treelet passes); *sorted_out receives
// the primitive of each sorted position
Status build_binary_tree(BuildScratch& sc, const float4* prim_lo, const float4* prim_hi, uint32_t n, cudaStream_t st,
                         int treelet_passes, uint32_t leaf_max, uint32_t leaf_pack, const uint32_t** sorted_out) {
    if (leaf_max < 1 || leaf_max > LEAF_MAX_LIMIT || leaf_pack < leaf_max || leaf_pack > LEAF_MAX_LIMIT)
        return Status::Err(1, "build_wide_bvh: leaf size out of range");
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
    SNK_TRY_CUDA(sc.cost.reserve(2 * (size_t)n));
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

    SNK_TRY(sort_pairs(sc, n, st));
    const unsigned long long* keys = sc.keys.p;
    const uint32_t* sorted = sc.vals.p;
    *sorted_out = sorted;

    SNK_TRY_CUDA(cudaMemsetAsync(sc.flags.p, 0, sizeof(int) * n, st));
    int minus1 = -1;
    SNK_TRY_CUDA(cudaMemcpyAsync(sc.parent.p, &minus1, sizeof(int), cudaMemcpyHostToDevice, st));
    if (n > 1) k_karras<<<grid_for(n - 1), BLK, 0, st>>>(keys, (int)n, sc.children.p, sc.parent.p);
    k_bottom_up<<<g, BLK, 0, st>>>(sorted, prim_lo, prim_hi, (int)n, sc.children.p, sc.parent.p, sc.flags.p,
                                   sc.node_lo.p, sc.node_hi.p, sc.leaf_count.p);
    SNK_TRY_CUDA(cudaGetLastError());
    if (n >= (uint32_t)TL_LEAVES + 1) {
        for (int pass = 0; pass < treelet_passes; pass++) {
            SNK_TRY_CUDA(cudaMemsetAsync(sc.flags.p, 0, sizeof(int) * n, st));
            k_treelet_pass<<<g, BLK, 0, st>>>((int)n, sc.children.p, sc.parent.p, sc.flags.p, sc.node_lo.p,
                                              sc.node_hi.p, sc.leaf_count.p, sc.cost.p, leaf_max);
            SNK_TRY_CUDA(cudaGetLastError());
        }
    }
    return Status::Ok();
}
}  // namespace

Status build_wide_bvh(BuildScratch& sc, const float4* prim_lo, const float4* prim_hi, uint32_t n, WideNode* nodes,
                      uint32_t node_base, uint32_t prim_base, uint32_t* prim_order, cudaStream_t st,
                      BuildResult* out, int treelet_passes, uint32_t leaf_max, uint32_t leaf_pack,
                      bool sah_collapse) {
    const uint32_t* sorted = nullptr;
    SNK_TRY(build_binary_tree(sc, prim_lo, prim_hi, n, st, treelet_passes, leaf_max, leaf_pack, &sorted));
    // SAH-optimal choice of each wide node's children (bottom-up over the final binary tree)
    const uint32_t* wide_split = nullptr;
    if (n > 1 && sah_collapse) {
        SNK_TRY_CUDA(sc.wide_cost.reserve(8 * (size_t)(n - 1)));
        SNK_TRY_CUDA(sc.wide_split.reserve(n - 1));
        SNK_TRY_CUDA(cudaMemsetAsync(sc.flags.p, 0, sizeof(int) * n, st));
        k_collapse_cost<<<grid_for(n), BLK, 0, st>>>((int)n, sc.children.p, sc.parent.p, sc.flags.p, sc.node_lo.p,
                                                     sc.node_hi.p, sc.leaf_count.p, sc.wide_cost.p, sc.wide_split.p,
                                                     leaf_max, leaf_pack);
        SNK_TRY_CUDA(cudaGetLastError());
        wide_split = sc.wide_split.p;
    }
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
                                                     prim_base, prim_order, sc.sah.p, rha, leaf_max, leaf_pack,
                                                     wide_split);
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

Status build_wide_bvh_device(BuildScratch& sc, const float4* prim_lo, const float4* prim_hi, uint32_t n,
                             WideNode* nodes, uint32_t node_base, uint32_t prim_base, uint32_t* prim_order,
                             unsigned* err_word, cudaStream_t st, int treelet_passes, uint32_t leaf_max,
                             uint32_t leaf_pack, SmallBuildOut* out, uint32_t* wide_depth, bool sah_collapse) {
    const uint32_t* sorted = nullptr;
    SNK_TRY(build_binary_tree(sc, prim_lo, prim_hi, n, st, treelet_passes, leaf_max, leaf_pack, &sorted));
    const uint32_t* wide_split = nullptr;
    if (n > 1 && sah_collapse) {
        SNK_TRY_CUDA(sc.wide_cost.reserve(8 * (size_t)(n - 1)));
        SNK_TRY_CUDA(sc.wide_split.reserve(n - 1));
        SNK_TRY_CUDA(cudaMemsetAsync(sc.flags.p, 0, sizeof(int) * n, st));
        k_collapse_cost<<<grid_for(n), BLK, 0, st>>>((int)n, sc.children.p, sc.parent.p, sc.flags.p, sc.node_lo.p,
                                                     sc.node_hi.p, sc.leaf_count.p, sc.wide_cost.p, sc.wide_split.p,
                                                     leaf_max, leaf_pack);
        SNK_TRY_CUDA(cudaGetLastError());
        wide_split = sc.wide_split.p;
    }
    SNK_TRY_CUDA(sc.level_tasks.reserve(COLLAPSE_MAX_LEVELS + 1));
    k_collapse_init<<<1, 128, 0, st>>>(sc.tasks_a.p, sc.counters.p, sc.level_tasks.p, node_base);
    // enough warps for the widest level of a typical tree, at most 1024 blocks
    uint32_t grid = (n + 8u * LEVEL_WARPS - 1u) / (8u * LEVEL_WARPS);
    grid = grid < 1u ? 1u : (grid > 1024u ? 1024u : grid);
    // multi-block launches for about the depth of a balanced 8-wide tree; deeper
    // levels (unbalanced trees) go to the single-block finish
    int fast = 1;
    for (uint64_t cap = 8; cap < n && fast < COLLAPSE_FAST_LEVELS; cap *= 8) fast++;
    fast = fast + 1 < COLLAPSE_FAST_LEVELS ? fast + 1 : COLLAPSE_FAST_LEVELS;
    for (int level = 0; level < fast; level++)
        k_collapse_level<<<grid, 32 * LEVEL_WARPS, 0, st>>>(level, sc.tasks_a.p, sc.tasks_b.p, sc.level_tasks.p,
                                                            sc.counters.p, (int)n, sc.children.p, sc.node_lo.p,
                                                            sc.node_hi.p, sc.leaf_count.p, sorted, nodes, node_base,
                                                            prim_base, prim_order, leaf_max, leaf_pack, wide_depth,
                                                            wide_split);
    k_collapse_finish<<<1, 1024, 0, st>>>(fast, sc.tasks_a.p, sc.tasks_b.p, sc.level_tasks.p,
                                          sc.counters.p, (int)n, sc.children.p, sc.node_lo.p, sc.node_hi.p,
                                          sc.leaf_count.p, sorted, nodes, node_base, prim_base, prim_order, leaf_max,
                                          leaf_pack, err_word, wide_depth, out, wide_split);
    SNK_TRY_CUDA(cudaGetLastError());
    return Status::Ok();
}

Status build_wide_bvh_small(const float4* prim_lo, const float4* prim_hi, uint32_t n, WideNode* nodes,
                            uint32_t node_base, uint32_t prim_base, uint32_t* prim_order, int treelet_passes,
                            SmallBuildOut* out, unsigned* err_word, float4* wide_box, uint32_t* wide_depth,
                            cudaStream_t st, uint32_t leaf_max, bool sah_collapse) {
    if (n == 0 || n > (uint32_t)SMALL_BUILD_MAX) return Status::Err(1, "build_wide_bvh_small: bad primitive count");
    if (leaf_max < 1 || leaf_max > LEAF_MAX_LIMIT) return Status::Err(1, "build_wide_bvh_small: leaf size out of range");
    SNK_TRY_CUDA(cudaFuncSetAttribute(k_build_small, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sizeof(SmallSmem)));
    k_build_small<<<1, SMALL_THREADS, sizeof(SmallSmem), st>>>(prim_lo, prim_hi, (int)n, treelet_passes, nodes,
                                                                node_base, prim_base, prim_order, out, err_word,
                                                                wide_box, wide_depth, leaf_max, sah_collapse);
    SNK_TRY_CUDA(cudaGetLastError());
    return Status::Ok();
}

Status refit_wide_bvh(const float4* prim_lo, const float4* prim_hi, uint32_t n, WideNode* nodes, uint32_t node_base,
                      uint32_t prim_base, const uint32_t* prim_order, const SmallBuildOut* info, float4* wide_box,
                      const uint32_t* wide_depth, unsigned* err_word, cudaStream_t st) {
    if (n == 0 || n > (1u << 30)) return Status::Err(1, "refit_wide_bvh: bad primitive count");
    k_refit_small<<<1, SMALL_THREADS, 0, st>>>(nodes, node_base, prim_base, info, wide_box, wide_depth, prim_order,
                                               prim_lo, prim_hi, (int)n, err_word);
    SNK_TRY_CUDA(cudaGetLastError());
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
