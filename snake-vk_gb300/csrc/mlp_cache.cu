// mlp_cache.cu -- the online-trained MLP radiance cache: input encoding, fused
// inference, fused forward+backward training and the Adam update, on BF16
// tensor cores (mma.sync m16n8k16, FP32 accumulation).  There is no
// counterpart in the reference; this is the learned part of the path tracer
// (cache queries replace path tails, radiance-caching style, Mueller et al. 2021).
//
// Network: 64 encoded inputs -> 4 x (64, ReLU) -> 3 linear outputs, no biases
// (the encoding carries a constant 1).  FP32 master weights W_l[in][out]
// (4 x 64x64 then 64x3 = 16576 values) with Adam moments; the tensor cores read
// BF16 copies stored in MMA-fragment order, so a lane loads its B fragment with
// one 8-byte shared-memory load:
//   forward block (layer l, k-tile kt, n-tile nt), lane (g = lane/4, t = lane%4):
//     b0 = (W[16kt+2t][8nt+g], W[16kt+2t+1][8nt+g]), b1 = same at rows +8
//   transposed block (for dX = dY W^T) is the same with W replaced by W^T.
// Activations stay in registers between layers: the D fragment of one layer is
// the A fragment of the next.  Training keeps the post-ReLU activations and the
// back-propagated gradients transposed ([feature][sample]) in shared memory, so
// dW = act^T g runs as a CTA-wide GEMM with 4-byte operand loads.  Each CTA
// writes its dW partial; the Adam kernel sums the partials in a fixed order, so
// training is deterministic.
//
// Inference runs on the fifth-generation tensor cores: one CTA of 128 threads
// takes 128 queries, writes their encodings into shared memory in the tcgen05
// operand layout, and chains the 5 layers as 128x64x64 (last 128x16x64)
// tcgen05.mma issued by one thread, accumulating in tensor memory; after each
// layer every thread reads its row back with tcgen05.ld, applies the ReLU and
// stores the BF16 row as the next layer's operand.  Waits on the MMA completion
// barrier are bounded (a give-up sets a status bit, read by the host).
//
// Input encoding (64 features, from a 64-byte query record: position, outgoing
// direction, shading normal, roughness, albedo, metallic):
//   0..35   position normalised to the scene box, per axis 6 octaves of
//           sin/cos(2^k pi p) (12 features per axis)
//   36..41  sin/cos(pi d) per axis      42..47  sin/cos(pi n) per axis
//   48..50  d     51..53 n     54 roughness     55..57 albedo     58 metallic
//   59      n.d   60..62 f0 = mix(0.04, albedo, metallic)         63 1.0
#include <cuda_bf16.h>

#include "snk_mlp.h"

namespace snk {
namespace {

constexpr int ROW_PAD = 72;     // bf16 row stride of a [16][64] tile (conflict-free 4-byte loads)
constexpr int TS = 136;         // sample stride of transposed [64][128] tiles
constexpr int TRAIN_ROWS = 128; // samples per training CTA (8 warps x 16)

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float bf16_bits_to_float(unsigned short b) { return __uint_as_float((uint32_t)b << 16); }
__device__ __forceinline__ unsigned short float_to_bf16_bits(float f) {
    __nv_bfloat16 h = __float2bfloat16_rn(f);
    return *reinterpret_cast<unsigned short*>(&h);
}

__device__ __forceinline__ void mma16816(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Features [32*half, 32*half + 32) of one query record.
__device__ __forceinline__ void encode_half(const float4 q0, const float4 q1, const float4 q2, const float4 q3,
                                            const EncodeParams& ep, int half, float* f) {
    float p[3] = {(q0.x - ep.lo[0]) * ep.inv_ext[0], (q0.y - ep.lo[1]) * ep.inv_ext[1],
                  (q0.z - ep.lo[2]) * ep.inv_ext[2]};
    float oct[3][12];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float pa = fminf(fmaxf(p[a], 0.0f), 1.0f);
        float s = __sinf(3.14159265f * pa), c = __cosf(3.14159265f * pa);
#pragma unroll
        for (int k = 0; k < 6; k++) {
            oct[a][2 * k] = s;
            oct[a][2 * k + 1] = c;
            float s2 = 2.0f * s * c, c2 = (c - s) * (c + s);
            s = s2;
            c = c2;
        }
    }
    if (half == 0) {
#pragma unroll
        for (int j = 0; j < 12; j++) { f[j] = oct[0][j]; f[12 + j] = oct[1][j]; }
#pragma unroll
        for (int j = 0; j < 8; j++) f[24 + j] = oct[2][j];
    } else {
#pragma unroll
        for (int j = 0; j < 4; j++) f[j] = oct[2][8 + j];
        const float d[3] = {q1.x, q1.y, q1.z}, n[3] = {q2.x, q2.y, q2.z};
#pragma unroll
        for (int a = 0; a < 3; a++) {
            f[4 + 2 * a] = __sinf(3.14159265f * d[a]);
            f[5 + 2 * a] = __cosf(3.14159265f * d[a]);
            f[10 + 2 * a] = __sinf(3.14159265f * n[a]);
            f[11 + 2 * a] = __cosf(3.14159265f * n[a]);
            f[16 + a] = d[a];
            f[19 + a] = n[a];
        }
        f[22] = q0.w;
        f[23] = q3.x; f[24] = q3.y; f[25] = q3.z;
        f[26] = q1.w;
        f[27] = d[0] * n[0] + d[1] * n[1] + d[2] * n[2];
        float om = 1.0f - q1.w;
        f[28] = 0.04f * om + q3.x * q1.w;
        f[29] = 0.04f * om + q3.y * q1.w;
        f[30] = 0.04f * om + q3.z * q1.w;
        f[31] = 1.0f;
    }
}

// ---- weights to shared memory -------------------------------------------------
__device__ __forceinline__ void load_words(uint2* dst, const uint2* __restrict__ src, int n) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

// forward pass of one warp's 16-row tile whose A fragments are in a[4][4];
// returns the output fragment c5 (row g: cols 2t,2t+1; row g+8: cols 2t,2t+1)
template <bool STORE_ACT>
__device__ __forceinline__ void forward_tile(const uint2* wf, uint32_t (&a)[4][4], float (&c5)[4],
                                             unsigned short* actT, int row0) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int l = 0; l < 4; l++) {
        float c[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; nt++) c[nt][0] = c[nt][1] = c[nt][2] = c[nt][3] = 0.0f;
#pragma unroll
        for (int kt = 0; kt < 4; kt++)
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                uint2 b = wf[MLP_FWD_OFF(l) + (kt * 8 + nt) * 32 + lane];
                mma16816(c[nt], a[kt], b.x, b.y);
            }
#pragma unroll
        for (int nt = 0; nt < 8; nt++)
#pragma unroll
            for (int r = 0; r < 4; r++) c[nt][r] = fmaxf(c[nt][r], 0.0f);
        if (STORE_ACT) {
            unsigned short* A = actT + l * 64 * TS;
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                int f = 8 * nt + 2 * t;
                A[f * TS + row0 + g] = float_to_bf16_bits(c[nt][0]);
                A[(f + 1) * TS + row0 + g] = float_to_bf16_bits(c[nt][1]);
                A[f * TS + row0 + g + 8] = float_to_bf16_bits(c[nt][2]);
                A[(f + 1) * TS + row0 + g + 8] = float_to_bf16_bits(c[nt][3]);
            }
        }
#pragma unroll
        for (int kt = 0; kt < 4; kt++) {
            a[kt][0] = pack_bf16(c[2 * kt][0], c[2 * kt][1]);
            a[kt][1] = pack_bf16(c[2 * kt][2], c[2 * kt][3]);
            a[kt][2] = pack_bf16(c[2 * kt + 1][0], c[2 * kt + 1][1]);
            a[kt][3] = pack_bf16(c[2 * kt + 1][2], c[2 * kt + 1][3]);
        }
    }
    c5[0] = c5[1] = c5[2] = c5[3] = 0.0f;
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
        uint2 b = wf[MLP_FWD_OFF(4) + kt * 32 + lane];
        mma16816(c5, a[kt], b.x, b.y);
    }
}

// ---- tcgen05 helpers ---------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (row r, k) of an N x 64 K-major operand (no swizzle)
__host__ __device__ __forceinline__ uint32_t tc_off(uint32_t r, uint32_t k) {
    return (r >> 3) * 1024u + (k >> 3) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// shared-memory matrix descriptor: start address, leading (K) and stride (M/N)
// byte offsets between core matrices, fixed version bits 0b001, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr) {
    uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)(128u >> 4) << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// instruction descriptor: D FP32, A and B BF16, both K-major, M = 128
__device__ __forceinline__ uint32_t tc_idesc(uint32_t n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}

// D[tmem] (+)= A[128 x 64] B^T (B: n x 64), four K = 16 steps, then a commit to mbar
__device__ __forceinline__ void tc_gemm_k64(uint32_t tmem, uint32_t a_addr, uint32_t b_addr, uint32_t n,
                                            uint32_t mbar) {
    const uint32_t idesc = tc_idesc(n);
#pragma unroll
    for (uint32_t ks = 0; ks < 4; ks++) {
        const uint64_t da = tc_desc(a_addr + ks * 256u), db = tc_desc(b_addr + ks * 256u);
        const uint32_t acc = ks > 0 ? 1u : 0u;
        asm volatile("{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                     " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                     :: "r"(tmem), "l"(da), "l"(db), "r"(idesc), "r"(acc));
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(mbar));
}

// bounded wait for the barrier phase `parity`; false when it gave up
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    for (int it = 0; it < (1 << 24); it++) {
        uint32_t done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     " selp.u32 %0, 1, 0, p;\n}" : "=r"(done) : "r"(mbar), "r"(parity));
        if (done) return true;
    }
    return false;
}

#define SNK_TC_LD16(base, r, o)                                                                        \
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "                                             \
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"                   \
                 : "=r"(r[o + 0]), "=r"(r[o + 1]), "=r"(r[o + 2]), "=r"(r[o + 3]), "=r"(r[o + 4]),   \
                   "=r"(r[o + 5]), "=r"(r[o + 6]), "=r"(r[o + 7]), "=r"(r[o + 8]), "=r"(r[o + 9]),   \
                   "=r"(r[o + 10]), "=r"(r[o + 11]), "=r"(r[o + 12]), "=r"(r[o + 13]),              \
                   "=r"(r[o + 14]), "=r"(r[o + 15])                                                  \
                 : "r"(base))

constexpr int INFER_THREADS = 128;

struct InferSmem {
    unsigned short w[MLP_TC_ELEMS];   // the 5 layers, tcgen05 operand layout
    unsigned short a[128 * 64];       // this tile's activations (A operand)
    unsigned long long mbar;
    uint32_t tmem;
    uint32_t failed;
};

// ---- inference -------------------------------------------------------------------
// records: 4 float4 per query.  Result y (3 floats) goes to out[3i..] when out is
// given; otherwise, in render mode, L[path] += beta * max(y, 0) (one query per path).
__global__ void __launch_bounds__(INFER_THREADS) k_mlp_infer_tc(const unsigned short* __restrict__ wtc_g,
                                                                const float4* __restrict__ rec,
                                                                const uint32_t* __restrict__ n_ptr, uint32_t n_const,
                                                                EncodeParams ep, float* out,
                                                                const float4* __restrict__ beta, float4* L,
                                                                unsigned* status) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    InferSmem& S = *reinterpret_cast<InferSmem*>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5;
    {
        const uint4* src = reinterpret_cast<const uint4*>(wtc_g);
        uint4* dst = reinterpret_cast<uint4*>(S.w);
        for (int i = tid; i < MLP_TC_ELEMS / 8; i += INFER_THREADS) dst[i] = src[i];
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&S.mbar)));
        S.failed = 0u;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" :: "r"(smem_u32(&S.tmem)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = S.tmem, mbar = smem_u32(&S.mbar), a_addr = smem_u32(S.a), w_addr = smem_u32(S.w);
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);   // this warp's 32 lanes (rows)
    const uint32_t n = n_ptr ? *n_ptr : n_const;
    uint32_t parity = 0;
    unsigned char* arow = reinterpret_cast<unsigned char*>(S.a);
    for (uint32_t tile = blockIdx.x; tile * 128u < n; tile += gridDim.x) {
        const uint32_t i = tile * 128u + (uint32_t)tid;
        {   // encode this thread's query into its row of the A operand
            float f[64];
            if (i < n) {
                const float4* r = rec + 4ull * i;
                const float4 q0 = r[0], q1 = r[1], q2 = r[2], q3 = r[3];
                encode_half(q0, q1, q2, q3, ep, 0, f);
                encode_half(q0, q1, q2, q3, ep, 1, f + 32);
            } else {
#pragma unroll
                for (int j = 0; j < 64; j++) f[j] = 0.0f;
            }
#pragma unroll
            for (int kb = 0; kb < 8; kb++) {
                uint4 v = make_uint4(pack_bf16(f[8 * kb], f[8 * kb + 1]), pack_bf16(f[8 * kb + 2], f[8 * kb + 3]),
                                     pack_bf16(f[8 * kb + 4], f[8 * kb + 5]), pack_bf16(f[8 * kb + 6], f[8 * kb + 7]));
                *reinterpret_cast<uint4*>(arow + tc_off((uint32_t)tid, 8u * kb)) = v;
            }
        }
        float y[3] = {0.0f, 0.0f, 0.0f};
        bool ok = true;
#pragma unroll 1
        for (int l = 0; l < 5 && ok; l++) {
            asm volatile("fence.proxy.async.shared::cta;");
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncthreads();
            if (tid == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;");
                tc_gemm_k64(tmem, a_addr, w_addr + (uint32_t)l * 8192u, l < 4 ? 64u : 16u, mbar);
                if (!mbar_wait(mbar, parity)) S.failed = 1u;
            }
            parity ^= 1u;
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;");
            ok = S.failed == 0u;
            if (!ok) break;
            if (l < 4) {
                uint32_t r[64];
                SNK_TC_LD16(taddr + 0u, r, 0);
                SNK_TC_LD16(taddr + 16u, r, 16);
                SNK_TC_LD16(taddr + 32u, r, 32);
                SNK_TC_LD16(taddr + 48u, r, 48);
                asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
                for (int kb = 0; kb < 8; kb++) {
                    float v[8];
#pragma unroll
                    for (int j = 0; j < 8; j++) v[j] = fmaxf(__uint_as_float(r[8 * kb + j]), 0.0f);
                    uint4 pk = make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]),
                                          pack_bf16(v[6], v[7]));
                    *reinterpret_cast<uint4*>(arow + tc_off((uint32_t)tid, 8u * kb)) = pk;
                }
            } else {
                uint32_t r[16];
                SNK_TC_LD16(taddr, r, 0);
                asm volatile("tcgen05.wait::ld.sync.aligned;");
                y[0] = __uint_as_float(r[0]); y[1] = __uint_as_float(r[1]); y[2] = __uint_as_float(r[2]);
            }
        }
        if (!ok) break;
        if (i < n) {
            if (out) {
                out[3ull * i] = y[0]; out[3ull * i + 1] = y[1]; out[3ull * i + 2] = y[2];
            } else {
                const uint32_t p = __float_as_uint(rec[4ull * i + 3].w);
                float4 b = beta[i], l = L[p];
                L[p] = make_float4(l.x + b.x * fmaxf(y[0], 0.0f), l.y + b.y * fmaxf(y[1], 0.0f),
                                   l.z + b.z * fmaxf(y[2], 0.0f), 0.0f);
            }
        }
    }
    if (tid == 0 && S.failed && status) atomicOr(status, 16u);   // bit 16: a tensor-core wait gave up
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" :: "r"(tmem));
}

// ---- inference (mma.sync) --------------------------------------------------------
// records: 4 float4 per query.  Result y (3 floats) goes to out[3i..] when out is
// given; otherwise, in render mode, L[path] += beta * max(y, 0) (one query per path).
// records: 4 float4 per query.  Result y (3 floats) goes to out[3i..] when out is
// given; otherwise, in render mode, L[path] += beta * max(y, 0) (one query per path).
__global__ void __launch_bounds__(128) k_mlp_infer(const uint2* __restrict__ wf_g, const float4* __restrict__ rec,
                                                   const uint32_t* __restrict__ n_ptr, uint32_t n_const,
                                                   EncodeParams ep, float* out, const float4* __restrict__ beta,
                                                   float4* L) {
    __shared__ uint2 wf[MLP_FWD_WORDS];
    __shared__ __align__(16) unsigned short X[4][16 * ROW_PAD];
    load_words(wf, wf_g, MLP_FWD_WORDS);
    __syncthreads();
    const uint32_t n = n_ptr ? *n_ptr : n_const;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    unsigned short* Xw = X[warp];
    const uint32_t tiles = (n + 15) / 16;
    for (uint32_t tile = blockIdx.x * 4 + warp; tile < tiles; tile += gridDim.x * 4) {
        const uint32_t row0 = tile * 16;
        {   // encode: lane -> sample lane/2, half lane%2
            const int sl = lane >> 1, half = lane & 1;
            const uint32_t i = row0 + sl;
            float f[32];
            if (i < n) {
                const float4* r = rec + 4ull * i;
                encode_half(r[0], r[1], r[2], r[3], ep, half, f);
            } else {
#pragma unroll
                for (int j = 0; j < 32; j++) f[j] = 0.0f;
            }
            uint32_t* dst = reinterpret_cast<uint32_t*>(Xw + sl * ROW_PAD + 32 * half);
#pragma unroll
            for (int j = 0; j < 16; j++) dst[j] = pack_bf16(f[2 * j], f[2 * j + 1]);
        }
        __syncwarp();
        uint32_t a[4][4];
#pragma unroll
        for (int kt = 0; kt < 4; kt++) {
            a[kt][0] = *reinterpret_cast<const uint32_t*>(Xw + g * ROW_PAD + 16 * kt + 2 * t);
            a[kt][1] = *reinterpret_cast<const uint32_t*>(Xw + (g + 8) * ROW_PAD + 16 * kt + 2 * t);
            a[kt][2] = *reinterpret_cast<const uint32_t*>(Xw + g * ROW_PAD + 16 * kt + 8 + 2 * t);
            a[kt][3] = *reinterpret_cast<const uint32_t*>(Xw + (g + 8) * ROW_PAD + 16 * kt + 8 + 2 * t);
        }
        __syncwarp();
        float c5[4];
        forward_tile<false>(wf, a, c5, nullptr, 0);
        // outputs: lane (g,0) holds cols 0,1 of rows g, g+8; lane (g,1) holds col 2
        float y2a = __shfl_down_sync(0xFFFFFFFFu, c5[0], 1);
        float y2b = __shfl_down_sync(0xFFFFFFFFu, c5[2], 1);
        if (t == 0) {
            const float ya[3] = {c5[0], c5[1], y2a}, yb[3] = {c5[2], c5[3], y2b};
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const uint32_t i = row0 + g + 8 * h;
                if (i >= n) continue;
                const float* y = h ? yb : ya;
                if (out) {
                    out[3ull * i] = y[0]; out[3ull * i + 1] = y[1]; out[3ull * i + 2] = y[2];
                } else {
                    const uint32_t p = __float_as_uint(rec[4ull * i + 3].w);
                    float4 b = beta[i], l = L[p];
                    L[p] = make_float4(l.x + b.x * fmaxf(y[0], 0.0f), l.y + b.y * fmaxf(y[1], 0.0f),
                                       l.z + b.z * fmaxf(y[2], 0.0f), 0.0f);
                }
            }
        }
    }
}

// encodings as floats (test hook): features of each record, bf16-rounded as the
// network consumes them
__global__ void k_mlp_encode(const float4* __restrict__ rec, uint32_t n, EncodeParams ep, float* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4* r = rec + 4ull * i;
    float f[32];
    for (int half = 0; half < 2; half++) {
        encode_half(r[0], r[1], r[2], r[3], ep, half, f);
        for (int j = 0; j < 32; j++) out[64ull * i + 32 * half + j] = bf16_bits_to_float(float_to_bf16_bits(f[j]));
    }
}

// ---- training: forward + backward of 128 samples per CTA -----------------------------
struct TrainSmem {
    uint2 wf[MLP_FWD_WORDS];
    uint2 wb[MLP_BWD_WORDS];
    unsigned short XT[64 * TS];
    unsigned short actT[4 * 64 * TS];
    unsigned short gT[64 * TS];
    float loss[8];
};

// one warp's share of a CTA-wide dW = act^T (64 x 128) . g (128 x ncols) with the
// result written to part[in * ncols + out]; warp w takes in-feature tile w>>1 and
// output tiles (w&1)*4 .. +3 (ncols = 64), or tile w for ncols = 3 (warps 0..3)
__device__ __forceinline__ void dw_gemm(const unsigned short* actT, const unsigned short* gT, int ncols,
                                        float* part) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    int mt, nt0, ntn;
    if (ncols == 64) { mt = warp >> 1; nt0 = (warp & 1) * 4; ntn = 4; }
    else { if (warp >= 4) return; mt = warp; nt0 = 0; ntn = 1; }
    float c[4][4];
#pragma unroll
    for (int j = 0; j < 4; j++) c[j][0] = c[j][1] = c[j][2] = c[j][3] = 0.0f;
#pragma unroll
    for (int kt = 0; kt < 8; kt++) {
        uint32_t a[4];
        const unsigned short* A0 = actT + (16 * mt + g) * TS + 16 * kt + 2 * t;
        const unsigned short* A1 = actT + (16 * mt + g + 8) * TS + 16 * kt + 2 * t;
        a[0] = *reinterpret_cast<const uint32_t*>(A0);
        a[1] = *reinterpret_cast<const uint32_t*>(A1);
        a[2] = *reinterpret_cast<const uint32_t*>(A0 + 8);
        a[3] = *reinterpret_cast<const uint32_t*>(A1 + 8);
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (j >= ntn) break;
            const unsigned short* B = gT + (8 * (nt0 + j) + g) * TS + 16 * kt + 2 * t;
            mma16816(c[j], a, *reinterpret_cast<const uint32_t*>(B), *reinterpret_cast<const uint32_t*>(B + 8));
        }
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
        if (j >= ntn) break;
        const int in0 = 16 * mt + g, out0 = 8 * (nt0 + j) + 2 * t;
        const float v[4] = {c[j][0], c[j][1], c[j][2], c[j][3]};
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int in = in0 + (r >= 2 ? 8 : 0), out = out0 + (r & 1);
            if (out < ncols) part[in * ncols + out] = v[r];
        }
    }
}

// dX for this warp's rows: g_next = (g . W^T) masked by act > 0, from A fragments
// a (K = ktn 16-wide tiles) and transposed weight blocks at wb + off
__device__ __forceinline__ void dx_tile(const uint2* wb, int off, int ktn, const uint32_t (*a)[4],
                                        const unsigned short* act, int row0, float (&c)[8][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < 8; nt++) c[nt][0] = c[nt][1] = c[nt][2] = c[nt][3] = 0.0f;
    for (int kt = 0; kt < ktn; kt++)
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            uint2 b = wb[off + (kt * 8 + nt) * 32 + lane];
            mma16816(c[nt], a[kt], b.x, b.y);
        }
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        const int f = 8 * nt + 2 * t;
        // ReLU derivative: the stored bf16 activation is positive (sign bit clear, nonzero)
        if ((short)act[f * TS + row0 + g] <= 0) c[nt][0] = 0.0f;
        if ((short)act[(f + 1) * TS + row0 + g] <= 0) c[nt][1] = 0.0f;
        if ((short)act[f * TS + row0 + g + 8] <= 0) c[nt][2] = 0.0f;
        if ((short)act[(f + 1) * TS + row0 + g + 8] <= 0) c[nt][3] = 0.0f;
    }
}

__device__ __forceinline__ void store_gT(unsigned short* gT, const float (&c)[8][4], int row0) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        const int f = 8 * nt + 2 * t;
        gT[f * TS + row0 + g] = float_to_bf16_bits(c[nt][0]);
        gT[(f + 1) * TS + row0 + g] = float_to_bf16_bits(c[nt][1]);
        gT[f * TS + row0 + g + 8] = float_to_bf16_bits(c[nt][2]);
        gT[(f + 1) * TS + row0 + g + 8] = float_to_bf16_bits(c[nt][3]);
    }
}

__device__ __forceinline__ void frags_from_c(const float (&c)[8][4], uint32_t (&a)[4][4]) {
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
        a[kt][0] = pack_bf16(c[2 * kt][0], c[2 * kt][1]);
        a[kt][1] = pack_bf16(c[2 * kt][2], c[2 * kt][3]);
        a[kt][2] = pack_bf16(c[2 * kt + 1][0], c[2 * kt + 1][1]);
        a[kt][3] = pack_bf16(c[2 * kt + 1][2], c[2 * kt + 1][3]);
    }
}

// samples: 5 float4 each (4 record words + (target rgb, weight)); part: per CTA
// MLP_NW floats; loss_part: per CTA loss sum.  norm = 1 / (3 * batch).
__global__ void __launch_bounds__(256) k_mlp_train(const uint2* __restrict__ wf_g, const uint2* __restrict__ wb_g,
                                                   const float4* __restrict__ samples, uint32_t n, EncodeParams ep,
                                                   float norm, float* part_all, float* loss_part) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TrainSmem& S = *reinterpret_cast<TrainSmem*>(smem_raw);
    load_words(S.wf, wf_g, MLP_FWD_WORDS);
    load_words(S.wb, wb_g, MLP_BWD_WORDS);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int row0 = 16 * warp;
    const uint32_t base = blockIdx.x * TRAIN_ROWS;
    float* part = part_all + (size_t)blockIdx.x * MLP_NW;
    // encode this warp's 16 samples into XT (transposed)
    {
        const int sl = lane >> 1, half = lane & 1;
        const uint32_t i = base + row0 + sl;
        float f[32];
        if (i < n) {
            const float4* r = samples + 5ull * i;
            encode_half(r[0], r[1], r[2], r[3], ep, half, f);
        } else {
#pragma unroll
            for (int j = 0; j < 32; j++) f[j] = 0.0f;
        }
#pragma unroll
        for (int j = 0; j < 32; j++) S.XT[(32 * half + j) * TS + row0 + sl] = float_to_bf16_bits(f[j]);
    }
    __syncthreads();
    uint32_t a[4][4];
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
        const int k0 = 16 * kt + 2 * t;
        auto pk = [&](int k, int s) {
            return (uint32_t)S.XT[k * TS + s] | ((uint32_t)S.XT[(k + 1) * TS + s] << 16);
        };
        a[kt][0] = pk(k0, row0 + g);
        a[kt][1] = pk(k0, row0 + g + 8);
        a[kt][2] = pk(k0 + 8, row0 + g);
        a[kt][3] = pk(k0 + 8, row0 + g + 8);
    }
    float c5[4];
    forward_tile<true>(S.wf, a, c5, S.actT, row0);
    // relative L2 loss gradient at the outputs (lanes t = 0: cols 0,1; t = 1: col 2)
    float lsum = 0.0f;
    float gy[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (t < 2) {
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int col = 2 * t + (r & 1);
            const uint32_t i = base + row0 + g + (r >= 2 ? 8 : 0);
            if (col < 3 && i < n) {
                const float4 tg = samples[5ull * i + 4];
                const float target = col == 0 ? tg.x : (col == 1 ? tg.y : tg.z);
                const float y = c5[r], d = y - target, den = y * y + 0.01f;
                lsum += tg.w * d * d / den * norm;
                gy[r] = tg.w * 2.0f * d / den * norm;
            }
        }
    }
    // g_out into gT rows 0..15 (rows 3..15 zero: they pad the 16-wide k tile)
    for (int f = lane; f < 16 * 16; f += 32) S.gT[(f >> 4) * TS + row0 + (f & 15)] = 0;
    __syncwarp();
    if (t < 2) {
        S.gT[(2 * t) * TS + row0 + g] = float_to_bf16_bits(gy[0]);
        S.gT[(2 * t + 1) * TS + row0 + g] = float_to_bf16_bits(gy[1]);
        S.gT[(2 * t) * TS + row0 + g + 8] = float_to_bf16_bits(gy[2]);
        S.gT[(2 * t + 1) * TS + row0 + g + 8] = float_to_bf16_bits(gy[3]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xFFFFFFFFu, lsum, o);
    if (lane == 0) S.loss[warp] = lsum;
    __syncthreads();
    // dW4 = act3^T g_out (in-features x 3)
    dw_gemm(S.actT + 3 * 64 * TS, S.gT, 3, part + MLP_OFF(4));
    // g3 = (g_out W4^T) * (act3 > 0): A = g_out rows (k = outputs 0..15, only 0..2 nonzero)
    float c[8][4];
    {
        uint32_t ag[1][4];
        auto pk = [&](int k, int s) {
            return (uint32_t)S.gT[k * TS + s] | ((uint32_t)S.gT[(k + 1) * TS + s] << 16);
        };
        ag[0][0] = pk(2 * t, row0 + g);
        ag[0][1] = pk(2 * t, row0 + g + 8);
        ag[0][2] = pk(2 * t + 8, row0 + g);
        ag[0][3] = pk(2 * t + 8, row0 + g + 8);
        dx_tile(S.wb, MLP_BWD_OFF(4), 1, ag, S.actT + 3 * 64 * TS, row0, c);
    }
    __syncthreads();   // every warp has read g_out
    store_gT(S.gT, c, row0);
    frags_from_c(c, a);
    __syncthreads();
    // layers 3, 2, 1: dW_l = act_{l-1}^T g_l ; g_{l-1} = (g_l W_l^T) * (act_{l-1} > 0)
#pragma unroll 1
    for (int l = 3; l >= 1; l--) {
        dw_gemm(S.actT + (l - 1) * 64 * TS, S.gT, 64, part + MLP_OFF(l));
        dx_tile(S.wb, MLP_BWD_OFF(l), 4, a, S.actT + (l - 1) * 64 * TS, row0, c);
        __syncthreads();
        store_gT(S.gT, c, row0);
        frags_from_c(c, a);
        __syncthreads();
    }
    // dW0 = X^T g_0
    dw_gemm(S.XT, S.gT, 64, part + MLP_OFF(0));
    if (threadIdx.x == 0) {
        float s = 0.0f;
        for (int w = 0; w < 8; w++) s += S.loss[w];
        loss_part[blockIdx.x] = s;
    }
}

// position of master weight (layer l, in i, out o) in the fragment-ordered bf16 buffers
__device__ __forceinline__ int frag_index(int block_words_off, int ntiles, int k, int n) {
    const int kt = k >> 4, rem = k & 15, reg = rem >> 3, t = (rem & 7) >> 1, hi = rem & 1;
    const int nt = n >> 3, g = n & 7, lane = g * 4 + t;
    return ((block_words_off + (kt * ntiles + nt) * 32 + lane) * 2 + reg) * 2 + hi;
}

// sums the CTA partials in a fixed order, one Adam step in FP32, BF16 copies
__global__ void k_mlp_adam(const float* __restrict__ part, uint32_t nparts, float* w, float* m, float* v,
                           AdamParams ap, unsigned short* wf, unsigned short* wb, unsigned short* wtc,
                           float* grad_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= MLP_NW) return;
    float gsum = 0.0f;
    for (uint32_t c = 0; c < nparts; c++) gsum += part[(size_t)c * MLP_NW + i];
    if (grad_out) grad_out[i] = gsum;
    float wi = w[i];
    if (ap.lr > 0.0f) {
        float mi = ap.b1 * m[i] + (1.0f - ap.b1) * gsum;
        float vi = ap.b2 * v[i] + (1.0f - ap.b2) * gsum * gsum;
        m[i] = mi;
        v[i] = vi;
        wi -= ap.lr * (mi / ap.c1) / (sqrtf(vi / ap.c2) + ap.eps);
        w[i] = wi;
    }
    const unsigned short b = float_to_bf16_bits(wi);
    int l, in, out;
    if (i < 4 * 4096) { l = i >> 12; in = (i >> 6) & 63; out = i & 63; }
    else { l = 4; in = (i - 4 * 4096) / 3; out = (i - 4 * 4096) % 3; }
    wf[frag_index(MLP_FWD_OFF(l), l < 4 ? 8 : 1, in, out)] = b;
    if (l >= 1) wb[frag_index(MLP_BWD_OFF(l), 8, out, in)] = b;
    wtc[l * 4096 + tc_off((uint32_t)out, (uint32_t)in) / 2] = b;   // N = out, K = in
}

}  // namespace

// ---- host side ------------------------------------------------------------------------
Status mlp_init(MlpState& M, const float* w_host, cudaStream_t st) {
    SNK_TRY_CUDA(M.w.reserve(MLP_NW));
    SNK_TRY_CUDA(M.m.reserve(MLP_NW));
    SNK_TRY_CUDA(M.v.reserve(MLP_NW));
    SNK_TRY_CUDA(M.wf.reserve(MLP_FWD_WORDS));
    SNK_TRY_CUDA(M.wb.reserve(MLP_BWD_WORDS));
    SNK_TRY_CUDA(M.wtc.reserve(MLP_TC_ELEMS));
    SNK_TRY_CUDA(cudaMemcpyAsync(M.w.p, w_host, MLP_NW * sizeof(float), cudaMemcpyHostToDevice, st));
    SNK_TRY_CUDA(cudaMemsetAsync(M.wtc.p, 0, MLP_TC_ELEMS * sizeof(unsigned short), st));
    SNK_TRY_CUDA(cudaMemsetAsync(M.m.p, 0, MLP_NW * sizeof(float), st));
    SNK_TRY_CUDA(cudaMemsetAsync(M.v.p, 0, MLP_NW * sizeof(float), st));
    SNK_TRY_CUDA(cudaMemsetAsync(M.wf.p, 0, MLP_FWD_WORDS * sizeof(uint2), st));
    SNK_TRY_CUDA(cudaMemsetAsync(M.wb.p, 0, MLP_BWD_WORDS * sizeof(uint2), st));
    // the training kernel's shared memory exceeds the default limit (set here, not
    // per launch, so frames can be captured into CUDA graphs)
    SNK_TRY_CUDA(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sizeof(TrainSmem)));
    SNK_TRY_CUDA(cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sizeof(InferSmem)));
    AdamParams ap{};   // lr 0: only refresh the BF16 copies
    k_mlp_adam<<<(MLP_NW + 255) / 256, 256, 0, st>>>(M.w.p, 0, M.w.p, M.m.p, M.v.p, ap,
                                                     reinterpret_cast<unsigned short*>(M.wf.p),
                                                     reinterpret_cast<unsigned short*>(M.wb.p), M.wtc.p, nullptr);
    SNK_TRY_CUDA(cudaGetLastError());
    M.step = 0;
    M.ready = true;
    return Status::Ok();
}

Status mlp_infer(const MlpState& M, const float4* rec, const uint32_t* n_dev, uint32_t n, const EncodeParams& ep,
                 float* out, const float4* beta, float4* L, int grid, unsigned* err_word, cudaStream_t st) {
    k_mlp_infer_tc<<<grid, INFER_THREADS, sizeof(InferSmem), st>>>(M.wtc.p, rec, n_dev, n, ep, out, beta, L,
                                                                     err_word);
    SNK_TRY_CUDA(cudaGetLastError());
    return Status::Ok();
}

Status mlp_encode(const float4* rec, uint32_t n, const EncodeParams& ep, float* out, cudaStream_t st) {
    if (n) k_mlp_encode<<<(n + 127) / 128, 128, 0, st>>>(rec, n, ep, out);
    SNK_TRY_CUDA(cudaGetLastError());
    return Status::Ok();
}

Status mlp_train_reserve(MlpState& M, uint32_t n) {
    const uint32_t ctas = (n + TRAIN_ROWS - 1) / TRAIN_ROWS;
    SNK_TRY_CUDA(M.part.reserve((size_t)ctas * MLP_NW));
    SNK_TRY_CUDA(M.loss.reserve(ctas));
    return Status::Ok();
}

Status mlp_train_step(MlpState& M, const float4* samples, uint32_t n, const EncodeParams& ep, float lr,
                      float* grad_out, float* loss_host, cudaStream_t st) {
    if (n == 0) return Status::Ok();
    const uint32_t ctas = (n + TRAIN_ROWS - 1) / TRAIN_ROWS;
    Status rs = mlp_train_reserve(M, n);
    if (!rs.ok()) return rs;
    k_mlp_train<<<ctas, 256, sizeof(TrainSmem), st>>>(M.wf.p, M.wb.p, samples, n, ep, 1.0f / (3.0f * (float)n),
                                                      M.part.p, M.loss.p);
    SNK_TRY_CUDA(cudaGetLastError());
    M.step++;
    AdamParams ap;
    ap.lr = lr;
    ap.b1 = 0.9f;
    ap.b2 = 0.99f;
    ap.eps = 1e-8f;
    ap.c1 = (float)(1.0 - std::pow(0.9, (double)M.step));
    ap.c2 = (float)(1.0 - std::pow(0.99, (double)M.step));
    k_mlp_adam<<<(MLP_NW + 255) / 256, 256, 0, st>>>(M.part.p, ctas, M.w.p, M.m.p, M.v.p, ap,
                                                     reinterpret_cast<unsigned short*>(M.wf.p),
                                                     reinterpret_cast<unsigned short*>(M.wb.p), M.wtc.p, grad_out);
    SNK_TRY_CUDA(cudaGetLastError());
    if (loss_host) {
        std::vector<float> lp(ctas);
        SNK_TRY_CUDA(cudaMemcpyAsync(lp.data(), M.loss.p, ctas * sizeof(float), cudaMemcpyDeviceToHost, st));
        SNK_TRY_CUDA(cudaStreamSynchronize(st));
        double s = 0.0;
        for (float x : lp) s += x;
        *loss_host = (float)s;
    }
    return Status::Ok();
}

}  // namespace snk
