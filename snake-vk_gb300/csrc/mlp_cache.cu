// mlp_cache.cu -- the online-trained MLP radiance cache: input encoding, fused
// inference, fused forward+backward training and the Adam update, on the
// fifth-generation BF16 tensor cores (tcgen05.mma, FP32 accumulation in tensor
// memory).  There is no counterpart in the reference; this is the learned part
// of the path tracer (cache queries replace path tails, radiance-caching style,
// Mueller et al. 2021).
//
// Network: 64 encoded inputs -> 4 x (64, ReLU) -> 3 linear outputs, no biases
// (the encoding carries a constant 1).  FP32 master weights W_l[in][out]
// (4 x 64x64 then 64x3 = 16576 values) with Adam moments; the tensor cores read
// BF16 copies that the Adam kernel writes in the tcgen05 shared-memory operand
// layout (K-major, no swizzle: 8x8 core matrices of 128 contiguous bytes), one
// with N = outputs (forward) and one with N = inputs (input gradients).
//
// Inference: one CTA of 128 threads takes 128 queries, writes their encodings
// into shared memory in the operand layout, and chains the 5 layers as 128x64x64
// (last 128x16x64) tcgen05.mma issued by one thread, accumulating in tensor
// memory; after each layer every thread reads its row back with tcgen05.ld,
// applies the ReLU and stores the BF16 row as the next layer's operand.
// Training does the same forward pass for 128 samples, then the backward pass as
// tcgen05 GEMMs as well (input gradients M = 128, weight gradients M = 64 from
// the stored activations read as MN-major operands).  Each CTA writes its dW
// partial; the Adam kernel sums the partials in a fixed order, so training is
// deterministic.  Waits on the MMA completion barrier are bounded (a give-up sets
// a status bit, read by the host).
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

constexpr int TRAIN_ROWS = 128; // samples per training CTA (one per thread)

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float bf16_bits_to_float(unsigned short b) { return __uint_as_float((uint32_t)b << 16); }
__device__ __forceinline__ unsigned short float_to_bf16_bits(float f) {
    __nv_bfloat16 h = __float2bfloat16_rn(f);
    return *reinterpret_cast<unsigned short*>(&h);
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

// Give-up protocol of the tensor-core kernels.  When a bounded wait gives up, the
// work it waited for (MMAs writing tensor memory, bulk copies writing shared
// memory) may still be in flight, so the CTA issues nothing more and records the
// abandoned barrier phase; before it frees its tensor memory and exits, thread 0
// waits for that phase once more, again with a bound (drain_abandoned).  Status
// bits: 16 a wait gave up; 32 the second wait gave up too (the tensor memory is
// then freed with that work still pending, as the kernel cannot stall forever).
struct GiveUp {
    uint32_t failed;    // a wait gave up: issue nothing more
    uint32_t bar, parity;   // the barrier phase that was abandoned
};
__device__ __forceinline__ void give_up(GiveUp& g, uint32_t bar, uint32_t parity) {
    g.failed = 1u;
    g.bar = bar;
    g.parity = parity;
}
// thread 0, before the final barrier of the CTA: drain, then report
__device__ __forceinline__ void drain_abandoned(const GiveUp& g, unsigned* status) {
    if (!g.failed) return;
    const bool drained = mbar_wait(g.bar, g.parity);
    if (status) atomicOr(status, drained ? 16u : 48u);
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
    GiveUp gu;
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
        S.gu.failed = 0u;
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
                if (!mbar_wait(mbar, parity)) give_up(S.gu, mbar, parity);
            }
            parity ^= 1u;
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;");
            ok = S.gu.failed == 0u;
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
    if (tid == 0) drain_abandoned(S.gu, status);
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" :: "r"(tmem));
}

// ---- training on tcgen05: forward + backward of 128 samples per CTA -------------------
// Sample s is owned by threads s and s + 128 (warps w and w + 4 share tensor-memory
// lanes 32 (w % 4) ..); thread half h = tid / 128 handles features / columns
// [32h, 32h + 32).  Every activation A_l (A_0 = encoded input, A_l = output of
// layer l-1) and the running output gradient G are stored once, row s, in the
// K-major operand layout of a 128 x 64 matrix.  The same bytes serve three GEMMs:
//   forward       A_{l+1} = relu(A_l W_l)          M = 128, A_l K-major, W_l (N = out, K = in)
//   input grad    G' = (G W_l^T) * [A_l > 0]        M = 128, G K-major, W_l^T (N = in, K = out)
//   weight grad   dW_l = A_l^T G                    M = 64 (in), N = out, K = 128 samples:
//                                                    A_l and G read as MN-major operands
// so no transpose is ever written.  Read as an MN-major operand, such a buffer has
// its 8-sample row groups (K direction) 1024 B apart, given as the leading byte
// offset, and its 8-feature chunks (M/N direction) 128 B apart, given as the
// stride byte offset: the two fields swap roles against the K-major descriptor
// (measured on GB300 with a 64 x 64 x 128 product).  The M = 64 accumulator puts row m
// in tensor-memory lane 32 (m / 16) + m % 16: warp w % 4, lanes 0..15 hold
// in-features 16 (w % 4) .. + 15.  Tensor memory: columns 0..63 forward / input
// gradient, 64..127 weight gradient.  The weights arrive by two bulk asynchronous
// copies that overlap the input encoding; the ReLU masks of A_1..A_4 stay in
// registers (32 bits per thread each).
constexpr int TRAIN_TC_THREADS = 256;

struct TrainTcSmem {
    unsigned short wf[MLP_TC_ELEMS];     // W_l: N = out x K = in (layer 4: N = 16)
    unsigned short wb[MLP_TCB_ELEMS];    // W_l^T, l = 1..4: N = in x K = out (layer 4: K = 3 of 16 used)
    unsigned short act[5][128 * 64];     // A_0 .. A_4
    unsigned short g[128 * 64];          // gradient at the current layer's output
    unsigned long long mbar;             // MMA completion
    unsigned long long wbar;             // weight copies
    uint32_t tmem;
    GiveUp gu;
    float loss[8];
};

// descriptor of a 128-sample x 64-feature buffer read as an MN-major operand
__device__ __forceinline__ uint64_t tc_desc_mn(uint32_t addr) {
    uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)(1024u >> 4) << 16;   // K direction: next 8 samples
    d |= (uint64_t)(128u >> 4) << 32;    // M/N direction: next 8 features
    d |= (uint64_t)1 << 46;
    return d;
}

// instruction descriptor of the weight-gradient GEMM: M = 64, A and B MN-major
__device__ __forceinline__ uint32_t tc_idesc_wgrad(uint32_t n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) | ((n >> 3) << 17) | ((64u >> 4) << 24);
}

// D[tmem] = sum over ksteps of A B^T; operand addresses advance by kstride bytes per K = 16 step
template <bool MN>
__device__ __forceinline__ void tc_issue(uint32_t tmem, uint32_t a_addr, uint32_t b_addr, uint32_t idesc,
                                         uint32_t ksteps, uint32_t kstride) {
#pragma unroll 1
    for (uint32_t ks = 0; ks < ksteps; ks++) {
        const uint64_t da = MN ? tc_desc_mn(a_addr + ks * kstride) : tc_desc(a_addr + ks * kstride);
        const uint64_t db = MN ? tc_desc_mn(b_addr + ks * kstride) : tc_desc(b_addr + ks * kstride);
        const uint32_t acc = ks > 0 ? 1u : 0u;
        asm volatile("{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                     " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                     :: "r"(tmem), "l"(da), "l"(db), "r"(idesc), "r"(acc));
    }
}

__device__ __forceinline__ void tc_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(mbar));
}

// global -> shared bulk copy (16-byte aligned, size a multiple of 16) completing on mbar
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(dst), "l"(src), "r"(bytes), "r"(mbar) : "memory");
}

// 32 values into columns [col0, col0 + 32) of row `row` of a K-major 128 x 64
// operand as BF16; returns the positive-value mask (bit j: value j > 0 after rounding)
__device__ __forceinline__ uint32_t store_row32(unsigned char* base, uint32_t row, uint32_t col0, const float* v) {
    uint32_t mask = 0;
#pragma unroll
    for (int kb = 0; kb < 4; kb++) {
        uint32_t w[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            w[j] = pack_bf16(v[8 * kb + 2 * j], v[8 * kb + 2 * j + 1]);
            if ((short)(w[j] & 0xFFFFu) > 0) mask |= 1u << (8 * kb + 2 * j);
            if ((short)(w[j] >> 16) > 0) mask |= 1u << (8 * kb + 2 * j + 1);
        }
        *reinterpret_cast<uint4*>(base + tc_off(row, col0 + 8u * kb)) = make_uint4(w[0], w[1], w[2], w[3]);
    }
    return mask;
}

// samples: 5 float4 each (4 record words + (target rgb, weight)); part: per CTA
// MLP_NW floats (W_l[in][out] order); loss_part: per CTA loss sum; norm = 1 / (3 * batch).
// wtc_g / wtcb_g: 16-byte aligned.  A give-up of a bounded wait sets bit 16 of *status.
__global__ void __launch_bounds__(TRAIN_TC_THREADS, 1) k_mlp_train_tc(const unsigned short* __restrict__ wtc_g,
                                                                   const unsigned short* __restrict__ wtcb_g,
                                                                   const float4* __restrict__ samples, uint32_t n,
                                                                   EncodeParams ep, float norm, float* part_all,
                                                                   float* loss_part, unsigned* status) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    TrainTcSmem& S = *reinterpret_cast<TrainTcSmem*>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t row = (uint32_t)tid & 127u, half = (uint32_t)tid >> 7, col0 = 32u * half;
    const uint32_t mbar = smem_u32(&S.mbar), wbar = smem_u32(&S.wbar);
    constexpr uint32_t WF_BYTES = MLP_TC_ELEMS * 2, WB_BYTES = MLP_TCB_ELEMS * 2;
    if (tid == 0) {
        S.gu.failed = 0u;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(mbar));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(wbar));
        asm volatile("fence.mbarrier_init.release.cluster;");
        asm volatile("fence.proxy.async.shared::cta;");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(wbar), "r"(WF_BYTES + WB_BYTES)
                     : "memory");
        bulk_load(smem_u32(S.wf), wtc_g, WF_BYTES, wbar);
        bulk_load(smem_u32(S.wb), wtcb_g, WB_BYTES, wbar);
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" :: "r"(smem_u32(&S.tmem)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    const uint32_t i = blockIdx.x * 128u + row;
    {   // encode this thread's half of its sample into A_0
        float f[32];
        if (i < n) {
            const float4* r = samples + 5ull * i;
            encode_half(r[0], r[1], r[2], r[3], ep, (int)half, f);
        } else {
#pragma unroll
            for (int j = 0; j < 32; j++) f[j] = 0.0f;
        }
        store_row32(reinterpret_cast<unsigned char*>(S.act[0]), row, col0, f);
    }
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = S.tmem, wf = smem_u32(S.wf), wb = smem_u32(S.wb), g_addr = smem_u32(S.g);
    const uint32_t lane_base = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    uint32_t parity = 0;
    uint32_t msk[4] = {0u, 0u, 0u, 0u};   // positive masks of this thread's columns of A_1 .. A_4
    float lsum = 0.0f;
    bool ok = true;
    if (tid == 0 && !mbar_wait(wbar, 0)) give_up(S.gu, wbar, 0u);   // the weights are in shared memory
    // runs the GEMMs `issue` queues (thread 0), then waits for them with a bound
    auto run = [&](auto issue) {
        asm volatile("fence.proxy.async.shared::cta;");
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
        if (tid == 0 && S.gu.failed == 0u) {
            asm volatile("tcgen05.fence::after_thread_sync;");
            issue();
            tc_commit(mbar);
            if (!mbar_wait(mbar, parity)) give_up(S.gu, mbar, parity);
        }
        parity ^= 1u;
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;");
        return S.gu.failed == 0u;
    };
    // forward
#pragma unroll
    for (int l = 0; l < 5; l++) {
        if (!ok) break;
        const uint32_t a_addr = smem_u32(S.act[l]);
        ok = run([&] { tc_issue<false>(tmem, a_addr, wf + (uint32_t)l * 8192u, tc_idesc(l < 4 ? 64u : 16u), 4, 256); });
        if (!ok) break;
        if (l < 4) {
            uint32_t r[32];
            SNK_TC_LD16(lane_base + col0, r, 0);
            SNK_TC_LD16(lane_base + col0 + 16u, r, 16);
            asm volatile("tcgen05.wait::ld.sync.aligned;");
            float v[32];
#pragma unroll
            for (int j = 0; j < 32; j++) v[j] = fmaxf(__uint_as_float(r[j]), 0.0f);
            msk[l] = store_row32(reinterpret_cast<unsigned char*>(S.act[l + 1]), row, col0, v);
        } else if (half == 0) {
            uint32_t r[16];
            SNK_TC_LD16(lane_base, r, 0);
            asm volatile("tcgen05.wait::ld.sync.aligned;");
            // relative L2 loss and its gradient at the 3 outputs (columns 3..15 of G zero)
            float gy[16];
#pragma unroll
            for (int j = 0; j < 16; j++) gy[j] = 0.0f;
            if (i < n) {
                const float4 tg = samples[5ull * i + 4];
                const float target[3] = {tg.x, tg.y, tg.z};
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const float y = __uint_as_float(r[c]), d = y - target[c], den = y * y + 0.01f;
                    lsum += tg.w * d * d / den * norm;
                    gy[c] = tg.w * 2.0f * d / den * norm;
                }
            }
            unsigned char* gb = reinterpret_cast<unsigned char*>(S.g);
#pragma unroll
            for (int kb = 0; kb < 2; kb++)
                *reinterpret_cast<uint4*>(gb + tc_off(row, 8u * kb)) =
                    make_uint4(pack_bf16(gy[8 * kb], gy[8 * kb + 1]), pack_bf16(gy[8 * kb + 2], gy[8 * kb + 3]),
                               pack_bf16(gy[8 * kb + 4], gy[8 * kb + 5]), pack_bf16(gy[8 * kb + 6], gy[8 * kb + 7]));
        }
    }
    // backward: layer l takes G (gradient at its output), writes dW_l and, for l >= 1,
    // the gradient at its input into G
    float* part = part_all + (size_t)blockIdx.x * MLP_NW;
#pragma unroll
    for (int l = 4; l >= 0; l--) {
        if (!ok) break;
        const uint32_t a_addr = smem_u32(S.act[l]);
        ok = run([&] {
            tc_issue<true>(tmem + 64u, a_addr, g_addr, tc_idesc_wgrad(l == 4 ? 16u : 64u), 8, 2048);
            if (l >= 1) tc_issue<false>(tmem, g_addr, wb + (uint32_t)(l - 1) * 8192u, tc_idesc(64u), l == 4 ? 1u : 4u, 256);
        });
        if (!ok) break;
        // dW_l: in-feature 16 (warp % 4) + lane on lanes 0..15, out-features col0 .. col0 + 31
        if (l == 4) {
            if (half == 0) {
                uint32_t r[16];
                SNK_TC_LD16(lane_base + 64u, r, 0);
                asm volatile("tcgen05.wait::ld.sync.aligned;");
                if (lane < 16) {
                    float* dst = part + MLP_OFF(4) + (16 * (warp & 3) + lane) * 3;
                    dst[0] = __uint_as_float(r[0]); dst[1] = __uint_as_float(r[1]); dst[2] = __uint_as_float(r[2]);
                }
            }
        } else {
            uint32_t r[32];
            SNK_TC_LD16(lane_base + 64u + col0, r, 0);
            SNK_TC_LD16(lane_base + 80u + col0, r, 16);
            asm volatile("tcgen05.wait::ld.sync.aligned;");
            if (lane < 16) {
                float4* dst = reinterpret_cast<float4*>(part + MLP_OFF(l) + (16 * (warp & 3) + lane) * 64 + col0);
#pragma unroll
                for (int q = 0; q < 8; q++)
                    dst[q] = make_float4(__uint_as_float(r[4 * q]), __uint_as_float(r[4 * q + 1]),
                                         __uint_as_float(r[4 * q + 2]), __uint_as_float(r[4 * q + 3]));
            }
        }
        if (l >= 1) {   // G <- (G W_l^T) * [A_l > 0]
            uint32_t r[32];
            SNK_TC_LD16(lane_base + col0, r, 0);
            SNK_TC_LD16(lane_base + col0 + 16u, r, 16);
            asm volatile("tcgen05.wait::ld.sync.aligned;");
            const uint32_t m = msk[l - 1];
            float v[32];
#pragma unroll
            for (int j = 0; j < 32; j++) v[j] = (m >> j) & 1u ? __uint_as_float(r[j]) : 0.0f;
            store_row32(reinterpret_cast<unsigned char*>(S.g), row, col0, v);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xFFFFFFFFu, lsum, o);
    if (lane == 0) S.loss[warp] = lsum;
    if (tid == 0) drain_abandoned(S.gu, status);
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (tid == 0) {
        float t = 0.0f;
        for (int w = 0; w < 8; w++) t += S.loss[w];
        loss_part[blockIdx.x] = t;
    }
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" :: "r"(tmem));
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

// sums the CTA partials in a fixed order, one Adam step in FP32, the two BF16 operand copies
__global__ void k_mlp_adam(const float* __restrict__ part, uint32_t nparts, float* w, float* m, float* v,
                           AdamParams ap, unsigned short* wtc, unsigned short* wtcb, float* grad_out) {
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
    wtc[l * 4096 + tc_off((uint32_t)out, (uint32_t)in) / 2] = b;                        // N = out, K = in
    if (l >= 1) wtcb[(l - 1) * 4096 + tc_off((uint32_t)in, (uint32_t)out) / 2] = b;   // N = in, K = out
}

}  // namespace

// ---- host side ------------------------------------------------------------------------
Status mlp_init(MlpState& M, const float* w_host, cudaStream_t st) {
    SNK_TRY_CUDA(M.w.reserve(MLP_NW));
    SNK_TRY_CUDA(M.m.reserve(MLP_NW));
    SNK_TRY_CUDA(M.v.reserve(MLP_NW));
    SNK_TRY_CUDA(M.wtc.reserve(MLP_TC_ELEMS));
    SNK_TRY_CUDA(M.wtcb.reserve(MLP_TCB_ELEMS));
    SNK_TRY_CUDA(cudaMemcpyAsync(M.w.p, w_host, MLP_NW * sizeof(float), cudaMemcpyHostToDevice, st));
    SNK_TRY_CUDA(cudaMemsetAsync(M.wtc.p, 0, MLP_TC_ELEMS * sizeof(unsigned short), st));
    SNK_TRY_CUDA(cudaMemsetAsync(M.wtcb.p, 0, MLP_TCB_ELEMS * sizeof(unsigned short), st));
    SNK_TRY_CUDA(cudaMemsetAsync(M.m.p, 0, MLP_NW * sizeof(float), st));
    SNK_TRY_CUDA(cudaMemsetAsync(M.v.p, 0, MLP_NW * sizeof(float), st));
    // the kernels' shared memory exceeds the default limit (set here, not per
    // launch, so frames can be captured into CUDA graphs)
    SNK_TRY_CUDA(cudaFuncSetAttribute(k_mlp_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sizeof(TrainTcSmem)));
    SNK_TRY_CUDA(cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sizeof(InferSmem)));
    AdamParams ap{};   // lr 0: only refresh the BF16 copies
    k_mlp_adam<<<(MLP_NW + 255) / 256, 256, 0, st>>>(M.w.p, 0, M.w.p, M.m.p, M.v.p, ap, M.wtc.p, M.wtcb.p,
                                                     nullptr);
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
                      float* grad_out, float* loss_host, unsigned* err_word, cudaStream_t st) {
    if (n == 0) return Status::Ok();
    const uint32_t ctas = (n + TRAIN_ROWS - 1) / TRAIN_ROWS;
    Status rs = mlp_train_reserve(M, n);
    if (!rs.ok()) return rs;
    k_mlp_train_tc<<<ctas, TRAIN_TC_THREADS, sizeof(TrainTcSmem), st>>>(
        M.wtc.p, M.wtcb.p, samples, n, ep, 1.0f / (3.0f * (float)n), M.part.p, M.loss.p, err_word);
    SNK_TRY_CUDA(cudaGetLastError());
    M.step++;
    AdamParams ap;
    ap.lr = lr;
    ap.b1 = 0.9f;
    ap.b2 = 0.99f;
    ap.eps = 1e-8f;
    ap.c1 = (float)(1.0 - std::pow(0.9, (double)M.step));
    ap.c2 = (float)(1.0 - std::pow(0.99, (double)M.step));
    k_mlp_adam<<<(MLP_NW + 255) / 256, 256, 0, st>>>(M.part.p, ctas, M.w.p, M.m.p, M.v.p, ap, M.wtc.p, M.wtcb.p,
                                                     grad_out);
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
