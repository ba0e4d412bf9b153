// taa.cu -- temporal anti-aliasing resolve of the path tracer's radiance.
//
// Restates TAA_Resolve.comp (Core/res/shaders/TAA_Resolve.comp:12-86) and the
// history handling of TAA_ResolvePass (Core/src/renderpasses/TAA_ResolvePass.cpp:
// 6-56).  Compiled with --fmad=false: every operation is a binary32 basic
// operation in the shader's order, so the CPU oracle reproduces it bit for bit.
//
// Differences from the pass, by design:
//   * out-of-place: every pixel reads the unresolved frame (the shader resolves
//     img_current_frame in place, so a pixel's 3x3 neighbourhood may already hold
//     resolved values of neighbouring invocations);
//   * every pixel is resolved (the pass dispatches floor(W/8) x floor(H/8) groups
//     and leaves a right/bottom remainder unresolved when W or H is not a
//     multiple of 8);
//   * bilinear history/velocity fetches in FP32 with exact weights (texture units
//     quantise the weights to a few bits);
//   * the history starts as the first frame (the pass's history image starts
//     undefined).
//
// Kernel: 32x8 pixels per block, the 34x10 halo tile of the current frame staged
// in shared memory (coalesced float4 loads, issued first and held in registers
// until the motion-dependent gathers are in flight), history and previous
// velocity fetched through L1 (neighbouring pixels share texels).  HBM bound: 88 B per
// pixel (16 current + 8 motion + 16 history + 8 previous motion in; 16 out, 16
// next history, 8 next previous motion).
#include <cstring>
#include <string>

#include "snk_host.h"
#include "../../include/snk_pt.h"

namespace snk {
namespace {

constexpr int TX = 32, TY = 8;

struct TaaImages {
    const float4* cur;
    const float2* motion;
    const float4* hist;
    const float2* pmot;
    float4* out;        // may be null
    float4* hist_next;
    float2* pmot_next;
    int w, h;
};

__device__ __forceinline__ int wrap_repeat(int i, int n) {
    int r = i % n;
    return r < 0 ? r + n : r;
}

// texture() with a linear filter and repeat addressing, in FP32: the four texels
// are fetched first (so that their loads are in flight together with the
// frame's tile), the weights are applied later
template <class T>
struct Bilinear {
    T t00, t10, t01, t11;
    float w00, w10, w01, w11;
    __device__ __forceinline__ void fetch(const T* __restrict__ img, int w, int h, float cu, float cv) {
        const float u = cu * (float)w - 0.5f, v = cv * (float)h - 0.5f;
        const float fu = floorf(u), fv = floorf(v);
        const float a = u - fu, b = v - fv;
        const int i0 = wrap_repeat((int)fu, w), i1 = wrap_repeat((int)fu + 1, w);
        const int j0 = wrap_repeat((int)fv, h), j1 = wrap_repeat((int)fv + 1, h);
        w00 = (1.0f - a) * (1.0f - b); w10 = a * (1.0f - b); w01 = (1.0f - a) * b; w11 = a * b;
        t00 = img[(size_t)j0 * w + i0];
        t10 = img[(size_t)j0 * w + i1];
        t01 = img[(size_t)j1 * w + i0];
        t11 = img[(size_t)j1 * w + i1];
    }
    template <int C>
    __device__ __forceinline__ void apply(float* o) const {
        const float* a = reinterpret_cast<const float*>(&t00);
        const float* b = reinterpret_cast<const float*>(&t10);
        const float* c = reinterpret_cast<const float*>(&t01);
        const float* d = reinterpret_cast<const float*>(&t11);
        for (int k = 0; k < C; k++) o[k] = ((w00 * a[k] + w10 * b[k]) + w01 * c[k]) + w11 * d[k];
    }
};

__global__ void __launch_bounds__(TX * TY) k_taa_resolve(TaaImages I) {
    __shared__ float4 tile[TY + 2][TX + 2];
    const int bx = blockIdx.x * TX, by = blockIdx.y * TY;
    const int t = threadIdx.y * TX + threadIdx.x;
    const int x = bx + threadIdx.x, y = by + threadIdx.y;
    const bool inside = x < I.w && y < I.h;
    const size_t pix = inside ? (size_t)y * I.w + x : 0;
    // the tile's texels first (independent loads, into registers), then this
    // pixel's motion and its reprojected history and previous-velocity texels
    constexpr int TN = ((TX + 2) * (TY + 2) + TX * TY - 1) / (TX * TY);
    float4 tv[TN];
#pragma unroll
    for (int q = 0; q < TN; q++) {
        const int k = t + q * TX * TY;
        if (k < (TX + 2) * (TY + 2)) {
            const int ly = k / (TX + 2), lx = k % (TX + 2);
            const int gx = min(max(bx + lx - 1, 0), I.w - 1), gy = min(max(by + ly - 1, 0), I.h - 1);
            tv[q] = I.cur[(size_t)gy * I.w + gx];
        }
    }
    float2 vel = make_float2(0.0f, 0.0f);
    Bilinear<float4> hb;
    Bilinear<float2> pb;
    if (inside) {
        vel = I.motion[pix];
        float hx = ((float)x + 0.5f) / (float)I.w + vel.x;
        float hy = ((float)y + 0.5f) / (float)I.h + vel.y;
        hx = fminf(fmaxf(hx, 0.0f), 1.0f);
        hy = fminf(fmaxf(hy, 0.0f), 1.0f);
        hb.fetch(I.hist, I.w, I.h, hx, hy);
        pb.fetch(I.pmot, I.w, I.h, hx, hy);
    }
#pragma unroll
    for (int q = 0; q < TN; q++) {
        const int k = t + q * TX * TY;
        if (k < (TX + 2) * (TY + 2)) tile[k / (TX + 2)][k % (TX + 2)] = tv[q];
    }
    __syncthreads();
    if (!inside) return;
    const float4 cur4 = tile[threadIdx.y + 1][threadIdx.x + 1];
    const float cur[3] = {cur4.x, cur4.y, cur4.z};
    float mn[3] = {9999.0f, 9999.0f, 9999.0f}, mx[3] = {-9999.0f, -9999.0f, -9999.0f};
    float m[3] = {0.0f, 0.0f, 0.0f}, m2[3] = {0.0f, 0.0f, 0.0f};
    for (int ox = -1; ox <= 1; ox++) {
        for (int oy = -1; oy <= 1; oy++) {
            // the tile's halo already holds the clamped neighbours
            const float4 c4 = tile[threadIdx.y + 1 + oy][threadIdx.x + 1 + ox];
            const float col[3] = {fmaxf(c4.x, 0.0f), fmaxf(c4.y, 0.0f), fmaxf(c4.z, 0.0f)};
            for (int c = 0; c < 3; c++) {
                mn[c] = fminf(mn[c], col[c]);
                mx[c] = fmaxf(mx[c], col[c]);
                m[c] = m[c] + col[c];
                m2[c] = m2[c] + col[c] * col[c];
            }
        }
    }
    const float inv9 = 1.0f / 9.0f, gamma = 0.55f, eps = 0.00000001f;
    float mu[3], minc[3], maxc[3], p[3];
    for (int c = 0; c < 3; c++) {
        mu[c] = m[c] * inv9;
        const float sigma = sqrtf(fabsf(m2[c] * inv9 - mu[c] * mu[c]));
        minc[c] = mu[c] - gamma * sigma;
        maxc[c] = mu[c] + gamma * sigma;
        p[c] = fminf(fmaxf(mu[c], mn[c]), mx[c]);
    }
    float hist[3];
    hb.apply<3>(hist);
    // clip_aabb(minc, maxc, vec4(p, 1), vec4(hist, 1)); r.w stays 0
    float r[3];
    for (int c = 0; c < 3; c++) r[c] = fmaxf(hist[c], 0.0f) - p[c];
    for (int c = 0; c < 3; c++) {
        const float rmax = maxc[c] - p[c];
        if (r[c] > rmax + eps) {
            const float s = rmax / r[c];
            for (int k = 0; k < 3; k++) r[k] = r[k] * s;
        }
    }
    for (int c = 0; c < 3; c++) {
        const float rmin = minc[c] - p[c];
        if (r[c] < rmin - eps) {
            const float s = rmin / r[c];
            for (int k = 0; k < 3; k++) r[k] = r[k] * s;
        }
    }
    float pv[2];
    pb.apply<2>(pv);
    const float vx = pv[0] + vel.x, vy = pv[1] + vel.y;
    const float vlen = sqrtf(vx * vx + vy * vy);
    const float dis = fminf(fmaxf((vlen - 0.001f) * 10.0f, 0.0f), 1.0f);
    float fin[3];
    for (int c = 0; c < 3; c++) {
        const float hc = p[c] + r[c];
        const float f = cur[c] * (1.0f - 0.9f) + hc * 0.9f;
        fin[c] = f * (1.0f - dis) + mu[c] * dis;
    }
    const float4 o = make_float4(fin[0], fin[1], fin[2], 1.0f);
    if (I.out) I.out[pix] = o;
    I.hist_next[pix] = o;
    I.pmot_next[pix] = vel;
}

}  // namespace
}  // namespace snk

using namespace snk;

struct snk_taa {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    uint32_t w = 0, h = 0;
    DBuf<float4> hist[2];
    DBuf<float2> pmot[2];
    DBuf<float4> stage_in, stage_out;
    DBuf<float2> stage_motion;
    int cur = 0;
    bool valid = false;
    std::string err;
};

namespace {
int taa_fail(snk_taa* t, int code, const std::string& msg) {
    if (t) t->err = msg;
    return code;
}
}  // namespace

extern "C" {

int snk_taa_create(int32_t device, void* stream, uint32_t width, uint32_t height, snk_taa** out) {
    if (!out || width == 0 || height == 0 || (uint64_t)width * height > (1ull << 30)) return SNK_ERR_INVALID_ARG;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return SNK_ERR_CUDA;
    snk_taa* t = new snk_taa();
    t->device = device;
    t->w = width;
    t->h = height;
    if (stream) {
        t->stream = (cudaStream_t)stream;
    } else {
        if (cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking) != cudaSuccess) { delete t; return SNK_ERR_CUDA; }
        t->own_stream = true;
    }
    const size_t np = (size_t)width * height;
    for (int k = 0; k < 2; k++)
        if (t->hist[k].reserve(np) != cudaSuccess || t->pmot[k].reserve(np) != cudaSuccess) {
            if (t->own_stream) cudaStreamDestroy(t->stream);
            delete t;
            return SNK_ERR_OUT_OF_MEMORY;
        }
    *out = t;
    return SNK_OK;
}

int snk_taa_destroy(snk_taa* t) {
    if (!t) return SNK_OK;
    cudaSetDevice(t->device);
    cudaStreamSynchronize(t->stream);
    if (t->own_stream) cudaStreamDestroy(t->stream);
    delete t;
    return SNK_OK;
}

int snk_taa_reset(snk_taa* t) {
    if (!t) return SNK_ERR_INVALID_ARG;
    t->valid = false;
    return SNK_OK;
}

int snk_taa_resolve(snk_taa* t, const float* radiance, const float* motion, float* out, uint32_t memory) {
    if (!t || !radiance || !motion || !out || memory > SNK_MEM_HOST)
        return taa_fail(t, SNK_ERR_INVALID_ARG, "taa_resolve: bad arguments");
    if (cudaSetDevice(t->device) != cudaSuccess) return taa_fail(t, SNK_ERR_CUDA, "taa_resolve: device");
    const size_t np = (size_t)t->w * t->h;
    cudaStream_t st = t->stream;
    const float4* cur = reinterpret_cast<const float4*>(radiance);
    const float2* mot = reinterpret_cast<const float2*>(motion);
    if (memory == SNK_MEM_HOST) {
        if (t->stage_in.reserve(np) || t->stage_motion.reserve(np))
            return taa_fail(t, SNK_ERR_OUT_OF_MEMORY, "taa_resolve: staging");
        if (cudaMemcpyAsync(t->stage_in.p, radiance, np * sizeof(float4), cudaMemcpyHostToDevice, st) ||
            cudaMemcpyAsync(t->stage_motion.p, motion, np * sizeof(float2), cudaMemcpyHostToDevice, st))
            return taa_fail(t, SNK_ERR_CUDA, "taa_resolve: upload");
        cur = t->stage_in.p;
        mot = t->stage_motion.p;
    } else if (reinterpret_cast<uintptr_t>(radiance) % 16 || reinterpret_cast<uintptr_t>(motion) % 8 ||
               reinterpret_cast<uintptr_t>(out) % 16) {
        return taa_fail(t, SNK_ERR_INVALID_ARG, "taa_resolve: device buffers must be 16-byte (radiance, out) "
                                                "and 8-byte (motion) aligned");
    }
    const int nxt = t->cur ^ 1;
    if (!t->valid) {
        // first frame: the history is the current frame, the previous motion this frame's
        if (cudaMemcpyAsync(t->hist[t->cur].p, cur, np * sizeof(float4), cudaMemcpyDeviceToDevice, st) ||
            cudaMemcpyAsync(t->pmot[t->cur].p, mot, np * sizeof(float2), cudaMemcpyDeviceToDevice, st))
            return taa_fail(t, SNK_ERR_CUDA, "taa_resolve: history seed");
    }
    TaaImages I;
    I.cur = cur;
    I.motion = mot;
    I.hist = t->hist[t->cur].p;
    I.pmot = t->pmot[t->cur].p;
    // in place (or host output): write the history only, then copy it out
    const bool direct = memory == SNK_MEM_DEVICE && out != radiance;
    I.out = direct ? reinterpret_cast<float4*>(out) : nullptr;
    I.hist_next = t->hist[nxt].p;
    I.pmot_next = t->pmot[nxt].p;
    I.w = (int)t->w;
    I.h = (int)t->h;
    dim3 grid((t->w + TX - 1) / TX, (t->h + TY - 1) / TY);
    k_taa_resolve<<<grid, dim3(TX, TY), 0, st>>>(I);
    if (cudaGetLastError() != cudaSuccess) return taa_fail(t, SNK_ERR_CUDA, "taa_resolve: launch");
    if (!direct) {
        if (cudaMemcpyAsync(out, t->hist[nxt].p, np * sizeof(float4),
                            memory == SNK_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, st))
            return taa_fail(t, SNK_ERR_CUDA, "taa_resolve: copy out");
    }
    if (memory == SNK_MEM_HOST && cudaStreamSynchronize(st) != cudaSuccess)
        return taa_fail(t, SNK_ERR_CUDA, "taa_resolve: synchronise");
    t->cur = nxt;
    t->valid = true;
    return SNK_OK;
}

int snk_taa_get_last_error(const snk_taa* t, char* buf, size_t len) {
    if (!t || !buf || len == 0) return SNK_ERR_INVALID_ARG;
    std::strncpy(buf, t->err.c_str(), len - 1);
    buf[len - 1] = 0;
    return SNK_OK;
}

}  // extern "C"
