// snk_mlp.h -- MLP radiance cache: sizes, weight layouts and host entry points.
#pragma once
#include <cmath>
#include <vector>

#include "snk_host.h"

namespace snk {

constexpr int MLP_NW = 4 * 64 * 64 + 64 * 3;   // master weights (FP32)
// master weight offset of layer l (W_l[in][out], row major)
#define MLP_OFF(l) ((l) * 4096)
// BF16 copy in the tcgen05 shared-memory operand layout (K-major, no swizzle: 8x8
// core matrices of 128 contiguous bytes): layer l < 4 as N = 64 outputs x K = 64
// inputs at element offset l * 4096, layer 4 as N = 16 (3 outputs + 13 zero rows)
// x K = 64 at 4 * 4096
constexpr int MLP_TC_ELEMS = 4 * 4096 + 16 * 64;
// BF16 transposed copy in the same layout, for the input-gradient GEMMs: layer
// l = 1..4 as N = 64 inputs x K = 64 outputs at element offset (l - 1) * 4096
// (layer 4: outputs 0..2, zero beyond)
constexpr int MLP_TCB_ELEMS = 4 * 4096;

struct EncodeParams {
    float lo[3];        // scene box the positions are normalised to
    float inv_ext[3];
};

struct AdamParams {
    float lr, b1, b2, eps, c1, c2;   // c1, c2: bias corrections 1 - b^step
};

struct MlpState {
    DBuf<float> w, m, v;             // FP32 master weights and Adam moments
    DBuf<unsigned short> wtc, wtcb;  // BF16 forward / transposed copies in the tcgen05 operand layout
    DBuf<float> part, loss;          // per-CTA gradient partials and losses
    uint32_t step = 0;
    bool ready = false;
};

Status mlp_init(MlpState& M, const float* w_host, cudaStream_t st);
// records: 4 float4 per query (position+roughness, direction+metallic, normal, albedo+path id)
// (tcgen05 kernel; a give-up of its bounded tensor-core waits sets bit 16 of *err_word)
Status mlp_infer(const MlpState& M, const float4* rec, const uint32_t* n_dev, uint32_t n, const EncodeParams& ep,
                 float* out, const float4* beta, float4* L, int grid, unsigned* err_word, cudaStream_t st);
Status mlp_encode(const float4* rec, uint32_t n, const EncodeParams& ep, float* out, cudaStream_t st);
// samples: 5 float4 each (the 4 record words, then target rgb + weight)
// grows the per-CTA gradient/loss buffers for batches of up to n samples (call
// before a stream capture: the training step itself then allocates nothing);
// a give-up of the training kernel's bounded tensor-core waits sets bit 16 of *err_word
Status mlp_train_reserve(MlpState& M, uint32_t n);
Status mlp_train_step(MlpState& M, const float4* samples, uint32_t n, const EncodeParams& ep, float lr,
                      float* grad_out, float* loss_host, unsigned* err_word, cudaStream_t st);

}  // namespace snk
