// Radiance-cache network: tiny-cuda-nn style config, parameters and the
// FP32 kernels.  Replaces TINY_MLP (cuda_headers/neural_network.cuh:33-50,
// cuda/neural_network.cu:17-64) and the tiny-cuda-nn objects it owns
// (NetworkWithInputEncoding, Trainer, Adam/ExponentialDecay, loss).
//
// Semantics follow tiny-cuda-nn's documented behaviour (the library is an
// absent submodule of the reference, so its source cannot be consulted):
//  * encodings Identity / Frequency / OneBlob (quartic kernel, periodic on
//    [0,1)) / HashGrid (multiresolution hash, Mueller et al. 2022) combined by
//    Composite in input order; the encoded width is padded to a multiple of
//    16 with ones (the padding acts as a learnable bias: the MLP has none);
//  * FullyFusedMLP: n_hidden_layers ReLU layers of n_neurons, a linear output
//    layer padded to 16 outputs, weights row-major [out][in], network
//    parameters first and encoding parameters after them;
//  * losses L2, RelativeL2, RelativeL2Luminance (gradient through the
//    numerator only), averaged over batch x output dims;
//  * Adam with l2_reg on the matrix weights only and sparse updates (zero
//    gradient => untouched) of encoding parameters, wrapped by
//    ExponentialDecay.
#pragma once
#include <string>
#include <vector>

#include "hm_common.cuh"

namespace hm {

enum EncType { ENC_IDENTITY = 0, ENC_FREQUENCY = 1, ENC_ONEBLOB = 2, ENC_HASHGRID = 3 };
// LOSS_OUTPUT_GRAD: the "target" is dL/d(output) itself (tcnn's backward
// with dL_doutput), used as the output gradient unscaled.
enum LossType { LOSS_L2 = 0, LOSS_REL_L2 = 1, LOSS_REL_L2_LUM = 2, LOSS_OUTPUT_GRAD = 3 };
enum Activation { ACT_NONE = 0, ACT_RELU = 1 };

constexpr int kMaxSegs = 8;
constexpr int kMaxLevels = 24;

struct EncSeg {
  int type;
  int in_off, n_dims;   // consumed input dims
  int out_off, n_out;   // produced features
  int n_freq;           // Frequency
  int n_bins;           // OneBlob
  // HashGrid
  int n_levels, n_feat, base_res;
  float log2_scale;     // log2(per_level_scale)
  int64_t param_off;    // offset of this grid's table inside the encoding params
  uint32_t level_size[kMaxLevels];    // table entries per level
  uint32_t level_res[kMaxLevels];     // grid resolution per level
  float level_scale[kMaxLevels];      // position scale per level
  uint32_t level_off[kMaxLevels];     // entry offset per level
};

struct MlpDims {
  int in_ch, out_ch;
  int n_enc;      // encoded features before padding
  int in_pad;     // encoded width padded to 16
  int width;      // n_neurons
  int n_hidden;   // n_hidden_layers
  int out_pad;    // output width padded to 16
  int n_segs;
  EncSeg segs[kMaxSegs];
  int activation, output_activation;
  int64_t n_net_params;  // matrix weights
  int64_t n_enc_params;  // hash tables
  int64_t layer_off[16]; // offset of each weight matrix (layer 0..n_hidden)
};

struct AdamCfg {
  float lr, beta1, beta2, eps, l2_reg;
  int decay_start, decay_interval;
  float decay_base;
};

struct MlpConfig {
  MlpDims d;
  AdamCfg adam;
  int loss;
  std::string init;  // "xavier_uniform" (tcnn default) or "he_normal"
};

// Parses a tcnn-style JSON config (loss / optimizer / encoding / network).
MlpConfig mlp_config_from_json(const char* text, int in_ch, int out_ch);


// ---- encoding helpers shared by the FP32 and tensor-core kernels
// OneBlob quartic-kernel CDF with radius one bin (inv_radius = n_bins).
HM_D float quartic_cdf(float x, float inv_radius) {
  float u = x * inv_radius;
  float u2 = u * u;
  float u4 = u2 * u2;
  return fminf(fmaxf((1.0f / 16.0f) * u * (15.0f - 10.0f * u2 + 3.0f * u4) + 0.5f, 0.f), 1.f);
}
// Periodic (on [0,1)) cumulative mass left of `boundary` for a blob at x.
HM_D float oneblob_cdf(float boundary, float x, float nb) {
  return quartic_cdf(boundary - x, nb) + quartic_cdf(boundary - x - 1.0f, nb) +
         quartic_cdf(boundary - x + 1.0f, nb);
}

HM_D uint32_t grid_index(const EncSeg& s, int l, uint32_t x, uint32_t y, uint32_t z) {
  const uint32_t size = s.level_size[l], res = s.level_res[l];
  uint32_t stride = 1, index = 0;
  index += x * stride;
  stride *= res;
  if (stride <= size) {
    index += y * stride;
    stride *= res;
    if (stride <= size) {
      index += z * stride;
      stride *= res;
    }
  }
  if (size < stride) index = (x * 1u) ^ (y * 2654435761u) ^ (z * 805459861u);
  return index % size;
}


// Loss gradient of one query (tcnn semantics, averaged over n * out_ch).
HM_D void loss_grad(int loss, const float* pred, const float* tgt, int out_ch, float inv_total,
                    float* grad, float* value) {
  if (loss == LOSS_OUTPUT_GRAD) {
    for (int o = 0; o < out_ch; ++o) grad[o] = tgt[o];
    *value = 0.f;
    return;
  }
  float lum2 = 0.f;
  if (loss == LOSS_REL_L2_LUM) {
    float lum = 0.299f * pred[0] + 0.587f * pred[1] + 0.114f * pred[2];
    lum2 = lum * lum + 0.01f;
  }
  float v = 0.f;
  for (int o = 0; o < out_ch; ++o) {
    float diff = pred[o] - tgt[o];
    float den = loss == LOSS_L2 ? 1.f : (loss == LOSS_REL_L2 ? pred[o] * pred[o] + 0.01f : lum2);
    v += diff * diff / den * inv_total;
    grad[o] = 2.f * diff / den * inv_total;
  }
  *value = v;
}

// ---- tensor-core (tcgen05) forward for HM_PREC_FP16 / BF16 / FP8_E4M3
// Weights are repacked from the FP32 master copy into the operand layout of
// the MMA (K-major, 8-row x 16-byte core matrices) whenever they change.
struct TcPack {
  int precision = 0;
  int elem_bytes = 2;
  int kinst = 16;           // K of one MMA instruction (elements)
  int n_layers = 0;         // hidden layers + output
  int N[16], K[16];         // per layer: output rows, padded input columns
  int64_t boff[16];         // byte offset of each layer in the blob
  int64_t bytes = 0;
  uint8_t* blob = nullptr;  // device
  float* scales = nullptr;  // device [16]: 1/weight scale per layer; [15]: hash-grid amax
  // training (FP16 / BF16 only): the transposed matrices W_l^T as B operands
  // of the backward pass (rows = layer inputs, K = layer outputs)
  int NT[16], KT[16];
  int64_t boff_t[16];
  int64_t bytes_t = 0;
  uint8_t* blob_t = nullptr;
};

// Device buffers of a tensor-core training step (batch capacity rows).
struct TcTrainBufs {
  uint16_t* x16 = nullptr;   // [cap][K0] encoded inputs as rounded for layer 0
  uint16_t* h16 = nullptr;   // [L][cap][W] hidden activations
  uint16_t* dz16 = nullptr;  // [L+1][cap][max(W,16)] loss-scaled dZ per layer
  float* pred = nullptr;     // [cap][16]
  float* dX = nullptr;       // [cap][in_pad] loss-scaled input gradient (hash grids only)
  float* loss_part = nullptr;
  int64_t cap = 0;
};

// Whether the tensor-core path covers this network at this precision.
bool tc_supported(const MlpDims& d, int precision, std::string* why);
// Layout, allocation (once) and repacking of the weights.
int tc_pack_alloc(const MlpDims& d, int precision, TcPack* pk);
int tc_pack(const MlpDims& d, const float* params, TcPack& pk, cudaStream_t st);
void tc_pack_free(TcPack* pk);
// Encoding + all layers of n queries on the tensor cores: in [n][in_ch],
// out [n][out_stride] (the first out_ch columns written).  Three forms, the
// same bits: the warp-specialised kernel (16-bit operands, width 32 / 64:
// encoder warps and layer warps overlapped in one CTA per SM, no
// workspace); with a workspace of at least tc_encode_bytes, the encode
// kernel and then the layer kernel loading its input tiles by bulk copies
// (networks with a hash grid, E4M3, width 128); without one, the layer
// kernel encoding its own tiles.
int64_t tc_encode_bytes(const MlpDims& d, const TcPack& pk, int64_t n);
// Whether tc_forward would use a workspace (false where the warp-specialised
// kernel runs: no encoded operands in device memory).
bool tc_wants_workspace(const MlpDims& d, const TcPack& pk);
int tc_forward(const MlpDims& d, const TcPack& pk, const float* enc_params, const float* in, float* out,
               int out_stride, int64_t n, int* err_flag, cudaStream_t st, uint8_t* work = nullptr,
               int64_t work_bytes = 0);
// Training on the tensor cores (FP16 / BF16): forward keeping the operands,
// backward (loss gradient scaled by loss_scale, dgrad chain, dX when the
// encoding has parameters), weight gradients as per-chunk partials reduced
// in a fixed order into grads (still scaled by loss_scale).
bool tc_trainable(const MlpDims& d, int precision);
int tc_train_alloc(const MlpDims& d, int64_t cap, bool need_dx, TcTrainBufs* b);
void tc_train_free(TcTrainBufs* b);
int tc_train_forward(const MlpDims& d, const TcPack& pk, const float* enc_params, const float* in, int64_t n,
                     const TcTrainBufs& b, int* err_flag, cudaStream_t st);
int tc_backward(const MlpDims& d, const TcPack& pk, const TcTrainBufs& b, const float* target, int loss,
                float loss_scale, int64_t n, float* loss_out, float* grads, float** dw_part, int64_t* dw_cap,
                int* err_flag, cudaStream_t st);

}  // namespace hm
