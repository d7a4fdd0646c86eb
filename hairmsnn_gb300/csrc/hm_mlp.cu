// Radiance-cache network (see hm_mlp.cuh for the semantics) — FP32 path.
//
// Per batch:
//   encode_kernel      inputs [n][in_ch] -> encoded X [n][in_pad] (pad = 1)
//   mlp_fwd_kernel     fused: all layers of a 64-query tile in shared memory,
//                      register-blocked SIMT GEMMs; optionally stores every
//                      hidden activation for the backward pass
//   mlp_bwd_kernel     fused: loss gradient + back-propagation of one tile,
//                      stores dZ of every layer (and dX when the encoding
//                      has parameters)
//   dw_partial_kernel  weight gradients dW_l = dZ_{l+1}^T H_l, split over the
//                      batch into fixed chunks -> partial tiles
//   adam_kernel        sums the partial tiles in a fixed order (bitwise
//                      reproducible), adds l2, updates moments and weights
//   grid_bwd_kernel    hash-grid gradient scatter (float atomics)
#include <math.h>
#include <stdio.h>
#include <ctype.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "hm_json.h"
#include "hm_mlp.cuh"

namespace hm {

// ====================================================================== config
static int pad16(int x) { return (x + 15) / 16 * 16; }

MlpConfig mlp_config_from_json(const char* text, int in_ch, int out_ch) {
  Json j = json_parse(text);
  MlpConfig c{};
  MlpDims& d = c.d;
  d.in_ch = in_ch;
  d.out_ch = out_ch;
  if (in_ch <= 0 || out_ch <= 0 || out_ch > 16) throw JsonError("mlp: bad in/out channel count");

  // ---- loss
  std::string loss = j["loss"].string_or("otype", "L2");
  if (loss == "L2") c.loss = LOSS_L2;
  else if (loss == "RelativeL2") c.loss = LOSS_REL_L2;
  else if (loss == "RelativeL2Luminance") c.loss = LOSS_REL_L2_LUM;
  else throw JsonError("mlp: unsupported loss " + loss);
  if (c.loss == LOSS_REL_L2_LUM && out_ch < 3) throw JsonError("mlp: luminance loss needs 3 outputs");

  // ---- optimizer (optionally wrapped in ExponentialDecay)
  const Json* opt = &j["optimizer"];
  c.adam.decay_start = 1 << 30;
  c.adam.decay_interval = 1 << 30;
  c.adam.decay_base = 1.f;
  if (opt->string_or("otype", "Adam") == "ExponentialDecay") {
    c.adam.decay_start = (int)opt->number_or("decay_start", 10000);
    c.adam.decay_interval = (int)opt->number_or("decay_interval", 10000);
    c.adam.decay_base = (float)opt->number_or("decay_base", 0.33);
    opt = &(*opt)["nested"];
  }
  std::string ot = opt->string_or("otype", "Adam");
  if (ot != "Adam") throw JsonError("mlp: unsupported optimizer " + ot);
  c.adam.lr = (float)opt->number_or("learning_rate", 1e-3);
  c.adam.beta1 = (float)opt->number_or("beta1", 0.9);
  c.adam.beta2 = (float)opt->number_or("beta2", 0.999);
  c.adam.eps = (float)opt->number_or("epsilon", 1e-8);
  c.adam.l2_reg = (float)opt->number_or("l2_reg", 1e-8);

  // ---- encoding
  const Json& enc = j["encoding"];
  std::vector<const Json*> parts;
  std::string et = enc.string_or("otype", "Identity");
  if (et == "Composite") {
    for (size_t i = 0; i < enc["nested"].size(); ++i) parts.push_back(&enc["nested"][i]);
  } else {
    parts.push_back(&enc);
  }
  if (parts.empty() || parts.size() > (size_t)kMaxSegs) throw JsonError("mlp: bad encoding list");
  int in_off = 0, out_off = 0;
  int64_t enc_params = 0;
  d.n_segs = 0;
  for (size_t pi = 0; pi < parts.size(); ++pi) {
    const Json& e = *parts[pi];
    EncSeg s{};
    std::string t = e.string_or("otype", "Identity");
    int rest = in_ch - in_off;
    s.n_dims = e.has("n_dims_to_encode") ? (int)e["n_dims_to_encode"].as_number() : rest;
    if (s.n_dims < 0 || s.n_dims > rest) throw JsonError("mlp: n_dims_to_encode exceeds the input");
    if (s.n_dims == 0) continue;
    s.in_off = in_off;
    s.out_off = out_off;
    if (t == "Identity") {
      s.type = ENC_IDENTITY;
      s.n_out = s.n_dims;
    } else if (t == "Frequency") {
      s.type = ENC_FREQUENCY;
      s.n_freq = (int)e.number_or("n_frequencies", 12);
      s.n_out = s.n_dims * s.n_freq * 2;
    } else if (t == "OneBlob") {
      s.type = ENC_ONEBLOB;
      s.n_bins = (int)e.number_or("n_bins", 16);
      if (s.n_bins < 2) throw JsonError("mlp: OneBlob needs n_bins >= 2");
      s.n_out = s.n_dims * s.n_bins;
    } else if (t == "HashGrid" || t == "Grid") {
      if (t == "Grid" && e.string_or("type", "Hash") != "Hash") throw JsonError("mlp: only hash grids");
      s.type = ENC_HASHGRID;
      if (s.n_dims != 3) throw JsonError("mlp: HashGrid supports 3 input dims");
      s.n_levels = (int)e.number_or("n_levels", 16);
      s.n_feat = (int)e.number_or("n_features_per_level", 2);
      int log2_T = (int)e.number_or("log2_hashmap_size", 19);
      s.base_res = (int)e.number_or("base_resolution", 16);
      float pls = (float)e.number_or("per_level_scale", 2.0);
      if (s.n_levels < 1 || s.n_levels > kMaxLevels || s.n_feat < 1 || s.n_feat > 8 || log2_T < 4 ||
          log2_T > 26)
        throw JsonError("mlp: bad HashGrid parameters");
      s.log2_scale = log2f(pls);
      uint32_t off = 0;
      for (int l = 0; l < s.n_levels; ++l) {
        // scale = base * per_level_scale^l - 1, resolution = ceil(scale) + 1
        float scale = exp2f((float)l * s.log2_scale) * (float)s.base_res - 1.f;
        uint32_t res = (uint32_t)ceilf(scale) + 1;
        double dense = (double)res * res * res;
        uint64_t size = std::min<uint64_t>(1ull << log2_T, ((uint64_t)std::min(dense, 1e18) + 7) / 8 * 8);
        s.level_scale[l] = scale;
        s.level_res[l] = res;
        s.level_size[l] = (uint32_t)size;
        s.level_off[l] = off;
        off += (uint32_t)size;
      }
      s.param_off = enc_params;
      enc_params += (int64_t)off * s.n_feat;
      s.n_out = s.n_levels * s.n_feat;
    } else {
      throw JsonError("mlp: unsupported encoding " + t);
    }
    in_off += s.n_dims;
    out_off += s.n_out;
    d.segs[d.n_segs++] = s;
  }
  if (in_off != in_ch) throw JsonError("mlp: encoding does not consume every input dim");
  d.n_enc = out_off;
  d.in_pad = pad16(out_off);
  d.n_enc_params = enc_params;

  // ---- network
  const Json& net = j["network"];
  std::string nt = net.string_or("otype", "FullyFusedMLP");
  if (nt != "FullyFusedMLP" && nt != "CutlassMLP") throw JsonError("mlp: unsupported network " + nt);
  d.width = (int)net.number_or("n_neurons", 64);
  d.n_hidden = (int)net.number_or("n_hidden_layers", 2);
  if (!(d.width == 16 || d.width == 32 || d.width == 64 || d.width == 128))
    throw JsonError("mlp: n_neurons must be 16, 32, 64 or 128");
  if (d.n_hidden < 1 || d.n_hidden > 14) throw JsonError("mlp: n_hidden_layers must be 1..14");
  std::string act = net.string_or("activation", "ReLU");
  std::string oact = net.string_or("output_activation", "None");
  if (act != "ReLU") throw JsonError("mlp: only ReLU hidden activation");
  if (oact != "None") throw JsonError("mlp: only linear output");
  d.activation = ACT_RELU;
  d.output_activation = ACT_NONE;
  d.out_pad = 16;
  int64_t off = 0;
  for (int l = 0; l <= d.n_hidden; ++l) {
    int fan_in = l == 0 ? d.in_pad : d.width;
    int fan_out = l == d.n_hidden ? d.out_pad : d.width;
    d.layer_off[l] = off;
    off += (int64_t)fan_in * fan_out;
  }
  d.n_net_params = off;
  c.init = net.string_or("init", "xavier_uniform");
  if (c.init != "xavier_uniform" && c.init != "he_normal") throw JsonError("mlp: unknown init " + c.init);
  return c;
}

// ====================================================================== encoding
__constant__ MlpDims c_dims[1];

// One thread per (query, encoded feature group): writes X[q][*].
__global__ void __launch_bounds__(256) encode_kernel(const float* __restrict__ in, const float* __restrict__ enc_params,
                                                     float* __restrict__ X, int64_t n) {
  const MlpDims& d = c_dims[0];
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= n) return;
  const float* xin = in + q * d.in_ch;
  float* xo = X + q * d.in_pad;
  for (int si = 0; si < d.n_segs; ++si) {
    const EncSeg& s = d.segs[si];
    if (s.type == ENC_IDENTITY) {
      for (int k = 0; k < s.n_dims; ++k) xo[s.out_off + k] = xin[s.in_off + k];
    } else if (s.type == ENC_FREQUENCY) {
      for (int k = 0; k < s.n_dims; ++k) {
        float x = xin[s.in_off + k];
        for (int f = 0; f < s.n_freq; ++f) {
          float a = ldexpf(x, f) * kPi;
          xo[s.out_off + (k * s.n_freq + f) * 2 + 0] = sinf(a);
          xo[s.out_off + (k * s.n_freq + f) * 2 + 1] = sinf(a + 0.5f * kPi);
        }
      }
    } else if (s.type == ENC_ONEBLOB) {
      const float nb = (float)s.n_bins;
      for (int k = 0; k < s.n_dims; ++k) {
        float x = xin[s.in_off + k];
        float c0 = oneblob_cdf(0.f, x, nb);
        float left = c0;
        for (int b = 0; b < s.n_bins; ++b) {
          float right = (b == s.n_bins - 1) ? c0 + 1.f : oneblob_cdf((float)(b + 1) / nb, x, nb);
          xo[s.out_off + k * s.n_bins + b] = right - left;
          left = right;
        }
      }
    } else {  // hash grid, 3 dims
      const float* table = enc_params + s.param_off;
      float px = xin[s.in_off], py = xin[s.in_off + 1], pz = xin[s.in_off + 2];
      for (int l = 0; l < s.n_levels; ++l) {
        const float sc = s.level_scale[l];
        float fx = fmaf(sc, px, 0.5f), fy = fmaf(sc, py, 0.5f), fz = fmaf(sc, pz, 0.5f);
        float gx = floorf(fx), gy = floorf(fy), gz = floorf(fz);
        float wx = fx - gx, wy = fy - gy, wz = fz - gz;
        uint32_t ix = (uint32_t)(int)gx, iy = (uint32_t)(int)gy, iz = (uint32_t)(int)gz;
        float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int c = 0; c < 8; ++c) {
          uint32_t cx = ix + (c & 1), cy = iy + ((c >> 1) & 1), cz = iz + ((c >> 2) & 1);
          float w = ((c & 1) ? wx : 1.f - wx) * (((c >> 1) & 1) ? wy : 1.f - wy) * (((c >> 2) & 1) ? wz : 1.f - wz);
          uint32_t e = s.level_off[l] + grid_index(s, l, cx, cy, cz);
          const float* v = table + (int64_t)e * s.n_feat;
          for (int f = 0; f < s.n_feat; ++f) acc[f] += w * __ldg(v + f);
        }
        for (int f = 0; f < s.n_feat; ++f) xo[s.out_off + l * s.n_feat + f] = acc[f];
      }
    }
  }
  for (int k = d.n_enc; k < d.in_pad; ++k) xo[k] = 1.f;
}

// Hash-grid gradients are scattered as 64-bit fixed-point integers (2^-40
// resolution, range +-2^23): integer addition is associative, so the sum does
// not depend on the order the atomics land in and training stays bitwise
// reproducible.
constexpr double kGridFix = 1099511627776.0;  // 2^40

__global__ void grid_fix_to_float_kernel(const long long* __restrict__ acc, float* __restrict__ out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (float)((double)acc[i] * (1.0 / kGridFix));
}

// Hash-grid backward: dX columns of the grid features -> table gradients.
__global__ void __launch_bounds__(256) grid_bwd_kernel(const float* __restrict__ in, const float* __restrict__ dX,
                                                       long long* __restrict__ enc_grad, int64_t n) {
  const MlpDims& d = c_dims[0];
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= n) return;
  const float* xin = in + q * d.in_ch;
  const float* g = dX + q * d.in_pad;
  for (int si = 0; si < d.n_segs; ++si) {
    const EncSeg& s = d.segs[si];
    if (s.type != ENC_HASHGRID) continue;
    long long* tg = enc_grad + s.param_off;
    float px = xin[s.in_off], py = xin[s.in_off + 1], pz = xin[s.in_off + 2];
    for (int l = 0; l < s.n_levels; ++l) {
      const float sc = s.level_scale[l];
      float fx = fmaf(sc, px, 0.5f), fy = fmaf(sc, py, 0.5f), fz = fmaf(sc, pz, 0.5f);
      float gx = floorf(fx), gy = floorf(fy), gz = floorf(fz);
      float wx = fx - gx, wy = fy - gy, wz = fz - gz;
      uint32_t ix = (uint32_t)(int)gx, iy = (uint32_t)(int)gy, iz = (uint32_t)(int)gz;
      for (int c = 0; c < 8; ++c) {
        uint32_t cx = ix + (c & 1), cy = iy + ((c >> 1) & 1), cz = iz + ((c >> 2) & 1);
        float w = ((c & 1) ? wx : 1.f - wx) * (((c >> 1) & 1) ? wy : 1.f - wy) * (((c >> 2) & 1) ? wz : 1.f - wz);
        uint32_t e = s.level_off[l] + grid_index(s, l, cx, cy, cz);
        for (int f = 0; f < s.n_feat; ++f) {
          float gv = g[s.out_off + l * s.n_feat + f];
          if (gv != 0.f) {
            const long long q = __double2ll_rn((double)(w * gv) * kGridFix);
            if (q != 0) atomicAdd((unsigned long long*)(tg + (int64_t)e * s.n_feat + f), (unsigned long long)q);
          }
        }
      }
    }
  }
}

// ====================================================================== fused MLP (FP32 SIMT)
// Tile: BM = 64 queries x N outputs per layer, 256 threads, each thread a
// TQ x TO register block.  Activations live in shared memory k-major
// (H[k][q], q contiguous) so both GEMM operands load as float4.
constexpr int BM = 64;
constexpr int KC = 32;  // K chunk staged per step
constexpr int APAD = 4; // row padding (floats) of k-major activation tiles

template <int N>
struct TileShape {
  static constexpr int TO = N >= 64 ? (N / 16) : (N >= 32 ? 2 : 1);  // outputs per thread
  static constexpr int NT_O = N / TO;                                 // threads along outputs
  static constexpr int NT_Q = 256 / NT_O;                             // threads along queries
  static constexpr int TQ = BM / NT_Q;                                // queries per thread
  static_assert(NT_O * NT_Q == 256 && TQ * NT_Q == BM, "tile");
};

// acc[TQ][TO] += A[BM x K] * B[K x N] where A is k-major in smem
// (AT[k * lda + q]) and B is read from global W (row-major [rows][cols]):
//   trans_w = false: B[k][o] = W[o][k]   (forward:  y = W x)
//   trans_w = true : B[k][o] = W[k][o]   (backward: dx = W^T dy)
template <int N, bool TRANS_W>
__device__ __forceinline__ void tile_gemm(const float* __restrict__ AT, int lda, int K,
                                          const float* __restrict__ W, int w_cols, float* Bs,
                                          float (&acc)[TileShape<N>::TQ][TileShape<N>::TO]) {
  using S = TileShape<N>;
  const int tid = threadIdx.x;
  const int to = tid % S::NT_O, tq = tid / S::NT_O;
  constexpr int BLD = N + 4;
  for (int k0 = 0; k0 < K; k0 += KC) {
    const int kc = min(KC, K - k0);
    __syncthreads();
    for (int i = tid; i < KC * N; i += 256) {
      int kk, o;
      float v = 0.f;
      if (!TRANS_W) {  // coalesced along k in W's rows
        o = i / KC;
        kk = i % KC;
        if (kk < kc) v = __ldg(W + (int64_t)o * w_cols + k0 + kk);
      } else {         // coalesced along o in W's rows
        kk = i / N;
        o = i % N;
        if (kk < kc) v = __ldg(W + (int64_t)(k0 + kk) * w_cols + o);
      }
      Bs[kk * BLD + o] = v;
    }
    __syncthreads();
    for (int kk = 0; kk < kc; ++kk) {
      float a[S::TQ], b[S::TO];
#pragma unroll
      for (int i = 0; i < S::TQ; ++i) a[i] = AT[(k0 + kk) * lda + tq * S::TQ + i];
#pragma unroll
      for (int j = 0; j < S::TO; ++j) b[j] = Bs[kk * BLD + to * S::TO + j];
#pragma unroll
      for (int i = 0; i < S::TQ; ++i)
#pragma unroll
        for (int j = 0; j < S::TO; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
  }
}

template <int N>
__device__ __forceinline__ void zero_acc(float (&acc)[TileShape<N>::TQ][TileShape<N>::TO]) {
#pragma unroll
  for (int i = 0; i < TileShape<N>::TQ; ++i)
#pragma unroll
    for (int j = 0; j < TileShape<N>::TO; ++j) acc[i][j] = 0.f;
}

// Load a [BM x cols] row-major tile of a global matrix into k-major smem.
__device__ __forceinline__ void load_kmajor(const float* __restrict__ G, int64_t q0, int64_t n, int cols,
                                            float* T, int lda) {
  for (int i = threadIdx.x; i < BM * cols; i += blockDim.x) {
    int q = i / cols, k = i % cols;
    float v = (q0 + q < n) ? __ldg(G + (q0 + q) * cols + k) : 0.f;
    T[k * lda + q] = v;
  }
}

template <int W>
__global__ void __launch_bounds__(256) mlp_fwd_kernel(const float* __restrict__ X, const float* __restrict__ params,
                                                      float* __restrict__ out, int out_stride,
                                                      float* __restrict__ acts, int64_t n) {
  using S = TileShape<W>;
  using SO = TileShape<16>;
  const MlpDims& d = c_dims[0];
  extern __shared__ float smem[];
  const int lda_in = BM + APAD;
  float* XT = smem;                                     // [in_pad][lda]
  float* H0 = XT + d.in_pad * lda_in;                   // [W][lda]
  float* H1 = H0 + W * lda_in;                          // [W][lda]
  float* Bs = H1 + W * lda_in;                          // [KC][W+4]
  const int64_t q0 = (int64_t)blockIdx.x * BM;
  load_kmajor(X, q0, n, d.in_pad, XT, lda_in);
  const int to = threadIdx.x % S::NT_O, tq = threadIdx.x / S::NT_O;

  const float* A = XT;
  int K = d.in_pad;
  float* Hout = H0;
  for (int l = 0; l < d.n_hidden; ++l) {
    float acc[S::TQ][S::TO];
    zero_acc<W>(acc);
    tile_gemm<W, false>(A, lda_in, K, params + d.layer_off[l], K, Bs, acc);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < S::TQ; ++i)
#pragma unroll
      for (int j = 0; j < S::TO; ++j) Hout[(to * S::TO + j) * lda_in + tq * S::TQ + i] = fmaxf(acc[i][j], 0.f);
    __syncthreads();
    if (acts) {  // store h_{l+1} as [n][W] row-major
      float* dst = acts + (int64_t)l * n * W;
      for (int i = threadIdx.x; i < BM * W; i += 256) {
        int q = i / W, k = i % W;
        if (q0 + q < n) dst[(q0 + q) * W + k] = Hout[k * lda_in + q];
      }
    }
    A = Hout;
    K = W;
    Hout = (Hout == H0) ? H1 : H0;
  }
  // output layer [out_pad x W]
  float acc[SO::TQ][SO::TO];
  zero_acc<16>(acc);
  tile_gemm<16, false>(A, lda_in, W, params + d.layer_off[d.n_hidden], W, Bs, acc);
  const int to2 = threadIdx.x % SO::NT_O, tq2 = threadIdx.x / SO::NT_O;
#pragma unroll
  for (int i = 0; i < SO::TQ; ++i) {
    int64_t q = q0 + tq2 * SO::TQ + i;
    if (q >= n) continue;
#pragma unroll
    for (int j = 0; j < SO::TO; ++j) {
      int o = to2 * SO::TO + j;
      if (o < out_stride) out[q * out_stride + o] = acc[i][j];
    }
  }
}

// Fused backward of one 64-query tile.  Inputs: X (encoded), acts (h_1..h_L),
// pred [n][16], target [n][out_ch].  Outputs: dZ of every layer
// (dz [L+1][n][16 or W]: index L is dOut), per-block loss partials, and dX
// (only when dX != NULL).
template <int W>
__global__ void __launch_bounds__(256) mlp_bwd_kernel(const float* __restrict__ params, const float* __restrict__ acts,
                                                      const float* __restrict__ pred, const float* __restrict__ target,
                                                      float* __restrict__ dz, float* __restrict__ dX,
                                                      float* __restrict__ loss_partial, int loss_type,
                                                      float inv_total, int64_t n) {
  using S = TileShape<W>;
  const MlpDims& d = c_dims[0];
  extern __shared__ float smem[];
  const int lda = BM + APAD;
  float* G0 = smem;                      // [max(W,16)][lda] gradient tile (k-major)
  float* G1 = G0 + W * lda;              // [W][lda]
  float* Bs = G1 + W * lda;              // [KC][max(W, in_pad) + 4]
  __shared__ float red[256];
  const int64_t q0 = (int64_t)blockIdx.x * BM;
  const int L = d.n_hidden;
  const int64_t dz_stride_W = (int64_t)n * W;

  // ---- loss gradient dOut [BM][16] -> G0 (k-major), and global dz[L]
  float lsum = 0.f;
  float* dout_g = dz + (int64_t)L * dz_stride_W;  // [n][16]
  for (int q = threadIdx.x; q < BM; q += 256) {
    int64_t gq = q0 + q;
    float g[16];
    for (int o = 0; o < 16; ++o) g[o] = 0.f;
    if (gq < n) {
      float p[16], t[16], v;
      for (int o = 0; o < d.out_ch; ++o) {
        p[o] = pred[gq * 16 + o];
        t[o] = target[gq * d.out_ch + o];
      }
      loss_grad(loss_type, p, t, d.out_ch, inv_total, g, &v);
      lsum += v;
      for (int o = 0; o < 16; ++o) dout_g[gq * 16 + o] = g[o];
    }
    for (int o = 0; o < 16; ++o) G0[o * lda + q] = g[o];
  }
  red[threadIdx.x] = lsum;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.f;
    for (int i = 0; i < BM && i < 256; ++i) s += red[i];  // fixed order
    loss_partial[blockIdx.x] = s;
  }
  const int to = threadIdx.x % S::NT_O, tq = threadIdx.x / S::NT_O;
  // ---- back-propagate: layer l = L (output) down to 1
  float* Gin = G0;
  float* Gout = G1;
  int Kin = 16;
  for (int l = L; l >= 1; --l) {
    float acc[S::TQ][S::TO];
    zero_acc<W>(acc);
    // dh_l = dz_{l+1} W_l  (W_l: [rows = Kin][cols = W])
    tile_gemm<W, true>(Gin, lda, Kin, params + d.layer_off[l], W, Bs, acc);
    __syncthreads();
    const float* h = acts + (int64_t)(l - 1) * n * W;  // h_l
    float* dzl = dz + (int64_t)(l - 1) * dz_stride_W;   // dz_l [n][W]
#pragma unroll
    for (int i = 0; i < S::TQ; ++i) {
      const int q = tq * S::TQ + i;
      const int64_t gq = q0 + q;
#pragma unroll
      for (int j = 0; j < S::TO; ++j) {
        const int k = to * S::TO + j;
        float g = 0.f;
        if (gq < n && h[gq * W + k] > 0.f) g = acc[i][j];
        Gout[k * lda + q] = g;
        if (gq < n) dzl[gq * W + k] = g;
      }
    }
    __syncthreads();
    float* t = Gin;
    Gin = Gout;
    Gout = t;
    Kin = W;
  }
  if (dX) {  // dX = dz_1 W_0   (W_0: [W][in_pad])
    for (int c0 = 0; c0 < d.in_pad; c0 += W) {
      float acc[S::TQ][S::TO];
      zero_acc<W>(acc);
      // columns c0..c0+W of W_0: B[k][o] = W0[k][c0 + o]
      tile_gemm<W, true>(Gin, lda, W, params + d.layer_off[0] + c0, d.in_pad, Bs, acc);
#pragma unroll
      for (int i = 0; i < S::TQ; ++i) {
        const int64_t gq = q0 + tq * S::TQ + i;
        if (gq >= n) continue;
#pragma unroll
        for (int j = 0; j < S::TO; ++j) {
          const int c = c0 + to * S::TO + j;
          if (c < d.in_pad) dX[gq * d.in_pad + c] = acc[i][j];
        }
      }
    }
  }
}

// Weight-gradient partials: part[s][M][N] = sum over queries of chunk s of
// G[q][m] * H[q][n]   (G: [n][M] row-major, H: [n][N] row-major).
constexpr int DW_TM = 64, DW_TN = 64, DW_QC = 32;
__global__ void __launch_bounds__(256) dw_partial_kernel(const float* __restrict__ G, int M,
                                                         const float* __restrict__ H, int N,
                                                         float* __restrict__ part, int64_t n,
                                                         int64_t chunk) {
  __shared__ float Gs[DW_QC][DW_TM + 4];
  __shared__ float Hs[DW_QC][DW_TN + 4];
  const int m0 = blockIdx.y * DW_TM, n0 = blockIdx.z * DW_TN;
  const int64_t qb = (int64_t)blockIdx.x * chunk, qe = min(n, qb + chunk);
  const int tm = threadIdx.x / 16, tn = threadIdx.x % 16;  // 16 x 16 threads, 4 x 4 each
  float acc[4][4] = {};
  for (int64_t qc = qb; qc < qe; qc += DW_QC) {
    __syncthreads();
    for (int i = threadIdx.x; i < DW_QC * DW_TM; i += 256) {
      int qq = i / DW_TM, mm = i % DW_TM;
      int64_t q = qc + qq;
      Gs[qq][mm] = (q < qe && m0 + mm < M) ? __ldg(G + q * M + m0 + mm) : 0.f;
    }
    for (int i = threadIdx.x; i < DW_QC * DW_TN; i += 256) {
      int qq = i / DW_TN, nn = i % DW_TN;
      int64_t q = qc + qq;
      Hs[qq][nn] = (q < qe && n0 + nn < N) ? __ldg(H + q * N + n0 + nn) : 0.f;
    }
    __syncthreads();
#pragma unroll 8
    for (int qq = 0; qq < DW_QC; ++qq) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = Gs[qq][tm * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Hs[qq][tn * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
  }
  float* dst = part + (int64_t)blockIdx.x * M * N;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int m = m0 + tm * 4 + i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int c = n0 + tn * 4 + j;
      if (c < N) dst[(int64_t)m * N + c] = acc[i][j];
    }
  }
}

// Sum split partials in split order into grad[off .. off + M*N).
__global__ void dw_reduce_kernel(const float* __restrict__ part, int splits, int64_t mn,
                                 float* __restrict__ grad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < mn; i += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int k = 0; k < splits; ++k) s += part[(int64_t)k * mn + i];
    grad[i] = s;
  }
}

// Adam (tcnn semantics).  Matrix weights [0, n_matrix) get l2_reg; encoding
// parameters with a zero gradient are left untouched (sparse update).
__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int64_t n, int64_t n_matrix, float lr, float beta1,
                            float beta2, float eps, float l2, float loss_scale) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float grad = g[i] / loss_scale;
    if (i >= n_matrix && grad == 0.f) continue;
    const float wf = w[i];
    if (i < n_matrix) grad += l2 * wf;
    const float m1 = m[i] = beta1 * m[i] + (1.f - beta1) * grad;
    const float v1 = v[i] = beta2 * v[i] + (1.f - beta2) * grad * grad;
    w[i] = wf - lr / (sqrtf(v1) + eps) * m1;
  }
}

__global__ void loss_reduce_kernel(const float* __restrict__ partial, int nb, float* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    float s = 0.f;
    for (int i = 0; i < nb; ++i) s += partial[i];
    *out = s;
  }
}

// ====================================================================== state
struct Mlp {
  MlpConfig cfg;
  int precision = 0;
  int64_t n_params = 0;
  float* params = nullptr;  // [net | enc]
  float* grads = nullptr;
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  int step = 0;
  float lr = 0.f;
  // workspace sized for `cap` queries
  int64_t cap = 0;
  float* X = nullptr;        // [cap][in_pad]
  float* acts = nullptr;     // [L][cap][W]
  float* pred = nullptr;     // [cap][16]
  float* dz = nullptr;       // [L][cap][W] + [cap][16]
  float* dX = nullptr;       // [cap][in_pad] (hash grids only)
  float* dw_part = nullptr;  // split partials
  int64_t dw_part_cap = 0;
  float* loss_part = nullptr;
  float* loss_dev = nullptr;
  long long* grid_acc = nullptr;  // fixed-point hash-grid gradient accumulator
  int64_t last_n = 0;        // batch of the last forward()
  const float* last_in = nullptr;
  // tensor-core inference (precision != FP32): packed weights, refreshed
  // when the FP32 master parameters change (params_version)
  TcPack tc;
  int64_t params_version = 1, packed_version = 0;
  int* tc_err_host = nullptr;  // host-mapped timeout flag of the kernel
  int* tc_err_dev = nullptr;
  // FP16 / BF16 handles also train on the tensor cores; FP16 gradients carry
  // a static loss scale of 128 (BF16: 1), divided out in the optimizer step
  TcTrainBufs tcb;
  uint8_t* tc_work = nullptr;  // tensor-core inference: encoded layer-0 operands
  int64_t tc_work_cap = 0;
  float loss_scale = 1.f;
  bool tc_train = false;
};

}  // namespace hm

using namespace hm;

static void free_ws(Mlp* m) {
  cudaFree(m->X);
  cudaFree(m->acts);
  cudaFree(m->pred);
  cudaFree(m->dz);
  cudaFree(m->dX);
  cudaFree(m->loss_part);
  m->X = m->acts = m->pred = m->dz = m->dX = m->loss_part = nullptr;
  m->cap = 0;
}

static int ensure_ws(Mlp* m, int64_t n) {
  if (n <= m->cap) return HM_OK;
  free_ws(m);
  const MlpDims& d = m->cfg.d;
  int64_t cap = std::max<int64_t>(n, 1024);
  cap = (cap + BM - 1) / BM * BM;
  cudaError_t e = cudaSuccess;
  e = cudaMalloc(&m->X, cap * d.in_pad * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->acts, (int64_t)d.n_hidden * cap * d.width * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->pred, cap * 16 * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->dz, ((int64_t)d.n_hidden * cap * d.width + cap * 16) * sizeof(float));
  if (e == cudaSuccess && d.n_enc_params > 0) e = cudaMalloc(&m->dX, cap * d.in_pad * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->loss_part, (cap / BM + 1) * sizeof(float));
  if (e != cudaSuccess) {
    free_ws(m);
    return hm_cuda_status(e, "mlp workspace");
  }
  m->cap = cap;
  return HM_OK;
}

static int set_dims_symbol(Mlp* m, cudaStream_t st) {
  cudaError_t e = cudaMemcpyToSymbolAsync(c_dims, &m->cfg.d, sizeof(MlpDims), 0, cudaMemcpyHostToDevice, st);
  return e == cudaSuccess ? HM_OK : hm_cuda_status(e, "mlp dims upload");
}

static size_t fwd_smem(const MlpDims& d) {
  const int lda = BM + APAD;
  return (size_t)(d.in_pad * lda + 2 * d.width * lda + KC * (std::max(d.width, 16) + 4)) * sizeof(float);
}
static size_t bwd_smem(const MlpDims& d) {
  const int lda = BM + APAD;
  return (size_t)(2 * std::max(d.width, 16) * lda + KC * (std::max(d.width, 16) + 4)) * sizeof(float);
}

template <int W>
static int launch_fwd(Mlp* m, const float* X, float* out, int out_stride, float* acts, int64_t n, cudaStream_t st) {
  size_t sm = fwd_smem(m->cfg.d);
  cudaFuncSetAttribute(mlp_fwd_kernel<W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  int blocks = (int)((n + BM - 1) / BM);
  mlp_fwd_kernel<W><<<blocks, 256, sm, st>>>(X, m->params, out, out_stride, acts, n);
  HM_CHECK_LAUNCH("mlp_fwd_kernel");
  return HM_OK;
}

template <int W>
static int launch_bwd(Mlp* m, const float* target, int loss, int64_t n, cudaStream_t st) {
  size_t sm = bwd_smem(m->cfg.d);
  cudaFuncSetAttribute(mlp_bwd_kernel<W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  int blocks = (int)((n + BM - 1) / BM);
  float inv_total = 1.f / ((float)n * (float)m->cfg.d.out_ch);
  mlp_bwd_kernel<W><<<blocks, 256, sm, st>>>(m->params, m->acts, m->pred, target, m->dz,
                                             m->cfg.d.n_enc_params > 0 ? m->dX : nullptr,
                                             m->loss_part, loss, inv_total, n);
  HM_CHECK_LAUNCH("mlp_bwd_kernel");
  loss_reduce_kernel<<<1, 32, 0, st>>>(m->loss_part, blocks, m->loss_dev);
  HM_CHECK_LAUNCH("loss_reduce_kernel");
  return HM_OK;
}

static int dispatch_fwd(Mlp* m, const float* X, float* out, int out_stride, float* acts, int64_t n, cudaStream_t st) {
  switch (m->cfg.d.width) {
    case 16: return launch_fwd<16>(m, X, out, out_stride, acts, n, st);
    case 32: return launch_fwd<32>(m, X, out, out_stride, acts, n, st);
    case 64: return launch_fwd<64>(m, X, out, out_stride, acts, n, st);
    default: return launch_fwd<128>(m, X, out, out_stride, acts, n, st);
  }
}
static int dispatch_bwd(Mlp* m, const float* target, int loss, int64_t n, cudaStream_t st) {
  switch (m->cfg.d.width) {
    case 16: return launch_bwd<16>(m, target, loss, n, st);
    case 32: return launch_bwd<32>(m, target, loss, n, st);
    case 64: return launch_bwd<64>(m, target, loss, n, st);
    default: return launch_bwd<128>(m, target, loss, n, st);
  }
}

static int encode(Mlp* m, const float* in, int64_t n, cudaStream_t st) {
  int s = set_dims_symbol(m, st);
  if (s) return s;
  encode_kernel<<<(int)((n + 255) / 256), 256, 0, st>>>(in, m->params + m->cfg.d.n_net_params, m->X, n);
  HM_CHECK_LAUNCH("encode_kernel");
  return HM_OK;
}

// ---- parameter initialisation (host, deterministic per seed)
static void init_params(const MlpConfig& c, uint32_t seed, std::vector<float>& p) {
  const MlpDims& d = c.d;
  p.assign(d.n_net_params + d.n_enc_params, 0.f);
  uint32_t st = rng_seed((int)seed, 0x5eedu);
  for (int l = 0; l <= d.n_hidden; ++l) {
    int fan_in = l == 0 ? d.in_pad : d.width;
    int fan_out = l == d.n_hidden ? d.out_pad : d.width;
    int64_t cnt = (int64_t)fan_in * fan_out;
    float* w = p.data() + d.layer_off[l];
    if (c.init == "he_normal") {
      float sd = sqrtf(2.f / (float)fan_in);
      for (int64_t i = 0; i < cnt; ++i) {
        float u1 = fmaxf(lcg_next(st), 1e-12f), u2 = lcg_next(st);
        w[i] = sd * sqrtf(-2.f * logf(u1)) * cosf(2.f * kPi * u2);
      }
    } else {
      float s = sqrtf(6.f / (float)(fan_in + fan_out));
      for (int64_t i = 0; i < cnt; ++i) w[i] = s * (2.f * lcg_next(st) - 1.f);
    }
  }
  for (int64_t i = 0; i < d.n_enc_params; ++i) p[d.n_net_params + i] = 1e-4f * (2.f * lcg_next(st) - 1.f);
}

// ====================================================================== C ABI
extern "C" hm_mlp* hm_mlp_create(const char* config_json, int in_ch, int out_ch, int precision,
                                 uint32_t seed, int* status) {
  int dummy;
  if (!status) status = &dummy;
  Mlp* m = new Mlp();
  try {
    m->cfg = mlp_config_from_json(config_json, in_ch, out_ch);
  } catch (const std::exception& e) {
    hm_set_error("%s", e.what());
    delete m;
    *status = HM_EPARSE;
    return nullptr;
  }
  if (precision != HM_PREC_FP32) {
    std::string why;
    if (!tc_supported(m->cfg.d, precision, &why)) {
      delete m;
      *status = HM_EUNSUPPORTED;
      hm_set_error("hm_mlp_create: precision %d is not available for this network (%s)", precision, why.c_str());
      return nullptr;
    }
  }
  m->precision = precision;
  m->n_params = m->cfg.d.n_net_params + m->cfg.d.n_enc_params;
  m->lr = m->cfg.adam.lr;
  size_t bytes = m->n_params * sizeof(float);
  cudaError_t e = cudaMalloc(&m->params, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&m->grads, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&m->adam_m, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&m->adam_v, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&m->loss_dev, sizeof(float));
  if (e == cudaSuccess && precision != HM_PREC_FP32) {
    e = cudaHostAlloc(&m->tc_err_host, sizeof(int), cudaHostAllocMapped);
    if (e == cudaSuccess) {
      *m->tc_err_host = 0;
      e = cudaHostGetDevicePointer(&m->tc_err_dev, m->tc_err_host, 0);
    }
    if (e == cudaSuccess) {
      int st = tc_pack_alloc(m->cfg.d, precision, &m->tc);
      if (st != HM_OK) e = cudaErrorMemoryAllocation;
    }
    m->tc_train = tc_trainable(m->cfg.d, precision);
    // FP16 operands in the backward pass (FP16 handles; E4M3 handles' backward)
    m->loss_scale = precision == HM_PREC_FP16 || precision == HM_PREC_FP8_E4M3 ? 128.f : 1.f;
  }
  if (e != cudaSuccess) {
    *status = hm_cuda_status(e, "hm_mlp_create");
    hm_mlp_destroy((hm_mlp*)m);
    return nullptr;
  }
  std::vector<float> p;
  init_params(m->cfg, seed, p);
  e = cudaMemcpy(m->params, p.data(), bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(m->adam_m, 0, bytes);
  if (e == cudaSuccess) e = cudaMemset(m->adam_v, 0, bytes);
  if (e == cudaSuccess) e = cudaMemset(m->grads, 0, bytes);
  if (e != cudaSuccess) {
    *status = hm_cuda_status(e, "hm_mlp_create upload");
    hm_mlp_destroy((hm_mlp*)m);
    return nullptr;
  }
  *status = HM_OK;
  return (hm_mlp*)m;
}

extern "C" void hm_mlp_destroy(hm_mlp* h) {
  Mlp* m = (Mlp*)h;
  if (!m) return;
  free_ws(m);
  cudaFree(m->params);
  cudaFree(m->grads);
  cudaFree(m->adam_m);
  cudaFree(m->adam_v);
  cudaFree(m->dw_part);
  cudaFree(m->loss_dev);
  cudaFree(m->grid_acc);
  tc_pack_free(&m->tc);
  tc_train_free(&m->tcb);
  cudaFree(m->tc_work);
  if (m->tc_err_host) cudaFreeHost(m->tc_err_host);
  delete m;
}

extern "C" int hm_mlp_info(const hm_mlp* h, hm_mlp_desc* out) {
  const Mlp* m = (const Mlp*)h;
  if (!m || !out) return hm_set_error("hm_mlp_info: NULL"), HM_EINVAL;
  const MlpDims& d = m->cfg.d;
  out->in_ch = d.in_ch;
  out->out_ch = d.out_ch;
  out->encoded_width = d.n_enc;
  out->padded_input_width = d.in_pad;
  out->width = d.width;
  out->n_hidden_layers = d.n_hidden;
  out->padded_output_width = d.out_pad;
  out->n_params = m->n_params;
  out->n_network_params = d.n_net_params;
  out->precision = m->precision;
  out->step = m->step;
  out->learning_rate = m->lr;
  return HM_OK;
}

extern "C" int hm_mlp_get_params(const hm_mlp* h, float* host_out) {
  const Mlp* m = (const Mlp*)h;
  if (!m || !host_out) return hm_set_error("hm_mlp_get_params: NULL"), HM_EINVAL;
  cudaError_t e = cudaMemcpy(host_out, m->params, m->n_params * sizeof(float), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? HM_OK : hm_cuda_status(e, "hm_mlp_get_params");
}

extern "C" int hm_mlp_set_params(hm_mlp* h, const float* host_in) {
  Mlp* m = (Mlp*)h;
  if (!m || !host_in) return hm_set_error("hm_mlp_set_params: NULL"), HM_EINVAL;
  cudaError_t e = cudaMemcpy(m->params, host_in, m->n_params * sizeof(float), cudaMemcpyHostToDevice);
  m->params_version += 1;
  return e == cudaSuccess ? HM_OK : hm_cuda_status(e, "hm_mlp_set_params");
}

extern "C" int hm_mlp_get_gradients(const hm_mlp* h, float* host_out) {
  const Mlp* m = (const Mlp*)h;
  if (!m || !host_out) return hm_set_error("hm_mlp_get_gradients: NULL"), HM_EINVAL;
  cudaError_t e = cudaMemcpy(host_out, m->grads, m->n_params * sizeof(float), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && m->tc_train && m->loss_scale != 1.f)  // undo the FP16 loss scale
    for (int64_t i = 0; i < m->n_params; ++i) host_out[i] /= m->loss_scale;
  return e == cudaSuccess ? HM_OK : hm_cuda_status(e, "hm_mlp_get_gradients");
}

// TINY_MLP::reset (cuda/neural_network.cu:17-21): every parameter set to zero.
extern "C" int hm_mlp_reset(hm_mlp* h) {
  Mlp* m = (Mlp*)h;
  if (!m) return hm_set_error("hm_mlp_reset: NULL"), HM_EINVAL;
  size_t bytes = m->n_params * sizeof(float);
  cudaError_t e = cudaMemset(m->params, 0, bytes);
  if (e == cudaSuccess) e = cudaMemset(m->adam_m, 0, bytes);
  if (e == cudaSuccess) e = cudaMemset(m->adam_v, 0, bytes);
  m->step = 0;
  m->lr = m->cfg.adam.lr;
  m->params_version += 1;
  return e == cudaSuccess ? HM_OK : hm_cuda_status(e, "hm_mlp_reset");
}

// A bounded tensor-core wait that expired in an earlier call is reported here.
static int tc_prepare(Mlp* m) {
  if (*(volatile int*)m->tc_err_host) {
    *m->tc_err_host = 0;
    return hm_set_error("mlp: a tensor-core wait expired in an earlier call"), HM_ETIMEOUT;
  }
  return HM_OK;
}

// Inference on the tensor cores (FP16 / BF16 / E4M3 operands, FP32
// accumulation).  With allow_alloc, where tc_forward runs the encode kernel
// before the layers, the encoded operands go through a workspace grown on
// demand; without it (hm_mlp_inference_noalloc) the encoding runs inside
// the layer kernels.  A bounded wait that expired in an earlier call is
// reported here.
static int tc_inference(Mlp* m, const float* d_in, float* d_out, int64_t n, cudaStream_t st, bool allow_alloc) {
  if (*(volatile int*)m->tc_err_host) {
    *m->tc_err_host = 0;
    return hm_set_error("mlp: a tensor-core wait expired in an earlier call"), HM_ETIMEOUT;
  }
  if (m->packed_version != m->params_version) {
    if (int s = tc_pack(m->cfg.d, m->params, m->tc, st)) return s;
    m->packed_version = m->params_version;
  }
  allow_alloc = allow_alloc && tc_wants_workspace(m->cfg.d, m->tc);
  if (allow_alloc) {
    const int64_t need = tc_encode_bytes(m->cfg.d, m->tc, n);
    if (need > m->tc_work_cap) {
      cudaFree(m->tc_work);
      m->tc_work = nullptr;
      m->tc_work_cap = 0;
      cudaError_t e = cudaMalloc(&m->tc_work, (size_t)need);
      if (e != cudaSuccess) return hm_cuda_status(e, "tensor-core encode workspace");
      m->tc_work_cap = need;
    }
  }
  return tc_forward(m->cfg.d, m->tc, m->params + m->cfg.d.n_net_params, d_in, d_out, m->cfg.d.out_ch, n,
                    m->tc_err_dev, st, allow_alloc ? m->tc_work : nullptr, allow_alloc ? m->tc_work_cap : 0);
}

static int check_io(const char* who, Mlp* m, const void* a, const void* b, int64_t n) {
  if (!m) return hm_set_error("%s: NULL handle", who), HM_EINVAL;
  if (n < 0) return hm_set_error("%s: n < 0", who), HM_EINVAL;
  if (n > 0 && (!a || !b)) return hm_set_error("%s: NULL buffer", who), HM_EINVAL;
  if (n > ((int64_t)1 << 31)) return hm_set_error("%s: n too large", who), HM_ECAPACITY;
  return HM_OK;
}

// TINY_MLP::inference (cuda/neural_network.cu:58-64): d_in [n][in_ch],
// d_out [n][out_ch], both row-major per query (tcnn column-major GPUMatrix).
extern "C" int hm_mlp_inference(hm_mlp* h, const float* d_in, float* d_out, int64_t n, void* stream) {
  Mlp* m = (Mlp*)h;
  if (int s = check_io("hm_mlp_inference", m, d_in, d_out, n)) return s;
  if (n == 0) return HM_OK;
  cudaStream_t st = (cudaStream_t)stream;
  if (m->precision != HM_PREC_FP32) return tc_inference(m, d_in, d_out, n, st, true);
  if (int s = ensure_ws(m, n)) return s;
  if (int s = encode(m, d_in, n, st)) return s;
  return dispatch_fwd(m, m->X, d_out, m->cfg.d.out_ch, nullptr, n, st);
}

// Training forward: keeps the activations for hm_mlp_backward; d_out may be NULL.
extern "C" int hm_mlp_forward(hm_mlp* h, const float* d_in, float* d_out, int64_t n, void* stream) {
  Mlp* m = (Mlp*)h;
  if (int s = check_io("hm_mlp_forward", m, d_in, d_in, n)) return s;
  if (n == 0) return HM_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const float* pred = nullptr;
  if (m->tc_train) {
    if (int s = tc_prepare(m)) return s;
    if (n > m->tcb.cap) {
      const int64_t cap = std::max<int64_t>((n + 127) / 128 * 128, 1024);
      if (int s = tc_train_alloc(m->cfg.d, cap, m->cfg.d.n_enc_params > 0, &m->tcb)) return s;
    }
    if (m->packed_version != m->params_version) {
      if (int s = tc_pack(m->cfg.d, m->params, m->tc, st)) return s;
      m->packed_version = m->params_version;
    }
    if (int s = tc_train_forward(m->cfg.d, m->tc, m->params + m->cfg.d.n_net_params, d_in, n, m->tcb, m->tc_err_dev,
                                 st))
      return s;
    pred = m->tcb.pred;
  } else {
    if (int s = ensure_ws(m, n)) return s;
    if (int s = encode(m, d_in, n, st)) return s;
    if (int s = dispatch_fwd(m, m->X, m->pred, 16, m->acts, n, st)) return s;
    pred = m->pred;
  }
  m->last_n = n;
  m->last_in = d_in;
  if (d_out) {
    cudaError_t e = cudaMemcpy2DAsync(d_out, m->cfg.d.out_ch * sizeof(float), pred, 16 * sizeof(float),
                                      m->cfg.d.out_ch * sizeof(float), n, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return hm_cuda_status(e, "hm_mlp_forward copy");
  }
  return HM_OK;
}

// Backward of the last forward against d_target [n][out_ch] under `loss`
// (LOSS_OUTPUT_GRAD: d_target is dL/d(output)): fills the parameter
// gradients and the loss (device scalar; d_loss may be NULL).
static int mlp_backward(Mlp* m, const char* who, const float* d_target, int loss, int64_t n, float* d_loss,
                        cudaStream_t st) {
  if (int s = check_io(who, m, d_target, d_target, n)) return s;
  if (n == 0) return HM_OK;
  if (n != m->last_n) return hm_set_error("%s: batch differs from the last forward", who), HM_EINVAL;
  const MlpDims& d = m->cfg.d;
  if (int s = set_dims_symbol(m, st)) return s;
  if (m->tc_train) {
    if (int s = tc_prepare(m)) return s;
    if (int s = tc_backward(d, m->tc, m->tcb, d_target, loss, m->loss_scale, n, m->loss_dev, m->grads,
                            &m->dw_part, &m->dw_part_cap, m->tc_err_dev, st))
      return s;
    if (d.n_enc_params > 0) {
      if (!m->grid_acc) {
        cudaError_t e = cudaMalloc(&m->grid_acc, d.n_enc_params * sizeof(long long));
        if (e != cudaSuccess) return hm_cuda_status(e, "grid grad accumulator");
      }
      cudaError_t e = cudaMemsetAsync(m->grid_acc, 0, d.n_enc_params * sizeof(long long), st);
      if (e != cudaSuccess) return hm_cuda_status(e, "grid grad clear");
      grid_bwd_kernel<<<(int)((n + 255) / 256), 256, 0, st>>>(m->last_in, m->tcb.dX, m->grid_acc, n);
      HM_CHECK_LAUNCH("grid_bwd_kernel");
      grid_fix_to_float_kernel<<<1024, 256, 0, st>>>(m->grid_acc, m->grads + d.n_net_params, d.n_enc_params);
      HM_CHECK_LAUNCH("grid_fix_to_float_kernel");
    }
    if (d_loss) {
      cudaError_t e = cudaMemcpyAsync(d_loss, m->loss_dev, sizeof(float), cudaMemcpyDeviceToDevice, st);
      if (e != cudaSuccess) return hm_cuda_status(e, "loss copy");
    }
    return HM_OK;
  }
  if (int s = dispatch_bwd(m, d_target, loss, n, st)) return s;
  // weight gradients, split over the batch in fixed chunks
  const int64_t chunk = 1024;
  const int splits = (int)((n + chunk - 1) / chunk);
  int64_t need = 0;
  for (int l = 0; l <= d.n_hidden; ++l) {
    int M = l == d.n_hidden ? d.out_pad : d.width;
    int N = l == 0 ? d.in_pad : d.width;
    need = std::max<int64_t>(need, (int64_t)splits * M * N);
  }
  if (need > m->dw_part_cap) {
    cudaFree(m->dw_part);
    m->dw_part = nullptr;
    cudaError_t e = cudaMalloc(&m->dw_part, need * sizeof(float));
    if (e != cudaSuccess) return hm_cuda_status(e, "dw partials");
    m->dw_part_cap = need;
  }
  for (int l = 0; l <= d.n_hidden; ++l) {
    int M = l == d.n_hidden ? d.out_pad : d.width;
    int N = l == 0 ? d.in_pad : d.width;
    const float* G = l == d.n_hidden ? m->dz + (int64_t)d.n_hidden * n * d.width : m->dz + (int64_t)l * n * d.width;
    const float* H = l == 0 ? m->X : m->acts + (int64_t)(l - 1) * n * d.width;
    dim3 grid(splits, (M + DW_TM - 1) / DW_TM, (N + DW_TN - 1) / DW_TN);
    dw_partial_kernel<<<grid, 256, 0, st>>>(G, M, H, N, m->dw_part, n, chunk);
    HM_CHECK_LAUNCH("dw_partial_kernel");
    dw_reduce_kernel<<<256, 256, 0, st>>>(m->dw_part, splits, (int64_t)M * N, m->grads + d.layer_off[l]);
    HM_CHECK_LAUNCH("dw_reduce_kernel");
  }
  if (d.n_enc_params > 0) {
    if (!m->grid_acc) {
      cudaError_t e = cudaMalloc(&m->grid_acc, d.n_enc_params * sizeof(long long));
      if (e != cudaSuccess) return hm_cuda_status(e, "grid grad accumulator");
    }
    cudaError_t e = cudaMemsetAsync(m->grid_acc, 0, d.n_enc_params * sizeof(long long), st);
    if (e != cudaSuccess) return hm_cuda_status(e, "grid grad clear");
    grid_bwd_kernel<<<(int)((n + 255) / 256), 256, 0, st>>>(m->last_in, m->dX, m->grid_acc, n);
    HM_CHECK_LAUNCH("grid_bwd_kernel");
    grid_fix_to_float_kernel<<<1024, 256, 0, st>>>(m->grid_acc, m->grads + d.n_net_params, d.n_enc_params);
    HM_CHECK_LAUNCH("grid_fix_to_float_kernel");
  }
  if (d_loss) {
    cudaError_t e = cudaMemcpyAsync(d_loss, m->loss_dev, sizeof(float), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return hm_cuda_status(e, "loss copy");
  }
  return HM_OK;
}

extern "C" int hm_mlp_backward(hm_mlp* h, const float* d_target, int64_t n, float* d_loss, void* stream) {
  Mlp* m = (Mlp*)h;
  if (!m) return hm_set_error("hm_mlp_backward: NULL"), HM_EINVAL;
  return mlp_backward(m, "hm_mlp_backward", d_target, m->cfg.loss, n, d_loss, (cudaStream_t)stream);
}

// tcnn's backward with a given dL/d(output) [n][out_ch] (no loss).
extern "C" int hm_mlp_backward_output_grad(hm_mlp* h, const float* d_dloss_doutput, int64_t n, void* stream) {
  Mlp* m = (Mlp*)h;
  if (!m) return hm_set_error("hm_mlp_backward_output_grad: NULL"), HM_EINVAL;
  return mlp_backward(m, "hm_mlp_backward_output_grad", d_dloss_doutput, LOSS_OUTPUT_GRAD, n, nullptr,
                      (cudaStream_t)stream);
}

// One optimizer step on the current gradients: ExponentialDecay wrapping
// Adam (tcnn semantics; bias correction folded into the learning rate).
extern "C" int hm_mlp_optimizer_step(hm_mlp* h, float loss_scale, void* stream) {
  Mlp* m = (Mlp*)h;
  if (!m) return hm_set_error("hm_mlp_optimizer_step: NULL"), HM_EINVAL;
  if (!(loss_scale > 0.f)) loss_scale = 1.f;
  const AdamCfg& a = m->cfg.adam;
  if (m->step >= a.decay_start && (m->step - a.decay_start) % a.decay_interval == 0) m->lr *= a.decay_base;
  m->step += 1;
  const double t = m->step;
  const float lr_t = (float)(m->lr * sqrt(1.0 - pow((double)a.beta2, t)) / (1.0 - pow((double)a.beta1, t)));
  adam_kernel<<<1024, 256, 0, (cudaStream_t)stream>>>(m->params, m->grads, m->adam_m, m->adam_v, m->n_params,
                                                      m->cfg.d.n_net_params, lr_t, a.beta1, a.beta2, a.eps,
                                                      a.l2_reg, loss_scale);
  HM_CHECK_LAUNCH("adam_kernel");
  m->params_version += 1;
  return HM_OK;
}

// Trainer::training_step (render_hair_msnn.cu:690): forward, loss, backward,
// optimizer step.  d_loss (device float) may be NULL.
extern "C" int hm_mlp_training_step(hm_mlp* h, const float* d_in, const float* d_target, int64_t n,
                                    float* d_loss, void* stream) {
  if (int s = hm_mlp_forward(h, d_in, nullptr, n, stream)) return s;
  if (n == 0) return HM_OK;
  if (int s = hm_mlp_backward(h, d_target, n, d_loss, stream)) return s;
  return hm_mlp_optimizer_step(h, ((Mlp*)h)->loss_scale, stream);
}

// trainer->loss(ctx) (render_hair_msnn.cu:691): the last loss, synchronously.
extern "C" int hm_mlp_last_loss(hm_mlp* h, float* host_loss) {
  Mlp* m = (Mlp*)h;
  if (!m || !host_loss) return hm_set_error("hm_mlp_last_loss: NULL"), HM_EINVAL;
  cudaError_t e = cudaMemcpy(host_loss, m->loss_dev, sizeof(float), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? HM_OK : hm_cuda_status(e, "hm_mlp_last_loss");
}

// ---- save / load: "HMMLP1\n" + one JSON line {n_params, step, lr} + raw
// float32 params.  TINY_MLP::loadWeights (cuda/neural_network.cu:23-32)
// deserialised a tcnn JSON snapshot; that format belongs to tcnn.
// ---- tiny-cuda-nn trainer snapshots (TINY_MLP::loadWeights deserializes
// one, neural_network.cu:23-32, from the scene's tcnn.init_weights,
// scene.cpp:330-331).  tiny-cuda-nn is an absent submodule of the
// reference; its Trainer serialises to a JSON object
//   {"n_params": N, "params_type": "float" | "__half",
//    "params_binary": <N parameters of that type, little-endian>, ...}
// where a binary value written as JSON text is {"bytes": [b0, b1, ...],
// "subtype": null}.  The parameters are the network's weight matrices, layer
// after layer, each row-major [outputs][inputs] with the input width padded
// to 16 and the last layer's outputs padded to 16, then the encoding's
// parameters (hash-grid tables level after level): the layout of this
// library's own parameter vector.  Optimizer state in a snapshot is not read
// (the optimizer restarts, as after TINY_MLP::reset).

static bool ends_with(const char* s, const char* suffix) {
  const size_t a = strlen(s), b = strlen(suffix);
  return a >= b && strcmp(s + a - b, suffix) == 0;
}

static float half_to_float(uint16_t h) {  // IEEE 754 binary16 -> binary32
  const uint32_t sign = (uint32_t)(h >> 15) << 31;
  uint32_t exp = (h >> 10) & 0x1f, man = h & 0x3ff, bits;
  if (exp == 0x1f) {
    bits = sign | 0x7f800000u | (man << 13);
  } else if (exp != 0) {
    bits = sign | ((exp + 112) << 23) | (man << 13);
  } else if (man == 0) {
    bits = sign;
  } else {  // subnormal: normalise
    int e = -1;
    do {
      ++e;
      man <<= 1;
    } while (!(man & 0x400));
    bits = sign | ((uint32_t)(112 - e) << 23) | ((man & 0x3ff) << 13);
  }
  float f;
  memcpy(&f, &bits, 4);
  return f;
}

// The value of "key": <number> / "key": "<word>" anywhere in text (the
// snapshot's top-level scalars), or false.
static bool scan_scalar(const std::string& text, const char* key, std::string* out) {
  const std::string k = std::string("\"") + key + "\"";
  size_t at = text.find(k);
  if (at == std::string::npos) return false;
  at = text.find(':', at + k.size());
  if (at == std::string::npos) return false;
  ++at;
  while (at < text.size() && isspace((unsigned char)text[at])) ++at;
  size_t end = at;
  if (at < text.size() && text[at] == '"') {
    end = text.find('"', at + 1);
    if (end == std::string::npos) return false;
    *out = text.substr(at + 1, end - at - 1);
    return true;
  }
  while (end < text.size() && (isdigit((unsigned char)text[end]) || text[end] == '.' || text[end] == '-' ||
                               text[end] == '+' || text[end] == 'e' || text[end] == 'E'))
    ++end;
  *out = text.substr(at, end - at);
  return end > at;
}

static int load_tcnn_snapshot(Mlp* m, const char* path) {
  FILE* f = fopen(path, "rb");
  if (!f) return hm_set_error("hm_mlp_load: cannot open %s", path), HM_EINVAL;
  std::string text;
  char buf[1 << 16];
  size_t r;
  while ((r = fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, r);
  fclose(f);
  std::string v;
  if (!scan_scalar(text, "n_params", &v)) return hm_set_error("hm_mlp_load: no n_params in %s", path), HM_EPARSE;
  const long long n = atoll(v.c_str());
  if (n != m->n_params)
    return hm_set_error("hm_mlp_load: %s holds %lld parameters, the network has %lld", path, n,
                        (long long)m->n_params),
           HM_EINVAL;
  std::string type = "float";
  scan_scalar(text, "params_type", &type);
  const int elem = type == "float" ? 4 : (type == "__half" ? 2 : 0);
  if (!elem) return hm_set_error("hm_mlp_load: params_type %s not supported", type.c_str()), HM_EUNSUPPORTED;
  size_t at = text.find("\"params_binary\"");
  if (at != std::string::npos) at = text.find("\"bytes\"", at);
  if (at != std::string::npos) at = text.find('[', at);
  if (at == std::string::npos) return hm_set_error("hm_mlp_load: no params_binary bytes in %s", path), HM_EPARSE;
  std::vector<uint8_t> bytes;
  bytes.reserve((size_t)n * elem);
  const char* p = text.c_str() + at + 1;
  for (;;) {
    while (*p && (isspace((unsigned char)*p) || *p == ',')) ++p;
    if (*p == ']') break;
    char* end = nullptr;
    const long b = strtol(p, &end, 10);
    if (end == p || b < 0 || b > 255) return hm_set_error("hm_mlp_load: bad byte in params_binary"), HM_EPARSE;
    bytes.push_back((uint8_t)b);
    p = end;
  }
  if ((long long)bytes.size() != n * elem)
    return hm_set_error("hm_mlp_load: params_binary holds %zu bytes, %lld expected", bytes.size(), n * elem),
           HM_EPARSE;
  std::vector<float> params((size_t)n);
  for (long long i = 0; i < n; ++i) {
    if (elem == 4) {
      memcpy(&params[i], &bytes[4 * i], 4);
    } else {
      uint16_t h;
      memcpy(&h, &bytes[2 * i], 2);
      params[i] = half_to_float(h);
    }
  }
  m->step = 0;
  m->lr = m->cfg.adam.lr;
  return hm_mlp_set_params((hm_mlp*)m, params.data());
}

static int save_tcnn_snapshot(const Mlp* m, const char* path) {
  std::vector<float> p(m->n_params);
  if (int s = hm_mlp_get_params((const hm_mlp*)m, p.data())) return s;
  FILE* f = fopen(path, "wb");
  if (!f) return hm_set_error("hm_mlp_save: cannot open %s", path), HM_EINVAL;
  fprintf(f, "{\"n_params\": %lld, \"params_type\": \"float\", \"params_binary\": {\"bytes\": [",
          (long long)m->n_params);
  const uint8_t* b = (const uint8_t*)p.data();
  for (size_t i = 0; i < p.size() * 4; ++i) fprintf(f, i ? ",%u" : "%u", (unsigned)b[i]);
  fprintf(f, "], \"subtype\": null}}\n");
  const bool ok = fclose(f) == 0;
  return ok ? HM_OK : (hm_set_error("hm_mlp_save: write failed"), HM_EINVAL);
}

extern "C" int hm_mlp_save(const hm_mlp* h, const char* path) {
  const Mlp* m = (const Mlp*)h;
  if (!m || !path) return hm_set_error("hm_mlp_save: NULL"), HM_EINVAL;
  if (ends_with(path, ".json")) return save_tcnn_snapshot(m, path);
  std::vector<float> p(m->n_params);
  if (int s = hm_mlp_get_params(h, p.data())) return s;
  FILE* f = fopen(path, "wb");
  if (!f) return hm_set_error("hm_mlp_save: cannot open %s", path), HM_EINVAL;
  fprintf(f, "HMMLP1\n{\"n_params\": %lld, \"step\": %d, \"lr\": %.9g}\n", (long long)m->n_params, m->step, m->lr);
  size_t w = fwrite(p.data(), sizeof(float), p.size(), f);
  fclose(f);
  return w == p.size() ? HM_OK : (hm_set_error("hm_mlp_save: short write"), HM_EINVAL);
}

extern "C" int hm_mlp_load(hm_mlp* h, const char* path) {
  Mlp* m = (Mlp*)h;
  if (!m || !path) return hm_set_error("hm_mlp_load: NULL"), HM_EINVAL;
  FILE* f = fopen(path, "rb");
  if (!f) return hm_set_error("hm_mlp_load: cannot open %s", path), HM_EINVAL;
  int first = fgetc(f);
  while (first == ' ' || first == '\n' || first == '\r' || first == '\t') first = fgetc(f);
  if (first == '{') {
    fclose(f);
    return load_tcnn_snapshot(m, path);
  }
  rewind(f);
  char magic[16] = {0}, line[512] = {0};
  if (!fgets(magic, sizeof(magic), f) || strcmp(magic, "HMMLP1\n") != 0 || !fgets(line, sizeof(line), f)) {
    fclose(f);
    return hm_set_error("hm_mlp_load: bad header in %s", path), HM_EPARSE;
  }
  try {
    Json j = json_parse(line);
    if ((int64_t)j["n_params"].as_number() != m->n_params) {
      fclose(f);
      return hm_set_error("hm_mlp_load: parameter count mismatch"), HM_EINVAL;
    }
    m->step = (int)j.number_or("step", 0);
    m->lr = (float)j.number_or("lr", m->cfg.adam.lr);
  } catch (const std::exception& e) {
    fclose(f);
    return hm_set_error("hm_mlp_load: %s", e.what()), HM_EPARSE;
  }
  std::vector<float> p(m->n_params);
  size_t r = fread(p.data(), sizeof(float), p.size(), f);
  fclose(f);
  if (r != p.size()) return hm_set_error("hm_mlp_load: truncated file"), HM_EPARSE;
  return hm_mlp_set_params(h, p.data());
}

// Host-side config check (no device work): parses the JSON and reports the
// derived sizes, or HM_EPARSE with the message.
extern "C" int hm_mlp_describe_config(const char* config_json, int in_ch, int out_ch, hm_mlp_desc* out) {
  if (!out) return hm_set_error("hm_mlp_describe_config: NULL"), HM_EINVAL;
  try {
    MlpConfig c = mlp_config_from_json(config_json, in_ch, out_ch);
    const MlpDims& d = c.d;
    out->in_ch = d.in_ch;
    out->out_ch = d.out_ch;
    out->encoded_width = d.n_enc;
    out->padded_input_width = d.in_pad;
    out->width = d.width;
    out->n_hidden_layers = d.n_hidden;
    out->padded_output_width = d.out_pad;
    out->n_params = d.n_net_params + d.n_enc_params;
    out->n_network_params = d.n_net_params;
    out->precision = HM_PREC_FP32;
    out->step = 0;
    out->learning_rate = c.adam.lr;
  } catch (const std::exception& e) {
    hm_set_error("%s", e.what());
    return HM_EPARSE;
  }
  return HM_OK;
}

// ============================================= inference without allocation
// hm_mlp_inference_noalloc: the same encode + fused forward kernels as
// hm_mlp_inference, but the encoded-input scratch ([n][in_pad] floats, the
// only per-call device memory inference needs) lives in a fixed file-scope
// device array instead of the handle's cudaMalloc'd workspace.  It exists for
// callers that may not allocate device memory once running: a frame loop that
// reserves all of its memory up front and must not stall on cudaMalloc (which
// can synchronise the device) or fail on it under memory pressure halfway
// through a frame.
//
// Limits and rules:
//  * n * in_pad <= kNoAllocScratchFloats (4 MiB of floats, e.g. 4,681
//    queries at in_pad 224, 16,384 at in_pad 64); larger n is rejected with
//    HM_ECAPACITY and nothing is launched.  Split larger batches.
//  * Nothing has to start at zero: the encode kernel writes every one of the
//    first n * in_pad floats before the forward kernel reads them.
//  * One scratch per device, shared by every handle: two calls whose work
//    overlaps on the device (different streams, threads or handles without an
//    ordering between them) overwrite each other's scratch.  Order them.
//  * The first call on a device resolves the array's address with
//    cudaGetSymbolAddress with that device current (this can load the
//    library's device code); make that first call before any stream capture.
//    The address is cached for the life of the process, so a device reset
//    (a new primary context) while the library is loaded is not supported.
constexpr int64_t kNoAllocScratchFloats = (int64_t)1 << 20;
constexpr int kNoAllocMaxDevices = 64;
static __device__ __align__(256) float g_noalloc_scratch[kNoAllocScratchFloats];
static float* s_noalloc_ptr[kNoAllocMaxDevices];
static std::mutex s_noalloc_mu;

static int noalloc_scratch(float** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return hm_cuda_status(e, "hm_mlp_inference_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= kNoAllocMaxDevices)
    return hm_set_error("hm_mlp_inference_noalloc: device %d beyond the %d supported", dev, kNoAllocMaxDevices),
           HM_EUNSUPPORTED;
  std::lock_guard<std::mutex> lock(s_noalloc_mu);
  if (!s_noalloc_ptr[dev]) {
    float* p = nullptr;
    e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return hm_cuda_status(e, "hm_mlp_inference_noalloc: cudaGetSymbolAddress");
    s_noalloc_ptr[dev] = p;
  }
  *out = s_noalloc_ptr[dev];
  return HM_OK;
}

extern "C" int hm_mlp_inference_noalloc(hm_mlp* h, const float* d_in, float* d_out, int64_t n, void* stream) {
  Mlp* m = (Mlp*)h;
  if (int s = check_io("hm_mlp_inference_noalloc", m, d_in, d_out, n)) return s;
  if (n == 0) return HM_OK;
  if (m->precision != HM_PREC_FP32) return tc_inference(m, d_in, d_out, n, (cudaStream_t)stream, false);
  const int64_t need = n * (int64_t)m->cfg.d.in_pad;
  if (need > kNoAllocScratchFloats)
    return hm_set_error("hm_mlp_inference_noalloc: %lld queries x %d encoded floats exceed the static scratch of "
                        "%lld floats (at most %lld queries per call for this network)",
                        (long long)n, m->cfg.d.in_pad, (long long)kNoAllocScratchFloats,
                        (long long)(kNoAllocScratchFloats / m->cfg.d.in_pad)),
           HM_ECAPACITY;
  float* X = nullptr;
  if (int s = noalloc_scratch(&X)) return s;
  cudaStream_t st = (cudaStream_t)stream;
  if (int s = set_dims_symbol(m, st)) return s;
  encode_kernel<<<(int)((n + 255) / 256), 256, 0, st>>>(d_in, m->params + m->cfg.d.n_net_params, X, n);
  HM_CHECK_LAUNCH("encode_kernel");
  return dispatch_fwd(m, X, d_out, m->cfg.d.out_ch, nullptr, n, st);
}
