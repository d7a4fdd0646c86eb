// ORACLE-side CPU transcription of the radiance-cache network (test
// infrastructure and the CPU baselines only; the product never calls it).
// It restates, in FP32 on host threads, what TINY_MLP::inference and the
// trainer's gradient (cuda/neural_network.cu:56-62, render_hair_msnn.cu:
// 683-691) ask of tiny-cuda-nn for the Composite encodings of the cache
// configs: Identity, Frequency (phase 2^f * x * 3.1415926 formed in FP32,
// cosine as the sine of the phase plus pi/2), OneBlob (quartic-kernel blobs
// of radius one bin, periodic on [0, 1)) and HashGrid (fmaf(scale, x, 0.5),
// trilinear over the eight corners, dense index while the level fits, else
// the (1, 2654435761, 805459861) xor hash), the encoded row padded with ones
// to a multiple of 16, then the FullyFusedMLP (ReLU hidden layers, linear
// output, weights row-major [out][in], no biases).  mlp_oracle is the FP64
// statement of the same network; tests pin this one against it.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

namespace {

constexpr float kPi = 3.1415926f;

float quartic_cdf(float x, float inv_radius) {
  const float u = x * inv_radius;
  const float u2 = u * u;
  const float u4 = u2 * u2;
  return std::min(std::max((1.0f / 16.0f) * u * (15.0f - 10.0f * u2 + 3.0f * u4) + 0.5f, 0.f), 1.f);
}

float oneblob_cdf(float boundary, float x, float nb) {
  return quartic_cdf(boundary - x, nb) + quartic_cdf(boundary - x - 1.0f, nb) +
         quartic_cdf(boundary - x + 1.0f, nb);
}

enum { SEG_IDENTITY = 0, SEG_FREQUENCY = 1, SEG_ONEBLOB = 2, SEG_HASHGRID = 3 };
constexpr int kSegInts = 8;  // type, in_off, n_dims, out_off, n_freq / n_bins / n_levels, n_feat, level base, param_off

struct Net {
  const int* seg;  // [n_segs][kSegInts]
  int n_segs, n_enc, in_pad, in_ch;
  const float* params;  // network weights, then encoding parameters
  int64_t n_net_params;
  const int* shapes;  // [n_layers][2]: out, in
  int n_layers, out_ch;
  const float* lvl_scale;  // hash-grid levels of all grid segments
  const int* lvl_res;
  const int* lvl_size;
  const int* lvl_off;
};

uint32_t grid_index(uint32_t res, uint32_t size, uint32_t x, uint32_t y, uint32_t z) {
  uint64_t stride = 1;
  uint32_t index = 0;
  const uint32_t c[3] = {x, y, z};
  for (int k = 0; k < 3; ++k) {
    if (stride > size) break;
    index = (uint32_t)(index + (uint64_t)c[k] * stride);
    stride *= res;
  }
  if (size < stride) index = x ^ (y * 2654435761u) ^ (z * 805459861u);
  return index % size;
}

// The eight corners of level l of a grid segment at p: table rows and weights.
void grid_corners(const Net& m, const int* s, int l, const float* p, int64_t* row, float* wt) {
  const int lv = s[6] + l;
  const float sc = m.lvl_scale[lv];
  float w[3];
  uint32_t g[3];
  for (int k = 0; k < 3; ++k) {
    const float f = std::fma(sc, p[k], 0.5f);
    const float fl = std::floor(f);
    w[k] = f - fl;
    g[k] = (uint32_t)(int64_t)fl;
  }
  for (int c = 0; c < 8; ++c) {
    const int b0 = c & 1, b1 = (c >> 1) & 1, b2 = (c >> 2) & 1;
    row[c] = m.lvl_off[lv] + grid_index((uint32_t)m.lvl_res[lv], (uint32_t)m.lvl_size[lv], g[0] + b0, g[1] + b1,
                                        g[2] + b2);
    wt[c] = (b0 ? w[0] : 1.f - w[0]) * (b1 ? w[1] : 1.f - w[1]) * (b2 ? w[2] : 1.f - w[2]);
  }
}

void encode_row(const Net& m, const float* x, float* X, std::vector<float>& edge) {
  for (int k = 0; k < m.in_pad; ++k) X[k] = k < m.n_enc ? 0.f : 1.f;
  for (int si = 0; si < m.n_segs; ++si) {
    const int* s = m.seg + kSegInts * si;
    const int type = s[0], in_off = s[1], n_dims = s[2], out_off = s[3], p = s[4];
    if (type == SEG_HASHGRID) {
      const int F = s[5];
      const float* table = m.params + m.n_net_params + s[7];
      int64_t row[8];
      float wt[8];
      for (int l = 0; l < p; ++l) {
        grid_corners(m, s, l, x + in_off, row, wt);
        for (int q = 0; q < F; ++q) {
          float acc = 0.f;
          for (int c = 0; c < 8; ++c) acc += wt[c] * table[row[c] * F + q];
          X[out_off + l * F + q] = acc;
        }
      }
      continue;
    }
    if (type == SEG_IDENTITY) {
      for (int d = 0; d < n_dims; ++d) X[out_off + d] = x[in_off + d];
    } else if (type == SEG_FREQUENCY) {
      for (int d = 0; d < n_dims; ++d)
        for (int f = 0; f < p; ++f) {
          const float a = (x[in_off + d] * std::ldexp(1.0f, f)) * kPi;
          X[out_off + 2 * (d * p + f)] = std::sin(a);
          X[out_off + 2 * (d * p + f) + 1] = std::sin(a + 0.5f * kPi);
        }
    } else {
      // bin b = edge(b + 1) - edge(b), edge(0) = C(0), edge(n_bins) = C(0) + 1
      const float nb = (float)p;
      edge.resize(p + 1);
      for (int d = 0; d < n_dims; ++d) {
        const float xd = x[in_off + d];
        edge[0] = oneblob_cdf(0.f, xd, nb);
        for (int b = 1; b < p; ++b) edge[b] = oneblob_cdf((float)b / nb, xd, nb);
        edge[p] = edge[0] + 1.f;
        for (int b = 0; b < p; ++b) X[out_off + d * p + b] = edge[b + 1] - edge[b];
      }
    }
  }
}

// Hidden activations of one row: acts[l] holds layer l's input (acts[0] the
// encoded row), the output goes to y [out_pad].
void forward_row(const Net& m, const float* x, std::vector<std::vector<float>>& acts, float* y,
                 std::vector<float>& edge) {
  encode_row(m, x, acts[0].data(), edge);
  const float* w = m.params;
  for (int l = 0; l < m.n_layers; ++l) {
    const int fo = m.shapes[2 * l], fi = m.shapes[2 * l + 1];
    const bool last = l == m.n_layers - 1;
    const float* a = acts[l].data();
    float* b = last ? y : acts[l + 1].data();
    for (int o = 0; o < fo; ++o) {
      const float* wr = w + (int64_t)o * fi;
      float part[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // independent sums: SIMD without reassociation
      int i = 0;
      for (; i + 8 <= fi; i += 8)
        for (int k = 0; k < 8; ++k) part[k] += wr[i + k] * a[i + k];
      float acc = ((part[0] + part[1]) + (part[2] + part[3])) + ((part[4] + part[5]) + (part[6] + part[7]));
      for (; i < fi; ++i) acc += wr[i] * a[i];
      b[o] = last ? acc : std::max(acc, 0.f);
    }
    w += (int64_t)fo * fi;
  }
}

std::vector<std::vector<float>> make_acts(const Net& m) {
  std::vector<std::vector<float>> acts(m.n_layers);
  acts[0].resize(m.in_pad);
  for (int l = 1; l < m.n_layers; ++l) acts[l].resize(m.shapes[2 * l + 1]);
  return acts;
}

void forward_rows(const Net& m, const float* x, int64_t r0, int64_t r1, float* out) {
  auto acts = make_acts(m);
  std::vector<float> y(m.shapes[2 * (m.n_layers - 1)]), edge;
  for (int64_t r = r0; r < r1; ++r) {
    forward_row(m, x + r * m.in_ch, acts, y.data(), edge);
    for (int c = 0; c < m.out_ch; ++c) out[r * m.out_ch + c] = y[c];
  }
}

// Loss gradient of rows [r0, r1) into g (weights, then encoding parameters),
// the rows' loss sum into *loss.  loss: 0 L2, 1 RelativeL2, 2
// RelativeL2Luminance (the prediction's luminance as a constant
// denominator); both averaged over total = n * out_ch.
void grad_rows(const Net& m, const float* x, const float* target, int64_t r0, int64_t r1, int loss_kind,
               double total, float* g, double* loss) {
  auto acts = make_acts(m);
  const int out_pad = m.shapes[2 * (m.n_layers - 1)];
  std::vector<float> y(out_pad), dz(out_pad), dh, edge;
  int wmax = m.in_pad;
  for (int l = 0; l < m.n_layers; ++l) wmax = std::max(wmax, m.shapes[2 * l + 1]);
  std::vector<int64_t> woff(m.n_layers);
  int64_t o = 0;
  for (int l = 0; l < m.n_layers; ++l) {
    woff[l] = o;
    o += (int64_t)m.shapes[2 * l] * m.shapes[2 * l + 1];
  }
  double lsum = 0.0;
  for (int64_t r = r0; r < r1; ++r) {
    const float* xr = x + r * m.in_ch;
    forward_row(m, xr, acts, y.data(), edge);
    std::fill(dz.begin(), dz.end(), 0.f);
    const float lum = 0.299f * y[0] + 0.587f * y[1] + 0.114f * y[2];
    for (int c = 0; c < m.out_ch; ++c) {
      const float diff = y[c] - target[r * m.out_ch + c];
      const float den = loss_kind == 0 ? 1.f : loss_kind == 1 ? y[c] * y[c] + 0.01f : lum * lum + 0.01f;
      lsum += (double)(diff * diff / den);
      dz[c] = (float)(2.0 * diff / den / total);
    }
    // back through the layers: dW_l += dz (x) acts[l], dh = W_l^T dz
    std::vector<float> cur(dz);
    for (int l = m.n_layers - 1; l >= 0; --l) {
      const int fo = m.shapes[2 * l], fi = m.shapes[2 * l + 1];
      const float* a = acts[l].data();
      const float* w = m.params + woff[l];
      float* gw = g + woff[l];
      dh.assign(fi, 0.f);
      for (int oo = 0; oo < fo; ++oo) {
        const float d = cur[oo];
        if (d == 0.f) continue;
        for (int i = 0; i < fi; ++i) {
          gw[(int64_t)oo * fi + i] += d * a[i];
          dh[i] += d * w[(int64_t)oo * fi + i];
        }
      }
      if (l > 0)
        for (int i = 0; i < fi; ++i) dh[i] = a[i] > 0.f ? dh[i] : 0.f;
      cur.assign(dh.begin(), dh.end());
    }
    // cur = dLoss/dEncoded: scattered into the hash-grid tables
    for (int si = 0; si < m.n_segs; ++si) {
      const int* s = m.seg + kSegInts * si;
      if (s[0] != SEG_HASHGRID) continue;
      const int F = s[5];
      float* tg = g + m.n_net_params + s[7];
      int64_t row[8];
      float wt[8];
      for (int l = 0; l < s[4]; ++l) {
        grid_corners(m, s, l, xr + s[1], row, wt);
        for (int c = 0; c < 8; ++c)
          for (int q = 0; q < F; ++q) tg[row[c] * F + q] += wt[c] * cur[s[3] + l * F + q];
      }
    }
  }
  *loss = lsum;
}

}  // namespace

extern "C" {

// x [n][in_ch] -> out [n][out_ch]; seg [n_segs][8] (type 0 Identity, 1
// Frequency, 2 OneBlob, 3 HashGrid; input offset, dimensions, output
// offset, n_freq / n_bins / n_levels, features per level, first level in
// the level arrays, table offset in the encoding parameters), shapes
// [n_layers][2] (out, in) of the consecutive row-major weight blocks at
// params (the encoding parameters follow them, n_net_params in).
void hmo_mlp_forward(const float* x, int64_t n, int in_ch, const int* seg, int n_segs, int n_enc, int in_pad,
                     const float* params, int64_t n_net_params, const int* shapes, int n_layers, int out_ch,
                     const float* lvl_scale, const int* lvl_res, const int* lvl_size, const int* lvl_off, float* out,
                     int threads) {
  const Net m{seg, n_segs, n_enc, in_pad, in_ch, params, n_net_params, shapes, n_layers, out_ch,
              lvl_scale, lvl_res, lvl_size, lvl_off};
  threads = std::max(1, threads);
  const int64_t per = (n + threads - 1) / threads;
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t) {
    const int64_t r0 = t * per, r1 = std::min<int64_t>(n, r0 + per);
    if (r0 >= r1) break;
    pool.emplace_back(forward_rows, std::cref(m), x, r0, r1, out);
  }
  for (auto& th : pool) th.join();
}

// The loss over n rows and its gradient with respect to every parameter
// (grads [n_params], overwritten): per-thread partial sums added in thread
// order.  Returns the loss.
double hmo_mlp_grad(const float* x, const float* target, int64_t n, int in_ch, const int* seg, int n_segs,
                    int n_enc, int in_pad, const float* params, int64_t n_net_params, int64_t n_params,
                    const int* shapes, int n_layers, int out_ch, const float* lvl_scale, const int* lvl_res,
                    const int* lvl_size, const int* lvl_off, int loss_kind, float* grads, int threads) {
  const Net m{seg, n_segs, n_enc, in_pad, in_ch, params, n_net_params, shapes, n_layers, out_ch,
              lvl_scale, lvl_res, lvl_size, lvl_off};
  if (n <= 0) {
    std::fill(grads, grads + n_params, 0.f);
    return 0.0;
  }
  threads = std::max(1, threads);
  const int64_t per = (n + threads - 1) / threads;
  const double total = (double)n * out_ch;
  std::vector<std::vector<float>> part;
  std::vector<double> loss(threads, 0.0);
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t) {
    const int64_t r0 = t * per, r1 = std::min<int64_t>(n, r0 + per);
    if (r0 >= r1) break;
    part.emplace_back(n_params, 0.f);
  }
  for (size_t t = 0; t < part.size(); ++t) {
    const int64_t r0 = t * per, r1 = std::min<int64_t>(n, r0 + per);
    pool.emplace_back(grad_rows, std::cref(m), x, target, r0, r1, loss_kind, total, part[t].data(), &loss[t]);
  }
  for (auto& th : pool) th.join();
  std::fill(grads, grads + n_params, 0.f);
  double lsum = 0.0;
  for (size_t t = 0; t < part.size(); ++t) {
    for (int64_t i = 0; i < n_params; ++i) grads[i] += part[t][i];
    lsum += loss[t];
  }
  return lsum / total;
}

}  // extern "C"
