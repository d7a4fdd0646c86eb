// ORACLE-side CPU transcription of the radiance-cache network's inference
// (test infrastructure and the CPU baseline of the vertex workload only; the
// product never calls it).  It restates, in FP32 on host threads, what
// TINY_MLP::inference (cuda/neural_network.cu:56-62) asks of tiny-cuda-nn
// for the Composite encodings the vertex queries use: Identity, Frequency
// (phase 2^f * x * 3.1415926 formed in FP32, cosine as the sine of the phase
// plus pi/2) and OneBlob (quartic-kernel blobs of radius one bin, periodic
// on [0, 1)), the encoded row padded with ones to a multiple of 16, then the
// FullyFusedMLP (ReLU hidden layers, linear output, weights row-major
// [out][in], no biases).  mlp_oracle.forward is the FP64 statement of the
// same network; tests pin this one against it.
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

enum { SEG_IDENTITY = 0, SEG_FREQUENCY = 1, SEG_ONEBLOB = 2 };

struct Net {
  const int* seg;  // [n_segs][5]: type, in_off, n_dims, out_off, n_freq or n_bins
  int n_segs, n_enc, in_pad, in_ch;
  const float* params;
  const int* shapes;  // [n_layers][2]: out, in
  int n_layers, out_ch;
};

void encode_row(const Net& m, const float* x, float* X, std::vector<float>& edge) {
  for (int k = 0; k < m.in_pad; ++k) X[k] = k < m.n_enc ? 0.f : 1.f;
  for (int si = 0; si < m.n_segs; ++si) {
    const int* s = m.seg + 5 * si;
    const int type = s[0], in_off = s[1], n_dims = s[2], out_off = s[3], p = s[4];
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

void forward_rows(const Net& m, const float* x, int64_t r0, int64_t r1, float* out) {
  int wmax = m.in_pad;
  for (int l = 0; l < m.n_layers; ++l) wmax = std::max(wmax, m.shapes[2 * l]);
  std::vector<float> a(wmax), b(wmax), edge;
  for (int64_t r = r0; r < r1; ++r) {
    encode_row(m, x + r * m.in_ch, a.data(), edge);
    const float* w = m.params;
    for (int l = 0; l < m.n_layers; ++l) {
      const int fo = m.shapes[2 * l], fi = m.shapes[2 * l + 1];
      const bool last = l == m.n_layers - 1;
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
      std::swap(a, b);
    }
    for (int c = 0; c < m.out_ch; ++c) out[r * m.out_ch + c] = a[c];
  }
}

}  // namespace

extern "C" {

// x [n][in_ch] -> out [n][out_ch]; seg [n_segs][5] (type 0 Identity, 1
// Frequency with n_freq, 2 OneBlob with n_bins; input offset, dimensions,
// output offset), shapes [n_layers][2] (out, in) of the consecutive
// row-major weight blocks at params.
void hmo_mlp_forward(const float* x, int64_t n, int in_ch, const int* seg, int n_segs, int n_enc, int in_pad,
                     const float* params, const int* shapes, int n_layers, int out_ch, float* out, int threads) {
  const Net m{seg, n_segs, n_enc, in_pad, in_ch, params, shapes, n_layers, out_ch};
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

}  // extern "C"
