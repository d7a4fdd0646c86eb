// Batched hair-BSDF kernels behind the C ABI (include/hairmsnn.h):
// hm_bsdf_eval / hm_bsdf_sample replace per-hit calls of the reference's
// disney_hair() / sample_disney_hair() (cuda_headers/disney_hair.cuh:186,277).
//
// Data layout: planar structure-of-arrays ([3][n] for vectors), one query per
// thread, so every warp-wide load or store is one contiguous 128-byte line
// per plane.  Inputs are read once through the non-coherent path and outputs
// are written with streaming stores (nothing is re-read).
#include <math.h>

#include "hm_hair_bsdf.cuh"
#include "hm_hair_grad.cuh"

namespace hm {

// setupHairShading and the other material-only terms, evaluated once on the
// host (hair_consts, hm_hair_bsdf.cuh).
HairConsts hair_consts_from_params(const hm_hair_params& p) { return hair_consts(p); }

HM_D float ldg(const float* p) { return __ldg(p); }

// Six 256-thread blocks per SM (40 registers; the eval needs 79 without
// spilling, and spills about 250 bytes to L1 at 40): the kernels wait on the
// latency of their transcendentals and dependent chains (a third of the
// issue slots used at three blocks per SM), so more warps beat the spills.
// Measured at 2^24 queries: eval 1.16 / 1.06 / 1.06 / 1.03 / 1.06 ms and
// sample 1.59 / 1.47 / 1.50 / 1.45 / 1.46 ms at 3 / 4 / 5 / 6 / 8 blocks per
// SM, results bit for bit the same.
__global__ void __launch_bounds__(256, 6) bsdf_eval_kernel(HairConsts hc, const float* __restrict__ wo,
                                                        const float* __restrict__ wi,
                                                        const float* __restrict__ t,
                                                        const float* __restrict__ h,
                                                        float* __restrict__ f,
                                                        float* __restrict__ pdf, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const f3 w_o = mk(ldg(wo + i), ldg(wo + n + i), ldg(wo + 2 * n + i));
    const f3 w_i = mk(ldg(wi + i), ldg(wi + n + i), ldg(wi + 2 * n + i));
    const f3 tg = mk(ldg(t + i), ldg(t + n + i), ldg(t + 2 * n + i));
    const Frame fr = hair_frame(w_o, tg);
    const f3 wol = normalize(to_local(fr, w_o));
    const f3 wil = normalize(to_local(fr, w_i));
    const HairEval e = hair_eval(wol, wil, ldg(h + i), hc);
    __stcs(f + i, e.f.x);
    __stcs(f + n + i, e.f.y);
    __stcs(f + 2 * n + i, e.f.z);
    __stcs(pdf + i, e.pdf);
  }
}

__global__ void __launch_bounds__(256, 6) bsdf_sample_kernel(HairConsts hc, const float* __restrict__ wo,
                                                          const float* __restrict__ t,
                                                          const float* __restrict__ h,
                                                          const float* __restrict__ u,
                                                          float* __restrict__ wi_out,
                                                          float* __restrict__ f,
                                                          float* __restrict__ pdf, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const f3 w_o = mk(ldg(wo + i), ldg(wo + n + i), ldg(wo + 2 * n + i));
    const f3 tg = mk(ldg(t + i), ldg(t + n + i), ldg(t + 2 * n + i));
    const Frame fr = hair_frame(w_o, tg);
    const f3 wol = normalize(to_local(fr, w_o));
    f3 wil;
    const HairEval e = hair_sample(wol, ldg(h + i), ldg(u + i), ldg(u + n + i), ldg(u + 2 * n + i),
                                   ldg(u + 3 * n + i), hc, &wil);
    const f3 w = normalize(to_world(fr, wil));
    __stcs(wi_out + i, w.x);
    __stcs(wi_out + n + i, w.y);
    __stcs(wi_out + 2 * n + i, w.z);
    __stcs(f + i, e.f.x);
    __stcs(f + n + i, e.f.y);
    __stcs(f + 2 * n + i, e.f.z);
    __stcs(pdf + i, e.pdf);
  }
}

// uniformSampleSphere (utils.cuh:115-121)
HM_D f3 uniform_sample_sphere(float u0, float u1) {
  float z = 1.f - 2.f * u0;
  float r = sqrtf(fmaxf(0.f, 1.f - z * z));
  float phi = 2.f * kPi * u1;
  return normalize(mk(r * cosf(phi), r * sinf(phi), z));
}

// Synthetic BSDF workload: one counter-based stream per query
// (murmur-seeded LCG of random.cuh, pixel index = query index), 11 draws:
// wo (2), wi (2), tangent (2), h (1), sampling uniforms (4).
__global__ void __launch_bounds__(256) bsdf_gen_kernel(uint32_t seed, float* __restrict__ wo,
                                                       float* __restrict__ wi,
                                                       float* __restrict__ t,
                                                       float* __restrict__ h,
                                                       float* __restrict__ u, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t st = rng_seed((int)seed, (uint32_t)i);
    float r[11];
#pragma unroll
    for (int k = 0; k < 11; ++k) r[k] = lcg_next(st);
    const f3 a = uniform_sample_sphere(r[0], r[1]);
    const f3 b = uniform_sample_sphere(r[2], r[3]);
    const f3 c = uniform_sample_sphere(r[4], r[5]);
    wo[i] = a.x; wo[n + i] = a.y; wo[2 * n + i] = a.z;
    if (wi) { wi[i] = b.x; wi[n + i] = b.y; wi[2 * n + i] = b.z; }
    t[i] = c.x; t[n + i] = c.y; t[2 * n + i] = c.z;
    h[i] = 2.f * r[6] - 1.f;
    if (u) {
#pragma unroll
      for (int k = 0; k < 4; ++k) u[k * n + i] = r[7 + k];
    }
  }
}

static int grid_for(int64_t n, int block) {
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int64_t blocks = (n + block - 1) / block;
  int64_t cap = (int64_t)sms * 16;  // persistent-enough grid: 16 x 256-thread CTAs per SM
  return (int)(blocks < cap ? blocks : cap);
}

}  // namespace hm

using namespace hm;

static int check_params(const hm_hair_params* p) {
  if (!p) {
    hm_set_error("hair params are NULL");
    return HM_EINVAL;
  }
  if (!(p->beta_m > 0.f) || !(p->beta_n > 0.f)) {
    hm_set_error("beta_m and beta_n must be > 0 (got %g, %g)", p->beta_m, p->beta_n);
    return HM_EINVAL;
  }
  return HM_OK;
}

extern "C" int hm_bsdf_eval(const hm_bsdf_queries* q, float* f, float* pdf, int64_t n,
                            const hm_hair_params* params, void* stream) {
  if (n < 0 || !q) return hm_set_error("hm_bsdf_eval: n < 0 or queries NULL"), HM_EINVAL;
  if (int s = check_params(params)) return s;
  if (n == 0) return HM_OK;
  if (!q->wo || !q->wi || !q->tangent || !q->h || !f || !pdf)
    return hm_set_error("hm_bsdf_eval: NULL array"), HM_EINVAL;
  HairConsts hc = hair_consts_from_params(*params);
  bsdf_eval_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(hc, q->wo, q->wi, q->tangent,
                                                                        q->h, f, pdf, n);
  HM_CHECK_LAUNCH("bsdf_eval_kernel");
  return HM_OK;
}

// f, pdf and their partials with respect to (sigma_a r, g, b, beta_m, beta_n,
// alpha): df [6][3][n], dpdf [6][n] (dpdf may be NULL).
__global__ void __launch_bounds__(256) bsdf_eval_grad_kernel(hm_hair_params p, const float* __restrict__ wo,
                                                             const float* __restrict__ wi,
                                                             const float* __restrict__ t,
                                                             const float* __restrict__ h,
                                                             float* __restrict__ f, float* __restrict__ pdf,
                                                             float* __restrict__ df, float* __restrict__ dpdf,
                                                             int64_t n) {
  const float gain[4] = {p.gain_r, p.gain_tt, p.gain_trt, p.gain_trrt};
  const HairConstsD hc = hair_consts_dual(p.sigma_a, p.beta_m, p.beta_n, p.alpha, gain);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const f3 w_o = mk(ldg(wo + i), ldg(wo + n + i), ldg(wo + 2 * n + i));
    const f3 w_i = mk(ldg(wi + i), ldg(wi + n + i), ldg(wi + 2 * n + i));
    const f3 tg = mk(ldg(t + i), ldg(t + n + i), ldg(t + 2 * n + i));
    const Frame fr = hair_frame(w_o, tg);
    const HairEvalD e = hair_eval_dual(normalize(to_local(fr, w_o)), normalize(to_local(fr, w_i)), ldg(h + i), hc);
    for (int c = 0; c < 3; ++c) {
      f[c * n + i] = e.f[c].v;
      for (int j = 0; j < kNd; ++j) df[(j * 3 + c) * n + i] = e.f[c].d[j];
    }
    pdf[i] = e.pdf.v;
    if (dpdf)
      for (int j = 0; j < kNd; ++j) dpdf[j * n + i] = e.pdf.d[j];
  }
}

extern "C" int hm_bsdf_eval_grad(const hm_bsdf_queries* q, float* f, float* pdf, float* df, float* dpdf, int64_t n,
                                 const hm_hair_params* params, void* stream) {
  if (n < 0 || !q) return hm_set_error("hm_bsdf_eval_grad: n < 0 or queries NULL"), HM_EINVAL;
  if (int s = check_params(params)) return s;
  if (n == 0) return HM_OK;
  if (!q->wo || !q->wi || !q->tangent || !q->h || !f || !pdf || !df)
    return hm_set_error("hm_bsdf_eval_grad: NULL array"), HM_EINVAL;
  bsdf_eval_grad_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(*params, q->wo, q->wi, q->tangent, q->h,
                                                                             f, pdf, df, dpdf, n);
  HM_CHECK_LAUNCH("bsdf_eval_grad_kernel");
  return HM_OK;
}

extern "C" int hm_bsdf_sample(const hm_bsdf_queries* q, float* wi_out, float* f, float* pdf,
                              int64_t n, const hm_hair_params* params, void* stream) {
  if (n < 0 || !q) return hm_set_error("hm_bsdf_sample: n < 0 or queries NULL"), HM_EINVAL;
  if (int s = check_params(params)) return s;
  if (n == 0) return HM_OK;
  if (!q->wo || !q->tangent || !q->h || !q->u || !wi_out || !f || !pdf)
    return hm_set_error("hm_bsdf_sample: NULL array"), HM_EINVAL;
  HairConsts hc = hair_consts_from_params(*params);
  bsdf_sample_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(
      hc, q->wo, q->tangent, q->h, q->u, wi_out, f, pdf, n);
  HM_CHECK_LAUNCH("bsdf_sample_kernel");
  return HM_OK;
}

extern "C" int hm_bsdf_gen_queries(uint32_t seed, int64_t n, float* wo, float* wi, float* tangent,
                                   float* h, float* u, void* stream) {
  if (n < 0 || !wo || !tangent || !h) return hm_set_error("hm_bsdf_gen_queries: bad args"), HM_EINVAL;
  if (n == 0) return HM_OK;
  bsdf_gen_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(seed, wo, wi, tangent, h, u, n);
  HM_CHECK_LAUNCH("bsdf_gen_kernel");
  return HM_OK;
}

extern "C" int hm_hair_setup(const hm_hair_params* params, float* out10) {
  if (int s = check_params(params)) return s;
  if (!out10) return hm_set_error("hm_hair_setup: out NULL"), HM_EINVAL;
  HairConsts hc = hair_consts_from_params(*params);
  for (int i = 0; i < 3; ++i) out10[i] = hc.v[i];
  out10[3] = hc.s;
  for (int i = 0; i < 3; ++i) out10[4 + i] = hc.sin2k[i];
  for (int i = 0; i < 3; ++i) out10[7 + i] = hc.cos2k[i];
  return HM_OK;
}
