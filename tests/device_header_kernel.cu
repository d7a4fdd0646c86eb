// User-side CUDA code built against include/hairmsnn_device.cuh by
// tests/test_gpu_device_header.py: kernels that call the reference-named
// hair BSDF functions per query (as a closest-hit routine would) and the
// head-surface GGX functions, with C launchers for ctypes.
#include "hairmsnn_device.cuh"
#include "hm_shading.cuh"

// wo, wi, t: [3][n]; h: [n] -> f [3][n], pdf [n], h_used [n] (dot(Y, n) of the vertex built here)
__global__ void dh_eval_kernel(const float* wo, const float* wi, const float* t, const float* h, hm::HairConsts hc,
                               float* f, float* pdf, float* h_used, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  HairVertex v;
  const float3 w_o = make_float3(wo[i], wo[n + i], wo[2 * n + i]);
  const float3 tg = make_float3(t[i], t[n + i], t[2 * n + i]);
  // a normal with dot(Y, n) = h: n = h Y + sqrt(1 - h^2) Z
  HairVertex tmp;
  hairVertexFrame(tmp, w_o, tg, make_float3(0.f, 0.f, 0.f));
  const float c = sqrtf(fmaxf(0.f, 1.f - h[i] * h[i]));
  const float3 nrm = make_float3(h[i] * tmp.to_local[1].x + c * tmp.to_local[2].x,
                                 h[i] * tmp.to_local[1].y + c * tmp.to_local[2].y,
                                 h[i] * tmp.to_local[1].z + c * tmp.to_local[2].z);
  hairVertexFrame(v, w_o, tg, nrm);
  v.hair = hc;
  v.wi = make_float3(wi[i], wi[n + i], wi[2 * n + i]);
  const hm::Frame fr{hm::mk(v.to_local[0].x, v.to_local[0].y, v.to_local[0].z),
                     hm::mk(v.to_local[1].x, v.to_local[1].y, v.to_local[1].z),
                     hm::mk(v.to_local[2].x, v.to_local[2].y, v.to_local[2].z)};
  const hm::f3 wl = hm::normalize(hm::to_local(fr, hm::mk(v.wi.x, v.wi.y, v.wi.z)));
  v.wi_local = make_float3(wl.x, wl.y, wl.z);
  float p = 0.f;
  const float3 r = disney_hair(v, &p);
  f[i] = r.x; f[n + i] = r.y; f[2 * n + i] = r.z;
  pdf[i] = p;
  h_used[i] = hm::dot(fr.r1, hm::mk(nrm.x, nrm.y, nrm.z));
}

__global__ void dh_sample_kernel(const float* wo, const float* t, const float* h, const float* u, hm::HairConsts hc,
                                 float* wi, float* f, float* pdf, float* h_used, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  HairVertex tmp, v;
  const float3 w_o = make_float3(wo[i], wo[n + i], wo[2 * n + i]);
  const float3 tg = make_float3(t[i], t[n + i], t[2 * n + i]);
  hairVertexFrame(tmp, w_o, tg, make_float3(0.f, 0.f, 0.f));
  const float c = sqrtf(fmaxf(0.f, 1.f - h[i] * h[i]));
  const float3 nrm = make_float3(h[i] * tmp.to_local[1].x + c * tmp.to_local[2].x,
                                 h[i] * tmp.to_local[1].y + c * tmp.to_local[2].y,
                                 h[i] * tmp.to_local[1].z + c * tmp.to_local[2].z);
  hairVertexFrame(v, w_o, tg, nrm);
  v.hair = hc;
  const float4 rnd = make_float4(u[i], u[n + i], u[2 * n + i], u[3 * n + i]);
  float p = 0.f;
  const float3 r = sample_disney_hair(v, rnd, &p);
  wi[i] = v.wi.x; wi[n + i] = v.wi.y; wi[2 * n + i] = v.wi.z;
  f[i] = r.x; f[n + i] = r.y; f[2 * n + i] = r.z;
  pdf[i] = p;
  h_used[i] = v.to_local[1].x * nrm.x + v.to_local[1].y * nrm.y + v.to_local[1].z * nrm.z;
}

// GGX of the head surface (frostbite_anisotropic.cuh:84-157), local frame,
// [n][3] rows: f, sampled L and its pdf, pdf of the half vector of (wo, wi).
__global__ void dh_ggx_kernel(const float* wo, const float* wi, const float* color, const float* alpha,
                              const float* r2, float* f, float* L, float* pdf, float* hpdf, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const hm::f3 o = hm::mk(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
  const hm::f3 w = hm::mk(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
  const hm::f3 col = hm::mk(color[3 * i], color[3 * i + 1], color[3 * i + 2]);
  const hm::f3 r = hm::frostbite_ggx(o, w, col, alpha[i]);
  f[3 * i] = r.x; f[3 * i + 1] = r.y; f[3 * i + 2] = r.z;
  float p = 0.f;
  const hm::f3 l = hm::sample_ggx(r2[2 * i], r2[2 * i + 1], alpha[i], o, &p);
  L[3 * i] = l.x; L[3 * i + 1] = l.y; L[3 * i + 2] = l.z;
  pdf[i] = p;
  hpdf[i] = hm::pdf_ggx(alpha[i], o, hm::normalize(o + w));
}

static int sync_status() { return cudaDeviceSynchronize() == cudaSuccess && cudaGetLastError() == cudaSuccess ? 0 : 1; }

extern "C" int dh_eval(const float* wo, const float* wi, const float* t, const float* h, const hm_hair_params* p,
                       float* f, float* pdf, float* h_used, int n) {
  dh_eval_kernel<<<(n + 127) / 128, 128>>>(wo, wi, t, h, hm::hair_consts(*p), f, pdf, h_used, n);
  return sync_status();
}

extern "C" int dh_sample(const float* wo, const float* t, const float* h, const float* u, const hm_hair_params* p,
                         float* wi, float* f, float* pdf, float* h_used, int n) {
  dh_sample_kernel<<<(n + 127) / 128, 128>>>(wo, t, h, u, hm::hair_consts(*p), wi, f, pdf, h_used, n);
  return sync_status();
}

extern "C" int dh_ggx(const float* wo, const float* wi, const float* color, const float* alpha, const float* r2,
                      float* f, float* L, float* pdf, float* hpdf, int n) {
  dh_ggx_kernel<<<(n + 127) / 128, 128>>>(wo, wi, color, alpha, r2, f, L, pdf, hpdf, n);
  return sync_status();
}
