// HairMSNN hot-path ORACLE (test infrastructure only; see hm_oracle.h).
// Scalar single-precision restatement of the reference, statement for
// statement where the floating-point result depends on the order.  Compiled
// with -ffp-contract=off so that no multiply-add is fused.
#include "hm_oracle.h"

#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <thread>
#include <vector>

#include "hm_oracle_math.h"

using namespace hmo;

int hmo::g_mp_force_fp32 = 0;
extern "C" void hmo_set_mp_force_fp32(int on) { g_mp_force_fp32 = on; }
extern "C" void hmo_set_ulp_perturb(int k) { hmo::ulp_perturb = k < -1 ? -1 : k; }

// ============================================================== RNG
extern "C" uint32_t hmo_get_rng(int frame_id, uint32_t px, uint32_t py, uint32_t dimx, uint32_t dimy) {
  return get_rng(frame_id, px, py, dimx, dimy);
}

extern "C" uint32_t hmo_lcg_stream(uint32_t state, int n, float* out) {
  for (int i = 0; i < n; ++i) out[i] = lcg_randomf(state);
  return state;
}

extern "C" uint32_t hmo_query_rng(uint32_t seed, uint32_t index) { return query_rng(seed, index); }

// ============================================================== hair BSDF
extern "C" void hmo_setup_hair(const float* hp, float* out) {
  HairShading hs = setup_hair_shading(hp);
  for (int i = 0; i < 3; ++i) out[i] = hs.v[i];
  out[3] = hs.s;
  for (int i = 0; i < 3; ++i) out[4 + i] = hs.sin2k[i];
  for (int i = 0; i < 3; ++i) out[7 + i] = hs.cos2k[i];
}

static void eval_range(int64_t b, int64_t e, const float* wo, const float* wi, const float* t,
                       const float* h, const HairShading& hs, float* f, float* pdf) {
  for (int64_t i = b; i < e; ++i) {
    HairFrame fr = hair_frame(V3(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]),
                              V3(t[3 * i], t[3 * i + 1], t[3 * i + 2]));
    V3 wil = normalize(apply_mat(fr.to_local, V3(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2])));
    float p = 0.f;
    V3 r = disney_hair(fr.wo_local, wil, h[i], hs, &p);
    f[3 * i] = r.x;
    f[3 * i + 1] = r.y;
    f[3 * i + 2] = r.z;
    pdf[i] = p;
  }
}

static void sample_range(int64_t b, int64_t e, const float* wo, const float* t, const float* h,
                         const float* u, const HairShading& hs, float* wi_out, float* f, float* pdf,
                         float* margin) {
  for (int64_t i = b; i < e; ++i) {
    HairFrame fr = hair_frame(V3(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]),
                              V3(t[3 * i], t[3 * i + 1], t[3 * i + 2]));
    float r4[4] = {u[4 * i], u[4 * i + 1], u[4 * i + 2], u[4 * i + 3]};
    float p = 0.f, mg = 0.f;
    V3 wil;
    V3 r = sample_disney_hair(fr.wo_local, h[i], r4, hs, &wil, &p, &mg);
    V3 w = normalize(apply_mat(fr.to_world, wil));
    wi_out[3 * i] = w.x;
    wi_out[3 * i + 1] = w.y;
    wi_out[3 * i + 2] = w.z;
    f[3 * i] = r.x;
    f[3 * i + 1] = r.y;
    f[3 * i + 2] = r.z;
    pdf[i] = p;
    if (margin) margin[i] = mg;
  }
}

template <class F>
static void parallel_for(int64_t n, int threads, F fn) {
  if (threads <= 1 || n < 1024) {
    fn((int64_t)0, n);
    return;
  }
  std::vector<std::thread> pool;
  int64_t chunk = (n + threads - 1) / threads;
  for (int k = 0; k < threads; ++k) {
    int64_t b = k * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    pool.emplace_back([=] { fn(b, e); });
  }
  for (auto& th : pool) th.join();
}

extern "C" void hmo_hair_eval(int64_t n, const float* wo, const float* wi, const float* t,
                              const float* h, const float* hp, float* f, float* pdf) {
  HairShading hs = setup_hair_shading(hp);
  eval_range(0, n, wo, wi, t, h, hs, f, pdf);
}

extern "C" void hmo_hair_sample(int64_t n, const float* wo, const float* t, const float* h,
                                const float* u, const float* hp, float* wi_out, float* f,
                                float* pdf, float* margin) {
  HairShading hs = setup_hair_shading(hp);
  sample_range(0, n, wo, t, h, u, hs, wi_out, f, pdf, margin);
}

extern "C" void hmo_hair_eval_mt(int64_t n, const float* wo, const float* wi, const float* t,
                                 const float* h, const float* hp, float* f, float* pdf,
                                 int threads) {
  HairShading hs = setup_hair_shading(hp);
  parallel_for(n, threads, [&](int64_t b, int64_t e) { eval_range(b, e, wo, wi, t, h, hs, f, pdf); });
}

extern "C" void hmo_hair_sample_mt(int64_t n, const float* wo, const float* t, const float* h,
                                   const float* u, const float* hp, float* wi_out, float* f,
                                   float* pdf, int threads) {
  HairShading hs = setup_hair_shading(hp);
  parallel_for(n, threads, [&](int64_t b, int64_t e) {
    sample_range(b, e, wo, t, h, u, hs, wi_out, f, pdf, nullptr);
  });
}

// Synthetic BSDF queries: per query one counter-based stream
// (get_rng(seed, (i, 0), (2^31, 1))), 11 draws in this order:
// wo (2, uniformSampleSphere), wi (2), tangent (2), h (1, mapped to [-1,1)),
// sample uniforms (4).  Outputs are planar [3][n] / [4][n] like the GPU API.
extern "C" void hmo_gen_bsdf_queries(uint32_t seed, int64_t n, float* wo, float* wi, float* t,
                                     float* h, float* u) {
  for (int64_t i = 0; i < n; ++i) {
    uint32_t st = query_rng(seed, (uint32_t)i);
    float r[11];
    for (int k = 0; k < 11; ++k) r[k] = lcg_randomf(st);
    V3 a = uniform_sample_sphere(r[0], r[1]);
    V3 b = uniform_sample_sphere(r[2], r[3]);
    V3 c = uniform_sample_sphere(r[4], r[5]);
    wo[i] = a.x; wo[n + i] = a.y; wo[2 * n + i] = a.z;
    wi[i] = b.x; wi[n + i] = b.y; wi[2 * n + i] = b.z;
    t[i] = c.x; t[n + i] = c.y; t[2 * n + i] = c.z;
    h[i] = 2.f * r[6] - 1.f;
    for (int k = 0; k < 4; ++k) u[k * n + i] = r[7 + k];
  }
}

// ============================================================== GGX
extern "C" void hmo_frostbite_ggx(const float* wo, const float* wi, const float* color, float alpha,
                                  float* out) {
  V3 r = frostbite_ggx(V3(wo[0], wo[1], wo[2]), V3(wi[0], wi[1], wi[2]),
                       V3(color[0], color[1], color[2]), alpha);
  out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

extern "C" void hmo_sample_ggx(const float* rand2, float alpha, const float* v, float* l_out,
                               float* pdf) {
  V3 L = sample_ggx(rand2[0], rand2[1], alpha, V3(v[0], v[1], v[2]), pdf);
  l_out[0] = L.x; l_out[1] = L.y; l_out[2] = L.z;
}

extern "C" float hmo_pdf_ggx(float alpha, const float* v, const float* ne) {
  return pdf_ggx(alpha, V3(v[0], v[1], v[2]), V3(ne[0], ne[1], ne[2]));
}

// ============================================================== curves
extern "C" void hmo_curve_eval(int basis, const float* q, float u, const float* ps_in, float* out) {
  V4 cp[4];
  for (int i = 0; i < 4; ++i) cp[i] = V4(q[4 * i], q[4 * i + 1], q[4 * i + 2], q[4 * i + 3]);
  Cubic c = basis == 1 ? Cubic::from_catrom(cp) : Cubic::from_bspline(cp);
  V4 p = c.position4(u), v = c.velocity4(u), a = c.acceleration4(u);
  V3 t = curve_tangent(c, u);
  V3 ps(ps_in[0], ps_in[1], ps_in[2]);
  V3 n = surface_normal(c, u, &ps);
  float vals[24] = {p.x, p.y, p.z, p.w, v.x, v.y, v.z, v.w, a.x, a.y, a.z, a.w,
                    t.x, t.y, t.z, n.x, n.y, n.z, ps.x, ps.y, ps.z, 0.f, 0.f, 0.f};
  memcpy(out, vals, sizeof(vals));
}

// ============================================================== utils
extern "C" void hmo_orthonormal_basis(const float* n, float* out) {
  V3 m[3], im[3];
  orthonormal_basis(V3(n[0], n[1], n[2]), m, im);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      out[3 * r + c] = m[r][c];
      out[9 + 3 * r + c] = im[r][c];
    }
}
extern "C" void hmo_uniform_sample_sphere(const float* u2, float* out) {
  V3 v = uniform_sample_sphere(u2[0], u2[1]);
  out[0] = v.x; out[1] = v.y; out[2] = v.z;
}
extern "C" float hmo_power_heuristic(float f, float g) { return power_heuristic(f, g); }
extern "C" float hmo_luminance(const float* rgb) { return luminance(V3(rgb[0], rgb[1], rgb[2])); }
extern "C" float hmo_spherical_theta(const float* v) { return spherical_theta(V3(v[0], v[1], v[2])); }
extern "C" float hmo_spherical_phi(const float* v) { return spherical_phi(V3(v[0], v[1], v[2])); }
