// C entry points around the reference's own header-only device math, compiled
// unmodified on the host through hm_owl_shim.h.  Built by oracle/build.py (build_ref)
// into oracle/_ref/ (never committed, never shipped); used only to generate
// and check golden vectors for the oracle restatement.
//
// Reference files included verbatim from the reference's cuda_headers/:
//   common.cuh (Interaction, HairInteraction), random.cuh, curve_utils.cuh,
//   utils.cuh, disney_hair.cuh, frostbite_anisotropic.cuh.
#include "hm_owl_shim.h"

thread_local HmShimHitContext hm_shim_ctx;
HmShimTexture hm_shim_textures[16];
extern "C" void hm_shim_trace_hook(int, const float*, const float*, float, float, void*) {}

#include "common.cuh"
#include "utils.cuh"
#include "disney_hair.cuh"
#include "frostbite_anisotropic.cuh"

namespace {

// Hair shading frame exactly as hairCH builds it (optix_common.cuh:571-583),
// plus the material fields hairCH copies (optix_common.cuh:585-598).  The
// surface normal is chosen so that dot(Y, n) = h (up to rounding).
Interaction make_hair_si(const float* wo, const float* t, float h, const float* hp) {
  Interaction si;
  si.wo = vec3f(wo[0], wo[1], wo[2]);
  si.t = vec3f(t[0], t[1], t[2]);
  vec3f X = si.t;
  vec3f Y = normalize(cross(si.wo, X));
  vec3f Z = normalize(cross(X, Y));
  si.to_local[0] = X;
  si.to_local[1] = Y;
  si.to_local[2] = Z;
  si.to_world[0] = vec3f(X.x, Y.x, Z.x);
  si.to_world[1] = vec3f(X.y, Y.y, Z.y);
  si.to_world[2] = vec3f(X.z, Y.z, Z.z);
  si.wo_local = normalize(apply_mat(si.to_local, si.wo));
  float c = sqrtf(fmaxf(0.f, 1.f - h * h));
  si.n = h * Y + c * Z;
  // hp: sigma_a[3], beta_m, beta_n, alpha(rad), gains R, TT, TRT, TRRT
  si.color = vec3f(hp[0], hp[1], hp[2]);
  si.beta_m = hp[3];
  si.beta_n = hp[4];
  si.alpha = hp[5];
  si.hair.R_G = hp[6];
  si.hair.TT_G = hp[7];
  si.hair.TRT_G = hp[8];
  si.hair.TRRT_G = hp[9];
  si.hit = true;
  si.isSurface = false;
  setupHairShading(si);
  return si;
}

}  // namespace

extern "C" {

unsigned ref_get_rng(int frame_id, unsigned px, unsigned py, unsigned dimx, unsigned dimy) {
  return get_rng(frame_id, make_uint2(px, py), make_uint2(dimx, dimy)).state;
}

unsigned ref_lcg_stream(unsigned state, int n, float* out) {
  LCGRand r;
  r.state = state;
  for (int i = 0; i < n; ++i) out[i] = lcg_randomf(r);
  return r.state;
}

// out: v[3], s, sin2kAlpha[3], cos2kAlpha[3]  (10 floats)
void ref_setup_hair(const float* hp, float* out) {
  Interaction si;
  si.beta_m = hp[3];
  si.beta_n = hp[4];
  si.alpha = hp[5];
  setupHairShading(si);
  for (int i = 0; i < 3; ++i) out[i] = si.hair.v[i];
  out[3] = si.hair.s;
  for (int i = 0; i < 3; ++i) out[4 + i] = si.hair.sin2kAlpha[i];
  for (int i = 0; i < 3; ++i) out[7 + i] = si.hair.cos2kAlpha[i];
}

// Per query i: wo, wi, t are [n][3] row-major world vectors.  Writes f[n][3],
// pdf[n] and the h the reference actually used (dot(Y, n)).
void ref_hair_eval(int n, const float* wo, const float* wi, const float* t, const float* h,
                   const float* hp, float* f, float* pdf, float* h_used) {
  for (int i = 0; i < n; ++i) {
    Interaction si = make_hair_si(wo + 3 * i, t + 3 * i, h[i], hp);
    si.wi = vec3f(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
    si.wi_local = normalize(apply_mat(si.to_local, si.wi));
    float p = 0.f;
    vec3f r = disney_hair(si, &p);
    f[3 * i] = r.x;
    f[3 * i + 1] = r.y;
    f[3 * i + 2] = r.z;
    pdf[i] = p;
    h_used[i] = dot(si.to_local[1], si.n);
  }
}

// u: [n][4] uniforms.  Writes wi[n][3] (world), f[n][3], pdf[n], h_used[n].
void ref_hair_sample(int n, const float* wo, const float* t, const float* h, const float* u,
                     const float* hp, float* wi, float* f, float* pdf, float* h_used) {
  for (int i = 0; i < n; ++i) {
    Interaction si = make_hair_si(wo + 3 * i, t + 3 * i, h[i], hp);
    vec4f r4(u[4 * i], u[4 * i + 1], u[4 * i + 2], u[4 * i + 3]);
    float p = 0.f;
    vec3f r = sample_disney_hair(si, r4, &p);
    wi[3 * i] = si.wi.x;
    wi[3 * i + 1] = si.wi.y;
    wi[3 * i + 2] = si.wi.z;
    f[3 * i] = r.x;
    f[3 * i + 1] = r.y;
    f[3 * i + 2] = r.z;
    pdf[i] = p;
    h_used[i] = dot(si.to_local[1], si.n);
  }
}

// Head-surface BRDF pieces (frostbite_anisotropic.cuh), local-frame vectors.
void ref_frostbite_ggx(const float* wo, const float* wi, const float* color, float alpha, float* out) {
  vec3f r = frostbite_GGX(vec3f(wo[0], wo[1], wo[2]), vec3f(wi[0], wi[1], wi[2]),
                          vec3f(color[0], color[1], color[2]), alpha);
  out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
void ref_sample_ggx(const float* rand2, float alpha, const float* v, float* l_out, float* pdf) {
  vec3f L = sample_GGX(vec2f(rand2[0], rand2[1]), alpha, vec3f(v[0], v[1], v[2]), pdf);
  l_out[0] = L.x; l_out[1] = L.y; l_out[2] = L.z;
}
float ref_pdf_ggx(float alpha, const float* v, const float* ne) {
  return pdf_GGX(alpha, vec3f(v[0], v[1], v[2]), vec3f(ne[0], ne[1], ne[2]));
}

// Catmull-Rom interpolator + surface projection (curve_utils.cuh).
// q: 4 control points (x,y,z,r).  out: position4, velocity4, acceleration4,
// tangent3, normal3, projected point3 (24 floats).
void ref_catrom_eval(const float* q, float u, const float* ps_in, float* out) {
  vec4f cp[4];
  for (int i = 0; i < 4; ++i) cp[i] = vec4f(q[4 * i], q[4 * i + 1], q[4 * i + 2], q[4 * i + 3]);
  CubicInterpolator ip;
  ip.initializeFromCatrom(cp);
  vec4f p = ip.position4(u), v = ip.velocity4(u), a = ip.acceleration4(u);
  vec3f t = curveTangent(ip, u);
  vec3f ps(ps_in[0], ps_in[1], ps_in[2]);
  vec3f nrm = surfaceNormal(ip, u, ps);
  float vals[24] = {p.x, p.y, p.z, p.w, v.x, v.y, v.z, v.w, a.x, a.y, a.z, a.w,
                    t.x, t.y, t.z, nrm.x, nrm.y, nrm.z, ps.x, ps.y, ps.z, 0.f, 0.f, 0.f};
  for (int i = 0; i < 24; ++i) out[i] = vals[i];
}

// utils.cuh helpers.  out: mat[9], invmat[9]
void ref_orthonormal_basis(const float* n, float* out) {
  vec3f m[3], im[3];
  orthonormalBasis(vec3f(n[0], n[1], n[2]), m, im);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      out[3 * r + c] = m[r][c];
      out[9 + 3 * r + c] = im[r][c];
    }
}
void ref_uniform_sample_sphere(const float* u2, float* out) {
  vec3f v = uniformSampleSphere(vec2f(u2[0], u2[1]));
  out[0] = v.x; out[1] = v.y; out[2] = v.z;
}
float ref_power_heuristic(float f, float g) { return powerHeuristic(1, f, 1, g); }
float ref_luminance(const float* rgb) { return luminance(vec3f(rgb[0], rgb[1], rgb[2])); }
float ref_spherical_theta(const float* v) { return sphericalTheta(vec3f(v[0], v[1], v[2])); }
float ref_spherical_phi(const float* v) { return sphericalPhi(vec3f(v[0], v[1], v[2])); }

}  // extern "C"
