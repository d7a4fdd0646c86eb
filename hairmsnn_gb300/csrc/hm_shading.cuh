// Per-vertex shading of the wavefront integrator: the reference's closest-hit
// programs, environment light, light/BSDF sampling with MIS and next-vertex
// sampling (cuda_headers/optix_common.cuh:10-309,527-616,
// cuda_headers/curve_utils.cuh:57-256, cuda/hair_msnn.cu:18-65), restated
// for SoA wavefront kernels.  Shadow-ray visibility is resolved by a later
// kernel, so light and BSDF samples return their contribution together with
// the shadow ray that gates it.
#pragma once
#include "hm_hair_bsdf.cuh"
#include "hm_scene.h"
#include "hm_trace.cuh"

namespace hm {

// ------------------------------------------------------------ small helpers
HM_D int clampi(int x, int lo, int hi) { return x < lo ? lo : (x > hi ? hi : x); }

// orthonormalBasis (utils.cuh:232-259): `a` is a float computed in double.
HM_D void orthonormal_basis(f3 n, Frame* fr) {
  f3 c1, c2;
  if (n.z < -0.999999f) {
    c1 = mk(0.f, -1.f, 0.f);
    c2 = mk(-1.f, 0.f, 0.f);
  } else {
    float a = (float)(1. / (1. + (double)n.z));
    float b = -n.x * n.y * a;
    c1 = normalize(mk((float)(1. - (double)(n.x * n.x * a)), b, -n.x));
    c2 = normalize(mk(b, (float)(1. - (double)(n.y * n.y * a)), -n.y));
  }
  fr->r0 = c1;
  fr->r1 = c2;
  fr->r2 = n;
}

HM_D float spherical_phi(f3 v) {  // utils.cuh:269-273
  float p = atan2f(v.y, v.x);
  return (p < 0.f) ? (p + 2.f * kPi) : p;
}
HM_D float power_heuristic(float f, float g) { return (f * f) / (f * f + g * g); }  // utils.cuh:290-293

// ------------------------------------------------------------ texture reads
// CUDA texture semantics with normalised coordinates and clamp addressing;
// nearest: texel floor(u * w); linear: bilinear around u * w - 0.5.
HM_D float tex_nearest(const float* t, int w, int h, float u, float v) {
  int x = clampi((int)floorf(u * (float)w), 0, w - 1);
  int y = clampi((int)floorf(v * (float)h), 0, h - 1);
  return __ldg(t + y * w + x);
}
HM_D f3 tex_linear(const float4* t, int w, int h, float u, float v) {
  float xb = u * (float)w - 0.5f, yb = v * (float)h - 0.5f;
  float fx = floorf(xb), fy = floorf(yb);
  float ax = xb - fx, ay = yb - fy;
  int x0 = (int)fx, y0 = (int)fy;
  auto fetch = [&](int x, int y) {
    float4 c = __ldg(t + clampi(y, 0, h - 1) * w + clampi(x, 0, w - 1));
    return mk(c.x, c.y, c.z);
  };
  f3 a = fetch(x0, y0), b = fetch(x0 + 1, y0), c = fetch(x0, y0 + 1), d = fetch(x0 + 1, y0 + 1);
  return (1.f - ay) * ((1.f - ax) * a + ax * b) + ay * ((1.f - ax) * c + ax * d);
}

// ------------------------------------------------------------ environment
HM_D f3 env_radiance(const SceneDev& s, f3 dir) {  // getEnvironmentRadiance :10-24
  if (!s.has_env) return splat(0.f);
  float theta = acosf(dir.z);
  float phi = spherical_phi(dir) + s.env_rot_phi;
  if (phi > kTwoPiRef) phi = phi - kTwoPiRef;
  float x = phi / (2.f * kPi);
  float y = theta / kPi;
  return s.env_scale * tex_linear(s.env, s.env_w, s.env_h, x, y);
}

HM_D float env_pdf(const SceneDev& s, f3 wi) {  // getEnvironmentPdf :26-64
  if (!s.env_pdf_sampling) return 1.f / (4.f * kPi);
  const float width = (float)s.env_w, height = (float)s.env_h;
  float theta = acosf(wi.z);
  float phi = spherical_phi(wi) + s.env_rot_phi;
  if (phi > kTwoPiRef) phi = phi - kTwoPiRef;
  float u = phi / (2.f * kPi);
  float v = theta / kPi;
  int iu = clampi((int)(u * s.env_w), 0, s.env_w - 1);
  int iv = clampi((int)(v * s.env_h), 0, s.env_h - 1);
  const int cw = s.env_w + 1;
  float cdf_last_u = tex_nearest(s.cpdf, cw, s.env_h, 1.f, iv / height);
  float cdf_last_v = tex_nearest(s.mpdf, s.env_h + 1, 1, 1.f, 0.f);
  float sin_theta = sinf(theta);
  float denom = (2.f * kPi * kPi * sin_theta) * cdf_last_u * cdf_last_v;
  float cdf_u = tex_nearest(s.cpdf, cw, s.env_h, iu / width, iv / height);
  float cdf_v = tex_nearest(s.mpdf, s.env_h + 1, 1, iv / height, 0.f);
  return denom != 0.f ? (cdf_u * cdf_v) / denom : 0.f;
}

// std::lower_bound over a CDF texture row (the lambda in sampleEnvironmentLight :72-89)
HM_D int cdf_lower_bound(float u, const float* cdf, int tw, int th, float y, float size) {
  int first = 0, count = (int)size;
  while (count > 0) {
    int step = count >> 1;
    int middle = first + step;
    if (tex_nearest(cdf, tw, th, middle / size, y) < u) {
      first = middle + 1;
      count -= step + 1;
    } else {
      count = step;
    }
  }
  return max(0, first - 1);
}

// sampleEnvironmentLight :66-149.  Returns radiance, writes wi (world) and pdf.
HM_D f3 env_sample(const SceneDev& s, uint32_t& rng, f3* wi, float* pdf) {
  if (s.env_pdf_sampling) {
    float ux = lcg_next(rng), uy = lcg_next(rng);
    const float width = (float)s.env_w, height = (float)s.env_h;
    const int cw = s.env_w + 1, mh = s.env_h + 1;
    int iv = cdf_lower_bound(uy, s.mcdf, mh, 1, 0.f, height);
    float cdf_v = tex_nearest(s.mcdf, mh, 1, iv / height, 0.f);
    float cdf_next_v = tex_nearest(s.mcdf, mh, 1, (iv + 1) / height, 0.f);
    float dv = (cdf_next_v - uy) / (cdf_next_v - cdf_v);
    float v = (iv + dv) / height;
    int iu = cdf_lower_bound(ux, s.ccdf, cw, s.env_h, iv / height, width);
    float cdf_u = tex_nearest(s.ccdf, cw, s.env_h, iu / width, iv / height);
    float cdf_next_u = tex_nearest(s.ccdf, cw, s.env_h, (iu + 1) / width, iv / height);
    float du = (cdf_next_u - ux) / (cdf_next_u - cdf_u);
    float u = (iu + du) / width;
    f3 rval = s.env_scale * tex_linear(s.env, s.env_w, s.env_h, u, v);
    float cdf_last_u = tex_nearest(s.cpdf, cw, s.env_h, 1.f, iv / height);
    float cdf_last_v = tex_nearest(s.mpdf, mh, 1, 1.f, 0.f);
    float pu = tex_nearest(s.cpdf, cw, s.env_h, iu / width, iv / height);
    float pv = tex_nearest(s.mpdf, mh, 1, iv / height, 0.f);
    float theta = kPi * v;
    float sin_theta = sinf(theta);
    float denom = (2.f * kPi * kPi * sin_theta) * cdf_last_u * cdf_last_v;
    *pdf = denom != 0.f ? (pu * pv) / denom : 0.f;
    float phi = 2.f * kPi * u - s.env_rot_phi;
    if (phi < 0.f) phi = kTwoPiRef + phi;
    *wi = mk(sin_theta * cosf(phi), sin_theta * sinf(phi), cosf(theta));
    return rval;
  }
  float u0 = lcg_next(rng), u1 = lcg_next(rng);
  float z = 1.f - 2.f * u0;
  float r = sqrtf(fmaxf(0.f, 1.f - z * z));
  float ph = 2.f * kPi * u1;
  *wi = normalize(mk(r * cosf(ph), r * sinf(ph), z));
  *pdf = 1.f / (4.f * kPi);
  return env_radiance(s, *wi);
}

// ------------------------------------------------------------ GGX (frostbite_anisotropic.cuh)
HM_D float ggx_d(float ax, float ay, f3 N) {
  float t1 = N.x / ax, t2 = N.y / ay, t3 = N.z;
  return 1.0f / (kPi * ax * ay * powf(t1 * t1 + t2 * t2 + t3 * t3, 2.0f));
}
HM_D float ggx_lambda(float ax, float ay, f3 V) {
  float t1 = V.x * ax, t2 = V.y * ay, t3 = V.z;
  return 0.5f * (-1.0f + sqrtf(1.0f + (t1 * t1 + t2 * t2) / (t3 * t3)));
}
HM_D float ggx_g1(float a, f3 V) { return V.z <= 0.f ? 0.f : 1.0f / (1.0f + ggx_lambda(a, a, V)); }
HM_D float ggx_g2(float a, f3 V, f3 L) {
  if (V.z <= 0.0f || L.z <= 0.0f) return 0.0f;
  return 1.0f / (1.0f + ggx_lambda(a, a, V) + ggx_lambda(a, a, L));
}
HM_D f3 frostbite_ggx(f3 wo, f3 wi, f3 color, float alpha) {
  f3 brdf = splat(0.f);
  if (wo.z > 0.f && wi.z > 0.f) {
    brdf = brdf + 0.5f * color / kPi;
    f3 H = normalize(wo + wi);
    float g = ggx_d(alpha, alpha, H) * ggx_g2(alpha, wo, wi) / 4.0f / wo.z / wi.z;
    brdf = brdf + splat(0.5f * g);
  }
  return brdf * fabsf(wi.z);
}
HM_D float pdf_ggx(float alpha, f3 V, f3 Ne) {
  float dv = ggx_g1(alpha, V) * fmaxf(0.f, dot(V, Ne)) * ggx_d(alpha, alpha, Ne) / V.z;
  return dv / (4.f * dot(V, Ne));
}
HM_D f3 sample_ggx(float u0, float u1, float alpha, f3 V, float* pdf) {
  f3 Vh = normalize(V * mk(alpha, alpha, 1.0f));
  float lensq = Vh.x * Vh.x + Vh.y * Vh.y;
  f3 T1 = lensq > 0.0f ? mk(-Vh.y, Vh.x, 0.0f) / sqrtf(lensq) : mk(1.0f, 0.0f, 0.0f);
  f3 T2 = cross(Vh, T1);
  float r = sqrtf(u0);
  float phi = 2.0f * kPi * u1;
  float t1 = r * cosf(phi);
  float t2 = r * sinf(phi);
  float s = 0.5f * (1.0f + Vh.z);
  t2 = (1.0f - s) * sqrtf(1.0f - t1 * t1) + s * t2;
  f3 Nh = t1 * T1 + t2 * T2 + sqrtf(fmaxf(0.0f, 1.0f - t1 * t1 - t2 * t2)) * Vh;
  f3 N = normalize(mk(alpha * Nh.x, alpha * Nh.y, fmaxf(0.0f, Nh.z)));
  f3 L = -V + 2.0f * N * dot(V, N);
  *pdf = pdf_ggx(alpha, V, N);
  return normalize(L);
}

// ------------------------------------------------------------ curves
struct Cubic {
  float4 p[4];
};
HM_D float4 f4add(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
HM_D float4 f4mul(float s, float4 a) { return make_float4(s * a.x, s * a.y, s * a.z, s * a.w); }
HM_D float4 f4div(float4 a, float s) { return make_float4(a.x / s, a.y / s, a.z / s, a.w / s); }
HM_D Cubic cubic_from_catrom(const float4* q) {  // curve_utils.cuh:62-73
  Cubic c;
  c.p[0] = f4div(f4add(f4add(f4add(f4mul(-1.0f, q[0]), f4mul(3.0f, q[1])), f4mul(-3.0f, q[2])), f4mul(1.0f, q[3])), 2.0f);
  c.p[1] = f4div(f4add(f4add(f4add(f4mul(2.0f, q[0]), f4mul(-5.0f, q[1])), f4mul(4.0f, q[2])), f4mul(-1.0f, q[3])), 2.0f);
  c.p[2] = f4div(f4add(f4mul(-1.0f, q[0]), f4mul(1.0f, q[2])), 2.0f);
  c.p[3] = f4div(f4mul(2.0f, q[1]), 2.0f);
  return c;
}
HM_D Cubic cubic_from_bspline(const float4* q) {  // uniform cubic B-spline, power basis
  Cubic c;
  c.p[0] = f4div(f4add(f4add(f4add(f4mul(-1.0f, q[0]), f4mul(3.0f, q[1])), f4mul(-3.0f, q[2])), f4mul(1.0f, q[3])), 6.0f);
  c.p[1] = f4div(f4add(f4add(f4mul(3.0f, q[0]), f4mul(-6.0f, q[1])), f4mul(3.0f, q[2])), 6.0f);
  c.p[2] = f4div(f4add(f4mul(-3.0f, q[0]), f4mul(3.0f, q[2])), 6.0f);
  c.p[3] = f4div(f4add(f4add(f4mul(1.0f, q[0]), f4mul(4.0f, q[1])), f4mul(1.0f, q[2])), 6.0f);
  return c;
}
HM_D float4 cubic_pos(const Cubic& c, float u) {
  return f4add(f4mul(u, f4add(f4mul(u, f4add(f4mul(u, c.p[0]), c.p[1])), c.p[2])), c.p[3]);
}
HM_D float4 cubic_vel(const Cubic& c, float u) {
  if (u == 0.f) u = 0.000001f;
  if (u == 1.f) u = 0.999999f;
  return f4add(f4mul(u, f4add(f4mul(u, f4mul(3.0f, c.p[0])), f4mul(2.0f, c.p[1]))), c.p[2]);
}
HM_D float4 cubic_acc(const Cubic& c, float u) { return f4add(f4mul(u, f4mul(6.0f, c.p[0])), f4mul(2.0f, c.p[1])); }
HM_D f3 xyz(float4 a) { return mk(a.x, a.y, a.z); }

// surfaceNormal (curve_utils.cuh:159-197); projects *ps onto the tube.
HM_D f3 curve_surface_normal(const Cubic& bc, float u, f3* ps) {
  f3 normal;
  if (u == 0.0f) {
    normal = -xyz(cubic_vel(bc, 0.f));
  } else if (u == 1.0f) {
    normal = xyz(cubic_vel(bc, 1.f));
  } else {
    float4 p4 = cubic_pos(bc, u);
    f3 p = xyz(p4);
    float r = p4.w;
    float4 d4 = cubic_vel(bc, u);
    f3 d = xyz(d4);
    float dr = d4.w;
    float dd = dot(d, d);
    f3 o1 = *ps - p;
    o1 = o1 - (dot(o1, d) / dd) * d;
    o1 = o1 * (r / length(o1));
    *ps = p + o1;
    dd -= dot(xyz(cubic_acc(bc, u)), o1);
    normal = dd * o1 - (dr * r) * d;
  }
  return normalize(normal);
}

// ------------------------------------------------------------ vertex (closest hit)
struct Vertex {
  f3 p, n, t, wo;
  Frame fr;
  f3 wo_local;
  int surface;
  float radius;
  int group;                  // strand group (0 for the surface)
  const HairConsts* hc;       // material that samples and weighs (pdfs, MIS)
  const HairConsts* hc_eval;  // material of the BSDF values (== hc but in detached renders)
};

// The traversal's hit recomputed for its own primitive with every operation
// rounded on its own: the shading translation units are compiled without
// multiply-add contraction, while the traversal contracts (its box and leaf
// tests run fused).  The hit point, and so the shading frame and the offset
// h across the fibre, then follow from exactly the same arithmetic as in an
// FP32 host build of the same intersector: at a grazing hit on a 0.04 mm
// fibre a contracted t moved h by percents.  A leaf that the refit no longer
// hits (a contracted near-miss) keeps the traversal's values.
HM_D float4 refit_hit(const SceneDev& s, f3 ro, f3 rd, float4 hit) {
  const int prim = __float_as_int(hit.y);
  const Ray r{ro, rd, 0.f, 1e30f};
  float t = 0.f, u = 0.f, v = 0.f;
  bool ok;
  if (prim < s.n_seg) {
    const int part = clampi((int)(hit.z * (float)s.seg_split), 0, s.seg_split - 1);
    ok = curve_intersect(s, prim, part, r, 1e30f, &t, &u);
  } else {
    ok = tri_intersect(s, prim - s.n_seg, r, 1e30f, &t, &u, &v);
  }
  return ok ? make_float4(t, hit.y, u, v) : hit;
}

// hairCH (optix_common.cuh:558-599) with computeCurveIntersection
// (curve_utils.cuh:218-256); triangleMeshCH (:527-556).  `hit` is the
// refit hit (refit_hit).
HM_D Vertex setup_vertex(const SceneDev& s, f3 ro, f3 rd, const float4 hit) {
  Vertex v;
  const int prim = __float_as_int(hit.y);
  v.wo = -1.f * rd;
  if (prim < s.n_seg) {
    const float u = hit.z;
    float4 q[4];
    const float4* cp = s.cp + s.seg[prim];
#pragma unroll
    for (int k = 0; k < 4; ++k) q[k] = __ldg(cp + k);
    Cubic ip = s.shading_catrom ? cubic_from_catrom(q) : cubic_from_bspline(q);
    f3 p = ro + hit.x * rd;  // getHitPoint
    v.radius = cubic_pos(ip, u).w;
    f3 n = curve_surface_normal(ip, u, &p);
    v.n = normalize(n);
    v.t = normalize(xyz(cubic_vel(ip, u)));  // curveTangent
    v.p = p;
    f3 X = v.t;
    f3 Y = normalize(cross(v.wo, X));
    f3 Z = normalize(cross(X, Y));
    v.fr.r0 = X;
    v.fr.r1 = Y;
    v.fr.r2 = Z;
    v.surface = 0;
    v.group = s.seg_group ? (int)__ldg(s.seg_group + prim) : 0;
    v.hc = s.n_groups ? s.group_hc + v.group : &s.hair;
  } else {
    const int3 tv = ldi3(s.tri + (prim - s.n_seg));
    const float bu = hit.z, bv = hit.w;
    const f3 a = ldf3(s.vtx + tv.x), b = ldf3(s.vtx + tv.y), c = ldf3(s.vtx + tv.z);
    v.p = (1.f - bu - bv) * a + bu * b + bv * c;
    const f3 na = ldf3(s.nrm + tv.x), nb = ldf3(s.nrm + tv.y), nc = ldf3(s.nrm + tv.z);
    v.n = normalize((1.f - bu - bv) * na + bu * nb + bv * nc);
    orthonormal_basis(v.n, &v.fr);
    v.t = v.fr.r0;
    v.radius = 0.f;
    v.surface = 1;
    v.group = 0;
    v.hc = &s.hair;
  }
  v.hc_eval = v.hc;
  v.wo_local = normalize(to_local(v.fr, v.wo));
  return v;
}

// One light-transport sample whose value counts only if its shadow ray is unoccluded.
struct ShadowSample {
  f3 c;       // contribution if visible
  f3 o, d;    // shadow ray
  f3 wl;      // its direction in the vertex frame
  int valid;  // 0: no ray, contributes nothing
};

HM_D f3 bsdf_eval_vertex(const SceneDev& s, const Vertex& v, f3 wi_local, float* pdf, bool light_pdf_path) {
  if (!v.surface) {
    f3 n_local = v.n;  // unused by the eval; h is taken from the frame
    (void)n_local;
    HairEval e = hair_eval(v.wo_local, wi_local, dot(v.fr.r1, v.n), *v.hc);
    *pdf = e.pdf;
    if (v.hc_eval != v.hc) return hair_eval(v.wo_local, wi_local, dot(v.fr.r1, v.n), *v.hc_eval).f;
    return e.f;
  }
  f3 f = frostbite_ggx(v.wo_local, wi_local, s.diffuse, s.alpha);
  if (light_pdf_path) *pdf = pdf_ggx(s.alpha, v.wo_local, normalize(v.wo_local + wi_local));
  return f;
}

// sampleLights (:205-277).  `p` is the (by-reference) position of the
// directLighting copy of the vertex: pushed through the fibre for a
// lower-hemisphere direction, and seen pushed by the following sampleBSDF.
HM_D ShadowSample sample_lights(const SceneDev& s, const Vertex& v, f3* p, uint32_t& rng, bool* is_delta) {
  ShadowSample out;
  out.valid = 0;
  out.c = splat(0.f);
  *is_delta = false;
  float lightPdf = 1.f, bsdfPdf = 1.f;
  float rand = lcg_next(rng);
  int sel = (int)floorf(rand * (float)s.n_total_lights);
  f3 emit, wi;
  if (sel >= s.n_dlights) {
    lightPdf = lightPdf * 1.f / (float)s.n_total_lights;
    float envPdf = 1.f;
    emit = env_sample(s, rng, &wi, &envPdf);
    lightPdf = lightPdf * envPdf;
  } else {
    lightPdf = lightPdf * 1.f / (float)s.n_total_lights;
    const float* L = s.dlights + 6 * sel;
    emit = mk(L[3], L[4], L[5]);
    wi = normalize(mk(L[0], L[1], L[2]));
    *is_delta = true;
  }
  const f3 wi_local = normalize(to_local(v.fr, wi));
  const bool lower = dot(wi, v.n) < 0.f;
  f3 nd = v.n;
  if (v.surface && lower) return out;
  if (!v.surface && lower) {
    nd = -1.f * v.n;
    *p = *p + 2.f * v.radius * nd;
  }
  out.o = *p + 1e-3f * nd;
  out.d = wi;
  out.wl = wi_local;
  out.valid = 1;
  f3 bsdf = bsdf_eval_vertex(s, v, wi_local, &bsdfPdf, true);
  if (s.mis && !*is_delta)
    out.c = bsdf * emit * power_heuristic(lightPdf, bsdfPdf) / lightPdf;
  else
    out.c = bsdf * emit / lightPdf;
  return out;
}

// sampleBSDF (:151-203)
HM_D ShadowSample sample_bsdf(const SceneDev& s, const Vertex& v, f3* p, uint32_t& rng) {
  ShadowSample out;
  out.valid = 0;
  out.c = splat(0.f);
  float r0 = lcg_next(rng), r1 = lcg_next(rng);
  float bsdfPdf = 1.f;
  f3 bsdf, wi_local;
  if (!v.surface) {
    float r2 = lcg_next(rng), r3 = lcg_next(rng);
    HairEval e = hair_sample(v.wo_local, dot(v.fr.r1, v.n), r0, r1, r2, r3, *v.hc, &wi_local);
    bsdf = e.f;
    bsdfPdf = e.pdf;
    if (v.hc_eval != v.hc) bsdf = hair_eval(v.wo_local, wi_local, dot(v.fr.r1, v.n), *v.hc_eval).f;
  } else {
    wi_local = sample_ggx(r0, r1, s.alpha, v.wo_local, &bsdfPdf);
    bsdf = frostbite_ggx(v.wo_local, wi_local, s.diffuse, s.alpha);
  }
  const f3 wi = normalize(to_world(v.fr, wi_local));
  const bool lower = dot(wi, v.n) < 0.f;
  f3 nd = v.n;
  if (v.surface && lower) return out;
  if (!v.surface && lower) {
    nd = -1.f * v.n;
    *p = *p + 2.f * v.radius * nd;
  }
  out.o = *p + 1e-3f * nd;
  out.d = wi;
  out.wl = wi_local;
  out.valid = 1;
  f3 emit = env_radiance(s, wi);
  float lightPdf = env_pdf(s, wi) * 1.f / (float)s.n_total_lights;
  if (s.mis)
    out.c = bsdf * emit * power_heuristic(bsdfPdf, lightPdf) / bsdfPdf;
  else
    out.c = bsdf * emit / bsdfPdf;
  return out;
}

// directLighting (:279-309): the two samples; the NaN check on their visible
// sum happens when the shadow rays are resolved.
HM_D void direct_lighting(const SceneDev& s, const Vertex& v, uint32_t& rng, ShadowSample out[2]) {
  f3 p = v.p;  // directLighting's by-value copy
  bool is_delta = false;
  out[0] = sample_lights(s, v, &p, rng, &is_delta);
  out[1].valid = 0;
  out[1].c = splat(0.f);
  if (s.mis && !is_delta) out[1] = sample_bsdf(s, v, &p, rng);
}

// msnnNextPathVertex / nextPathVertex (hair_msnn.cu:18-65,
// optix_common.cuh:311-360): sample, throughput factor, extension ray.
// Detached renders (v.hc_eval != v.hc) also give the factor of the sampling
// material in *mul_s; *wl receives the sampled direction in the vertex frame,
// *mul_nan whether the factor was a NaN replaced by 1 and *pdf_out the pdf
// of the sampled direction (nextPathVertexNRC's return value).
HM_D f3 next_vertex(const SceneDev& s, const Vertex& v, uint32_t& rng, f3* ro, f3* rd, f3* mul_s = nullptr,
                    f3* wl = nullptr, bool* mul_nan = nullptr, float* pdf_out = nullptr) {
  float r0 = lcg_next(rng), r1 = lcg_next(rng);
  float pdf = 1.f;
  f3 bsdf, wi_local, bsdf_s;
  if (!v.surface) {
    float r2 = lcg_next(rng), r3 = lcg_next(rng);
    HairEval e = hair_sample(v.wo_local, dot(v.fr.r1, v.n), r0, r1, r2, r3, *v.hc, &wi_local);
    bsdf = e.f;
    pdf = e.pdf;
    bsdf_s = bsdf;
    if (v.hc_eval != v.hc) bsdf = hair_eval(v.wo_local, wi_local, dot(v.fr.r1, v.n), *v.hc_eval).f;
  } else {
    wi_local = sample_ggx(r0, r1, s.alpha, v.wo_local, &pdf);
    bsdf = frostbite_ggx(v.wo_local, wi_local, s.diffuse, s.alpha);
    bsdf_s = bsdf;
  }
  const f3 wi = normalize(to_world(v.fr, wi_local));
  const bool lower = dot(wi, v.n) < 0.f;
  f3 nd = v.n;
  f3 p = v.p;
  if (lower && !v.surface) {
    nd = -1.f * v.n;
    p = p + 2.f * v.radius * nd;
  }
  f3 mul = pdf == 0.f ? bsdf : bsdf / pdf;
  const bool is_nan = isnan(mul.x) || isnan(mul.y) || isnan(mul.z);
  if (is_nan) mul = splat(1.f);
  if (mul_s) {
    *mul_s = mul;
    if (v.hc_eval != v.hc) {
      *mul_s = pdf == 0.f ? bsdf_s : bsdf_s / pdf;
      if (isnan(mul_s->x) || isnan(mul_s->y) || isnan(mul_s->z)) *mul_s = splat(1.f);
    }
  }
  if (wl) *wl = wi_local;
  if (mul_nan) *mul_nan = is_nan;
  if (pdf_out) *pdf_out = pdf;
  *ro = p + 1e-3f * nd;
  *rd = wi;  // -si.wo
  return mul;
}

}  // namespace hm
