// HairMSNN ORACLE per-vertex math (test infrastructure only).
//
// Scalar FP32 restatement of the reference's device math.  Every function
// cites the reference file:line it follows; statement order and the
// float/double promotions of the reference are kept where they change the
// rounded result (e.g. the double `0.5 *` in LogI0, the float `a` in
// orthonormalBasis).  Compile with -ffp-contract=off.
#pragma once
#include <math.h>
#include <stdint.h>

#include <cmath>

namespace hmo {

// ---- last-ulp perturbation (test infrastructure)
// The float transcendental functions of the restatement go through these
// wrappers.  With ulp_perturb = 0 (the default) they are libm's own, which is
// what the reference's host build and the golden vectors use.  Otherwise
// every result is moved by a few ulps: +1 / -1 one ulp up / down; k >= 2 a
// pseudo-random -2..+2 ulps per call, from a per-path stream (seeded by k and
// the pixel, so runs are reproducible).  The tests render a frame that way to
// see which paths depend on last-ulp differences of the transcendentals
// (where the device's functions and libm's can differ).  Set only between
// renders; read-only while one runs.
inline int ulp_perturb = 0;
inline thread_local uint32_t ulp_stream = 0;
inline void ulp_seed_path(uint32_t pixel) { ulp_stream = (uint32_t)ulp_perturb * 0x9e3779b9u ^ (pixel * 0x85ebca6bu); }
inline float nudge(float v) {
  if (ulp_perturb == 0 || !std::isfinite(v)) return v;
  int k = ulp_perturb > 0 ? 1 : -1;
  if (ulp_perturb >= 2) {
    ulp_stream = ulp_stream * 1664525u + 1013904223u;
    k = (int)((ulp_stream >> 16) % 5u) - 2;
  }
  for (; k > 0; --k) v = std::nextafter(v, INFINITY);
  for (; k < 0; ++k) v = std::nextafter(v, -INFINITY);
  return v;
}
inline float oexpf(float x) { return nudge(::expf(x)); }
inline float ologf(float x) { return nudge(::logf(x)); }
inline float osinf(float x) { return nudge(::sinf(x)); }
inline float ocosf(float x) { return nudge(::cosf(x)); }
inline float oasinf(float x) { return nudge(::asinf(x)); }
inline float oacosf(float x) { return nudge(::acosf(x)); }
inline float oatan2f(float y, float x) { return nudge(::atan2f(y, x)); }
inline float opowf(float x, float y) { return nudge(::powf(x, y)); }
inline float osinhf(float x) { return nudge(::sinhf(x)); }


// utils.cuh:10-11 — note the two different pi literals.
static const float kPi = 3.1415926f;
static const float kTwoPi = 2.f * 3.14159f;
// disney_hair.cuh:10-11
static const float kEta = 1.55f;
static const float kSqrtPiOver8 = 0.626657069f;

struct V3 {
  float x, y, z;
  V3() : x(0.f), y(0.f), z(0.f) {}
  explicit V3(float s) : x(s), y(s), z(s) {}
  V3(float a, float b, float c) : x(a), y(b), z(c) {}
  float& operator[](int i) { return (&x)[i]; }
  float operator[](int i) const { return (&x)[i]; }
};
inline V3 operator+(V3 a, V3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(V3 a, V3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline V3 operator/(V3 a, V3 b) { return V3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline V3 operator*(float s, V3 a) { return V3(s * a.x, s * a.y, s * a.z); }
inline V3 operator*(V3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
inline V3 operator/(V3 a, float s) { return V3(a.x / s, a.y / s, a.z / s); }
inline V3 operator-(V3 a) { return V3(-a.x, -a.y, -a.z); }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline float length(V3 a) { return sqrtf(dot(a, a)); }
inline V3 normalize(V3 a) { return a * (1.f / sqrtf(dot(a, a))); }
// utils.cuh:161-166
inline V3 apply_mat(const V3 m[3], V3 v) { return V3(dot(m[0], v), dot(m[1], v), dot(m[2], v)); }

struct V4 {
  float x, y, z, w;
  V4() : x(0.f), y(0.f), z(0.f), w(0.f) {}
  V4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
  V3 xyz() const { return V3(x, y, z); }
};
inline V4 operator+(V4 a, V4 b) { return V4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline V4 operator*(float s, V4 a) { return V4(s * a.x, s * a.y, s * a.z, s * a.w); }
inline V4 operator*(V4 a, float s) { return V4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline V4 operator/(V4 a, float s) { return V4(a.x / s, a.y / s, a.z / s, a.w / s); }

inline float sqr(float v) { return v * v; }                                 // disney_hair.cuh:13
inline float safe_asin(float x) { return oasinf(fminf(fmaxf(x, -1.f), 1.f)); }  // :16-18
inline float safe_sqrt(float x) { return sqrtf(fmaxf(0.f, x)); }            // :21-23

// ------------------------------------------------------------ RNG
// random.cuh:15-32
inline uint32_t murmur_mix(uint32_t hash, uint32_t k) {
  k *= 0xcc9e2d51u;
  k = (k << 15) | (k >> 17);
  k *= 0x1b873593u;
  hash ^= k;
  hash = ((hash << 13) | (hash >> 19)) * 5u + 0xe6546b64u;
  return hash;
}
// random.cuh:34-43
inline uint32_t murmur_finalize(uint32_t h) {
  h ^= h >> 16;
  h *= 0x85ebca6bu;
  h ^= h >> 13;
  h *= 0xc2b2ae35u;
  h ^= h >> 16;
  return h;
}
// random.cuh:45-56 — LCG step and its [0,1) float (u32 * 2^-32, rounded to float).
inline uint32_t lcg_random(uint32_t& s) {
  s = s * 1664525u + 1013904223u;
  return s;
}
inline float lcg_randomf(uint32_t& s) { return ldexpf((float)lcg_random(s), -32); }
// random.cuh:58-65
inline uint32_t get_rng(int frame_id, uint32_t px, uint32_t py, uint32_t dimx, uint32_t) {
  uint32_t s = murmur_mix(0u, px + py * dimx);
  s = murmur_mix(s, (uint32_t)frame_id);
  return murmur_finalize(s);
}
// Synthetic-input stream for query i: get_rng(seed, (i, 0), (2^31, 1)).
inline uint32_t query_rng(uint32_t seed, uint32_t i) { return get_rng((int)seed, i, 0u, 0x80000000u, 1u); }

// ------------------------------------------------------------ utils.cuh
inline float luminance(V3 c) { return 0.212671f * c.x + 0.715160f * c.y + 0.072169f * c.z; }  // :80-83
inline V3 uniform_sample_sphere(float u0, float u1) {                                          // :115-121
  float z = 1.f - 2.f * u0;
  float r = sqrtf(fmaxf(0.f, 1.f - z * z));
  float phi = 2.f * kPi * u1;
  return normalize(V3(r * ocosf(phi), r * osinf(phi), z));
}
inline void orthonormal_basis(V3 n, V3 mat[3], V3 inv[3]) {  // :232-259
  V3 c1, c2, c3;
  if (n.z < -0.999999f) {
    c1 = V3(0.f, -1.f, 0.f);
    c2 = V3(-1.f, 0.f, 0.f);
  } else {
    float a = (float)(1. / (1. + (double)n.z));
    float b = -n.x * n.y * a;
    c1 = normalize(V3((float)(1. - (double)(n.x * n.x * a)), b, -n.x));
    c2 = normalize(V3(b, (float)(1. - (double)(n.y * n.y * a)), -n.y));
  }
  c3 = n;
  mat[0] = c1;
  mat[1] = c2;
  mat[2] = c3;
  inv[0] = V3(c1.x, c2.x, c3.x);
  inv[1] = V3(c1.y, c2.y, c3.y);
  inv[2] = V3(c1.z, c2.z, c3.z);
}
inline float spherical_phi(V3 v) {  // :269-273
  float p = oatan2f(v.y, v.x);
  return (p < 0.f) ? (p + 2.f * kPi) : p;
}
inline float spherical_theta(V3 p) { return oacosf(p.z); }  // :275-278
inline float power_heuristic(float fp, float gp) {        // :290-293 with nf = ng = 1
  float f = fp, g = gp;
  return (f * f) / (f * f + g * g);
}

// ------------------------------------------------------------ hair BSDF
// When nonzero, the v <= 0.1 M_p branch stays in FP32 even for beta_m < 0.1
// (bit-for-bit the reference); default 0 = FP64 there for beta_m < 0.1.
extern int g_mp_force_fp32;

struct HairShading {
  float v[4];  // v[3] aliases `s` exactly like HairInteraction's layout (see sample)
  float s;
  float sin2k[3], cos2k[3];
  float sigma_a[3];
  float gain[4];  // R, TT, TRT, TRRT
  float beta_m;
};

// disney_hair.cuh:26-41 (+ the material copy of hairCH, optix_common.cuh:585-593)
inline HairShading setup_hair_shading(const float* hp) {
  HairShading hs;
  float bm = hp[3], bn = hp[4], alpha = hp[5];
  hs.v[0] = sqr(0.726f * bm + 0.812f * sqr(bm) + 3.7f * opowf(bm, 20.f));
  hs.v[1] = (float)(.25 * (double)hs.v[0]);
  hs.v[2] = 4.f * hs.v[0];
  hs.s = kSqrtPiOver8 * (0.265f * bn + 1.194f * sqr(bn) + 5.372f * opowf(bn, 22.f));
  hs.v[3] = hs.s;
  hs.sin2k[0] = osinf(alpha);
  hs.cos2k[0] = safe_sqrt(1.f - sqr(hs.sin2k[0]));
  for (int i = 1; i < 3; ++i) {
    hs.sin2k[i] = 2.f * hs.cos2k[i - 1] * hs.sin2k[i - 1];
    hs.cos2k[i] = sqr(hs.cos2k[i - 1]) - sqr(hs.sin2k[i - 1]);
  }
  for (int i = 0; i < 3; ++i) hs.sigma_a[i] = hp[i];
  for (int i = 0; i < 4; ++i) hs.gain[i] = hp[6 + i];
  hs.beta_m = g_mp_force_fp32 ? 1.f : bm;
  return hs;
}

inline float fresnel(float eta, float cos_theta) {  // disney_hair.cuh:46-51
  float F0 = sqr(1.f - eta) / sqr(1.f + eta);
  float xd = (1.f - cos_theta);
  return F0 + (1.f - F0) * xd * xd * xd * xd * xd;
}

inline float bessel_i0(float x) {  // disney_hair.cuh:54-67
  float val = 0.f, x2i = 1.f;
  int64_t ifact = 1;
  int i4 = 1;
  for (int i = 0; i < 10; ++i) {
    if (i > 1) ifact *= i;
    val += x2i / ((float)i4 * sqr((float)ifact));
    x2i *= x * x;
    i4 *= 4;
  }
  return val;
}

inline float log_i0(float x) {  // disney_hair.cuh:70-75 (the `0.5 *` is a double product)
  if (x > 12.f)
    return (float)((double)x + 0.5 * (double)(-ologf(2.f * kPi) + ologf(1.f / x) + 1.f / (8.f * x)));
  return ologf(bessel_i0(x));
}

// FP64 restatement of the v <= 0.1 branch, used when beta_m < 0.1 (where the
// single-precision cancellation between LogI0(a) and 1/v loses digits).
inline double bessel_i0_d(double x) {
  double val = 0.0, x2i = 1.0, ifact = 1.0, i4 = 1.0;
  for (int i = 0; i < 10; ++i) {
    if (i > 1) ifact *= i;
    val += x2i / (i4 * ifact * ifact);
    x2i *= x * x;
    i4 *= 4.0;
  }
  return val;
}
inline double log_i0_d(double x) {
  if (x > 12.0) return x + 0.5 * (-log(2.0 * (double)kPi) + log(1.0 / x) + 1.0 / (8.0 * x));
  return log(bessel_i0_d(x));
}

inline float mp(float cti, float cto, float sti, float sto, float v, bool fp64) {  // :78-88
  if (fp64 && v <= 0.1f) {
    double a = (double)cti * (double)cto / (double)v;
    double b = (double)sti * (double)sto / (double)v;
    double dv = v;
    return (float)exp(log_i0_d(a) - b - 1.0 / dv + 0.6931 + log(1.0 / (2.0 * dv)));
  }
  float a = cti * cto / v;
  float b = sti * sto / v;
  if (v <= 0.1f) return oexpf(log_i0(a) - b - 1.f / v + 0.6931f + ologf(1.f / (2.f * v)));
  return (oexpf(-b) * bessel_i0(a)) / (osinhf(1.f / v) * 2.f * v);
}

inline float phi_p(int p, float gamma_o, float gamma_t) {  // :112-114
  return (float)(2 * p) * gamma_t - 2.f * gamma_o + (float)p * kPi;
}
inline float logistic(float x, float s) {  // :117-120
  x = fabsf(x);
  return oexpf(-x / s) / (s * sqr(1.f + oexpf(-x / s)));
}
inline float logistic_cdf(float x, float s) { return 1.f / (1.f + oexpf(-x / s)); }  // :123-125
inline float trimmed_logistic(float x, float s, float a, float b) {                 // :128-130
  return logistic(x, s) / (logistic_cdf(b, s) - logistic_cdf(a, s));
}
inline float np(float phi, int p, float s, float gamma_o, float gamma_t) {  // :133-139
  float dphi = phi - phi_p(p, gamma_o, gamma_t);
  while (dphi > kPi) dphi -= 2.f * kPi;
  while (dphi < -kPi) dphi += 2.f * kPi;
  return trimmed_logistic(dphi, s, -kPi, kPi);
}

struct Ap {
  V3 a[4];
};
inline Ap attenuation(float f, V3 T) {  // Ap0..ApMax, :91-109
  Ap r;
  r.a[0] = V3(f);
  r.a[1] = sqr(1.f - f) * T;
  r.a[2] = sqr(1.f - f) * T * T * f;
  r.a[3] = r.a[2] * f * T / (V3(1.f) - T * f);
  return r;
}

inline void ap_pdf(const HairShading& hs, float sin_to, float cos_to, float cos_go, float eta,
                   float h, float out[4]) {  // computeApPdf :143-182
  float sin_tt = sin_to / eta;
  float cos_tt = safe_sqrt(1.f - sqr(sin_tt));
  float etap = sqrtf(eta * eta - sqr(sin_to)) / cos_to;
  float sin_gt = h / etap;
  float cos_gt = safe_sqrt(1.f - sqr(sin_gt));
  float fac = (2.f * cos_gt / cos_tt);
  V3 T(oexpf(-hs.sigma_a[0] * fac), oexpf(-hs.sigma_a[1] * fac), oexpf(-hs.sigma_a[2] * fac));
  float fr = fresnel(eta, cos_to * cos_go);
  Ap ap = attenuation(fr, T);
  for (int p = 0; p < 4; ++p) out[p] = (ap.a[p].x + ap.a[p].y + ap.a[p].z) / 3.f;
  float sum = out[0] + out[1] + out[2] + out[3];
  for (int p = 0; p < 4; ++p) out[p] = out[p] / sum;
}

// disney_hair(si, &pdf) :186-266 — wo, wi in the hair frame; h = dot(Y, n).
inline V3 disney_hair(V3 wo, V3 wi, float h, const HairShading& hs, float* pdf) {
  const bool fp64 = hs.beta_m < 0.1f;
  float sin_to = wo.x;
  float cos_to = safe_sqrt(1.f - sqr(sin_to));
  float phi_o = oatan2f(wo.z, wo.y);
  float sin_ti = wi.x;
  float cos_ti = safe_sqrt(1.f - sqr(sin_ti));
  float phi_i = oatan2f(wi.z, wi.y);
  float sin_tt = sin_to / kEta;
  float cos_tt = safe_sqrt(1.f - sqr(sin_tt));
  float gamma_o = oasinf(h);
  float cos_go = ocosf(gamma_o);
  float etap = sqrtf(kEta * kEta - sqr(sin_to)) / cos_to;
  float sin_gt = h / etap;
  float cos_gt = safe_sqrt(1.f - sqr(sin_gt));
  float gamma_t = safe_asin(sin_gt);
  float fac = (2.f * cos_gt / cos_tt);
  V3 T(oexpf(-hs.sigma_a[0] * fac), oexpf(-hs.sigma_a[1] * fac), oexpf(-hs.sigma_a[2] * fac));
  float fr = fresnel(kEta, cos_to * cos_go);
  Ap ap = attenuation(fr, T);
  float phi = phi_i - phi_o;
  V3 f(0.f);

  float sop = sin_to * hs.cos2k[1] - cos_to * hs.sin2k[1];
  float cop = fabsf(cos_to * hs.cos2k[1] + sin_to * hs.sin2k[1]);
  float mp0 = mp(cos_ti, cop, sin_ti, sop, hs.v[0], fp64);
  float np0 = np(phi, 0, hs.s, gamma_o, gamma_t);
  f = f + hs.gain[0] * mp0 * ap.a[0] * np0;

  sop = sin_to * hs.cos2k[0] + cos_to * hs.sin2k[0];
  cop = fabsf(cos_to * hs.cos2k[0] - sin_to * hs.sin2k[0]);
  float mp1 = mp(cos_ti, cop, sin_ti, sop, hs.v[1], fp64);
  float np1 = np(phi, 1, hs.s, gamma_o, gamma_t);
  f = f + hs.gain[1] * mp1 * ap.a[1] * np1;

  sop = sin_to * hs.cos2k[2] + cos_to * hs.sin2k[2];
  cop = fabsf(cos_to * hs.cos2k[2] - sin_to * hs.sin2k[2]);
  float mp2 = mp(cos_ti, cop, sin_ti, sop, hs.v[2], fp64);
  float np2 = np(phi, 2, hs.s, gamma_o, gamma_t);
  f = f + hs.gain[2] * mp2 * ap.a[2] * np2;

  float mpm = mp(cos_ti, cos_to, sin_ti, sin_to, hs.v[2], fp64);
  float npm = 1.f / (2.f * kPi);
  f = f + hs.gain[3] * mpm * ap.a[3] * npm;

  float apdf[4];
  ap_pdf(hs, sin_to, cos_to, cos_go, kEta, h, apdf);
  float p = 0.f;
  p = p + mp0 * apdf[0] * np0;
  p = p + mp1 * apdf[1] * np1;
  p = p + mp2 * apdf[2] * np2;
  p = p + mpm * apdf[3] * npm;
  *pdf = p;
  return f;
}

inline float sample_trimmed_logistic(float u, float s, float a, float b) {  // :269-274
  float k = logistic_cdf(b, s) - logistic_cdf(a, s);
  float x = -s * ologf(1.f / (u * k + logistic_cdf(a, s)) - 1.f);
  return fminf(fmaxf(x, a), b);
}

// sample_disney_hair :277-386.  Lobe p = 3 (TRRT) reads v[3], which in the
// reference's HairInteraction is the field right after v[2], i.e. `s`.
inline V3 sample_disney_hair(V3 wo, float h, const float r[4], const HairShading& hs,
                             V3* wi_local, float* pdf, float* margin) {
  float sin_to = wo.x;
  float cos_to = safe_sqrt(1.f - sqr(sin_to));
  float phi_o = oatan2f(wo.z, wo.y);
  float gamma_o = oasinf(h);
  float cos_go = ocosf(gamma_o);
  float apdf[4];
  ap_pdf(hs, sin_to, cos_to, cos_go, kEta, h, apdf);
  int p = 0;
  float eps1 = r[0];
  float mg = fabsf(eps1);
  for (p = 0; p < 3; ++p) {
    mg = fminf(mg, fabsf(eps1 - apdf[p]));
    if (eps1 < apdf[p]) break;
    eps1 -= apdf[p];
  }
  if (margin) *margin = mg;
  float sop, cop;
  if (p == 0) {
    sop = sin_to * hs.cos2k[1] - cos_to * hs.sin2k[1];
    cop = cos_to * hs.cos2k[1] + sin_to * hs.sin2k[1];
  } else if (p == 1) {
    sop = sin_to * hs.cos2k[0] + cos_to * hs.sin2k[0];
    cop = cos_to * hs.cos2k[0] - sin_to * hs.sin2k[0];
  } else if (p == 2) {
    sop = sin_to * hs.cos2k[2] + cos_to * hs.sin2k[2];
    cop = cos_to * hs.cos2k[2] - sin_to * hs.sin2k[2];
  } else {
    sop = sin_to;
    cop = cos_to;
  }
  float eps2 = fmaxf(r[1], 1e-5f);
  float vp = hs.v[p];
  float cos_theta = 1.f + vp * ologf(eps2 + (1.f - eps2) * oexpf(-2.f / vp));
  float sin_theta = safe_sqrt(1.f - sqr(cos_theta));
  float cos_phi = ocosf(2.f * kPi * r[2]);
  float sin_ti = -cos_theta * sop + sin_theta * cos_phi * cop;
  float cos_ti = safe_sqrt(1.f - sqr(sin_ti));
  float etap = sqrtf(kEta * kEta - sqr(sin_to)) / cos_to;
  float sin_gt = h / etap;
  float gamma_t = safe_asin(sin_gt);
  float dphi;
  if (p < 3)
    dphi = phi_p(p, gamma_o, gamma_t) + sample_trimmed_logistic(r[3], hs.s, -kPi, kPi);
  else
    dphi = 2.f * kPi * r[3];
  float phi_i = phi_o + dphi;
  V3 wil = normalize(V3(sin_ti, cos_ti * ocosf(phi_i), cos_ti * osinf(phi_i)));
  *wi_local = wil;
  return disney_hair(wo, wil, h, hs, pdf);
}

// Hair shading frame of hairCH (optix_common.cuh:571-583): X = t,
// Y = normalize(wo x X), Z = normalize(X x Y).
struct HairFrame {
  V3 to_local[3], to_world[3];
  V3 wo_local;
};
inline HairFrame hair_frame(V3 wo, V3 t) {
  HairFrame fr;
  V3 X = t;
  V3 Y = normalize(cross(wo, X));
  V3 Z = normalize(cross(X, Y));
  fr.to_local[0] = X;
  fr.to_local[1] = Y;
  fr.to_local[2] = Z;
  fr.to_world[0] = V3(X.x, Y.x, Z.x);
  fr.to_world[1] = V3(X.y, Y.y, Z.y);
  fr.to_world[2] = V3(X.z, Y.z, Z.z);
  fr.wo_local = normalize(apply_mat(fr.to_local, wo));
  return fr;
}

// ------------------------------------------------------------ GGX (frostbite_anisotropic.cuh)
inline float ggx_d(float ax, float ay, V3 N) {  // :24-32
  float t1 = N.x / ax, t2 = N.y / ay, t3 = N.z;
  float value = kPi * ax * ay * opowf(t1 * t1 + t2 * t2 + t3 * t3, 2.0f);
  return 1.0f / value;
}
inline float ggx_lambda(float ax, float ay, V3 V) {  // :34-42
  float t1 = V.x * ax, t2 = V.y * ay, t3 = V.z;
  float t4 = sqrtf(1.0f + (t1 * t1 + t2 * t2) / (t3 * t3));
  return 0.5f * (-1.0f + t4);
}
inline float ggx_g1(float ax, float ay, V3 V) {  // :44-51
  if (V.z <= 0.0f) return 0.0f;
  return 1.0f / (1.0f + ggx_lambda(ax, ay, V));
}
inline float ggx_g2(float ax, float ay, V3 V, V3 L) {  // :53-60
  if (V.z <= 0.0f || L.z <= 0.0f) return 0.0f;
  return 1.0f / (1.0f + ggx_lambda(ax, ay, V) + ggx_lambda(ax, ay, L));
}
inline float ggx_dv(float ax, float ay, V3 V, V3 Ne) {  // :62-70
  float g1 = ggx_g1(ax, ay, V);
  float m = fmaxf(0.f, dot(V, Ne));
  float d = ggx_d(ax, ay, Ne);
  return g1 * m * d / V.z;
}
inline float ggx(float ax, float ay, V3 V, V3 L) {  // :72-78
  V3 H = normalize(V + L);
  return ggx_d(ax, ay, H) * ggx_g2(ax, ay, V, L) / 4.0f / V.z / L.z;
}
inline V3 frostbite_ggx(V3 wo, V3 wi, V3 color, float alpha) {  // :84-100
  V3 brdf(0.f);
  if (wo.z > 0.f && wi.z > 0.f) {
    brdf = brdf + 0.5f * color / kPi;
    brdf = brdf + V3(0.5f * ggx(alpha, alpha, wo, wi));
  }
  return brdf * fabsf(wi.z);
}
inline V3 sample_vndf(float ax, float ay, V3 V, float U1, float U2) {  // :102-131
  V3 Vh = normalize(V * V3(ax, ay, 1.0f));
  float lensq = Vh.x * Vh.x + Vh.y * Vh.y;
  V3 T1 = lensq > 0.0f ? V3(-Vh.y, Vh.x, 0.0f) / sqrtf(lensq) : V3(1.0f, 0.0f, 0.0f);
  V3 T2 = cross(Vh, T1);
  float r = sqrtf(U1);
  float phi = 2.0f * kPi * U2;
  float t1 = r * ocosf(phi);
  float t2 = r * osinf(phi);
  float s = 0.5f * (1.0f + Vh.z);
  t2 = (1.0f - s) * sqrtf(1.0f - t1 * t1) + s * t2;
  V3 Nh = t1 * T1 + t2 * T2 + sqrtf(fmaxf(0.0f, 1.0f - t1 * t1 - t2 * t2)) * Vh;
  V3 Ne(ax * Nh.x, ay * Nh.y, fmaxf(0.0f, Nh.z));
  return normalize(Ne);
}
inline float pdf_ggx(float alpha, V3 V, V3 Ne) {  // :133-141
  return ggx_dv(alpha, alpha, V, Ne) / (4.f * dot(V, Ne));
}
inline V3 sample_ggx(float u0, float u1, float alpha, V3 V, float* pdf) {  // :143-157
  V3 N = sample_vndf(alpha, alpha, V, u0, u1);
  V3 L = -V + 2.0f * N * dot(V, N);
  *pdf = pdf_ggx(alpha, V, N);
  return normalize(L);
}

// ------------------------------------------------------------ curves (curve_utils.cuh)
struct Cubic {  // CubicInterpolator :57-129, P(u) = p0 u^3 + p1 u^2 + p2 u + p3
  V4 p[4];
  static Cubic from_catrom(const V4* q) {  // :62-73
    Cubic c;
    c.p[0] = (-1.0f * q[0] + (3.0f) * q[1] + (-3.0f) * q[2] + (1.0f) * q[3]) / 2.0f;
    c.p[1] = (2.0f * q[0] + (-5.0f) * q[1] + (4.0f) * q[2] + (-1.0f) * q[3]) / 2.0f;
    c.p[2] = (-1.0f * q[0] + (1.0f) * q[2]) / 2.0f;
    c.p[3] = ((2.0f) * q[1]) / 2.0f;
    return c;
  }
  // Uniform cubic B-spline in the same power basis (the standard basis
  // matrix / 6); the form the hair geometry is intersected and shaded with.
  static Cubic from_bspline(const V4* q) {
    Cubic c;
    c.p[0] = (-1.0f * q[0] + 3.0f * q[1] + (-3.0f) * q[2] + 1.0f * q[3]) / 6.0f;
    c.p[1] = (3.0f * q[0] + (-6.0f) * q[1] + 3.0f * q[2]) / 6.0f;
    c.p[2] = (-3.0f * q[0] + 3.0f * q[2]) / 6.0f;
    c.p[3] = (1.0f * q[0] + 4.0f * q[1] + 1.0f * q[2]) / 6.0f;
    return c;
  }
  V4 position4(float u) const { return (((p[0] * u) + p[1]) * u + p[2]) * u + p[3]; }  // :75-79
  V4 velocity4(float u) const {                                                         // :93-102
    if (u == 0.f) u = 0.000001f;
    if (u == 1.f) u = 0.999999f;
    return ((3.0f * p[0] * u) + 2.0f * p[1]) * u + p[2];
  }
  V4 acceleration4(float u) const { return 6.0f * p[0] * u + 2.0f * p[1]; }  // :116-120
};
inline V3 curve_tangent(const Cubic& c, float u) { return normalize(c.velocity4(u).xyz()); }  // :208-214
inline V3 surface_normal(const Cubic& bc, float u, V3* ps) {                                   // :159-197
  V3 normal;
  if (u == 0.0f) {
    normal = -bc.velocity4(0.f).xyz();
  } else if (u == 1.0f) {
    normal = bc.velocity4(1.f).xyz();
  } else {
    V4 p4 = bc.position4(u);
    V3 p = p4.xyz();
    float r = p4.w;
    V4 d4 = bc.velocity4(u);
    V3 d = d4.xyz();
    float dr = d4.w;
    float dd = dot(d, d);
    V3 o1 = *ps - p;
    o1 = o1 - (dot(o1, d) / dd) * d;
    o1 = o1 * (r / length(o1));
    *ps = p + o1;
    dd -= dot(bc.acceleration4(u).xyz(), o1);
    normal = dd * o1 - (dr * r) * d;
  }
  return normalize(normal);
}

}  // namespace hmo
