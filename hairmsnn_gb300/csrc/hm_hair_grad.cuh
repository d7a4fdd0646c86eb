// Derivatives of the hair BSDF (f * cos and the lobe-mixture pdf) with
// respect to the material: sigma_a (3), beta_m, beta_n, alpha (radians).
//
// Forward-mode differentiation with a 6-component dual number: every
// quantity carries its value and its partials, and each operation applies
// the chain rule.  The formulas and statement order are those of hair_eval
// (disney_hair.cuh:186-266) and setupHairShading (:26-41), with the
// material-only terms (v[k], s, sin/cos 2^k alpha, the trimmed-logistic
// normaliser) differentiated too, since they depend on the parameters.
// The branches (log-space M_p for v <= 0.1, LogI0 for x > 12, the wrap of
// delta phi, |cos theta'|) follow the value, as in the primal.  The M_p
// branch runs in FP32 here for every beta_m (the primal's FP64 branch for
// beta_m < 0.1 only changes rounding).
#pragma once
#include "hm_hair_bsdf.cuh"

namespace hm {

constexpr int kNd = 6;  // sigma_a r, g, b, beta_m, beta_n, alpha

struct Dual {
  float v;
  float d[kNd];
};

HM_D Dual dc(float x) {
  Dual r;
  r.v = x;
#pragma unroll
  for (int i = 0; i < kNd; ++i) r.d[i] = 0.f;
  return r;
}
HM_D Dual dvar(float x, int k) {
  Dual r = dc(x);
  r.d[k] = 1.f;
  return r;
}
// r = a * value, partials scaled by g (the derivative of a unary function)
HM_D Dual dmap(const Dual& a, float value, float g) {
  Dual r;
  r.v = value;
#pragma unroll
  for (int i = 0; i < kNd; ++i) r.d[i] = g * a.d[i];
  return r;
}
HM_D Dual operator+(const Dual& a, const Dual& b) {
  Dual r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < kNd; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
HM_D Dual operator-(const Dual& a, const Dual& b) {
  Dual r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < kNd; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
HM_D Dual operator-(const Dual& a) { return dmap(a, -a.v, -1.f); }
HM_D Dual operator*(const Dual& a, const Dual& b) {
  Dual r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < kNd; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
HM_D Dual operator/(const Dual& a, const Dual& b) {
  Dual r;
  r.v = a.v / b.v;
  const float ib = 1.f / b.v;
#pragma unroll
  for (int i = 0; i < kNd; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
HM_D Dual operator+(const Dual& a, float b) { Dual r = a; r.v += b; return r; }
HM_D Dual operator+(float a, const Dual& b) { return b + a; }
HM_D Dual operator-(const Dual& a, float b) { Dual r = a; r.v -= b; return r; }
HM_D Dual operator-(float a, const Dual& b) { return dmap(b, a - b.v, -1.f); }
HM_D Dual operator*(const Dual& a, float b) { return dmap(a, a.v * b, b); }
HM_D Dual operator*(float a, const Dual& b) { return dmap(b, a * b.v, a); }
HM_D Dual operator/(const Dual& a, float b) { return dmap(a, a.v / b, 1.f / b); }
HM_D Dual operator/(float a, const Dual& b) { return dmap(b, a / b.v, -a / (b.v * b.v)); }

HM_D Dual dsqr(const Dual& a) { return a * a; }
HM_D Dual dexp(const Dual& a) { const float e = expf(a.v); return dmap(a, e, e); }
HM_D Dual dlog(const Dual& a) { return dmap(a, logf(a.v), 1.f / a.v); }
HM_D Dual dsqrt_safe(const Dual& a) {
  if (a.v <= 0.f) return dc(0.f);
  const float s = sqrtf(a.v);
  return dmap(a, s, 0.5f / s);
}
HM_D Dual dsin(const Dual& a) { return dmap(a, sinf(a.v), cosf(a.v)); }
HM_D Dual dsinh(const Dual& a) { return dmap(a, sinhf(a.v), coshf(a.v)); }
HM_D Dual dabs(const Dual& a) { return a.v < 0.f ? -a : a; }
HM_D Dual dpow_int(const Dual& a, int n) {  // a^n, n >= 1
  const float p = powf(a.v, (float)n);
  return dmap(a, p, (float)n * powf(a.v, (float)(n - 1)));
}

struct HairConstsD {
  Dual v[4];  // v[3] == s, as in the reference's struct (sample_disney_hair quirk)
  Dual s;
  Dual sin2k[3], cos2k[3];
  Dual sigma_a[3];
  float gain[4];
  Dual trim_den;
};

// setupHairShading (disney_hair.cuh:26-41) with the parameters as variables.
HM_D HairConstsD hair_consts_dual(const float sigma_a[3], float beta_m, float beta_n, float alpha,
                                  const float gain[4]) {
  HairConstsD hc;
  const Dual bm = dvar(beta_m, 3), bn = dvar(beta_n, 4), al = dvar(alpha, 5);
  hc.v[0] = dsqr(0.726f * bm + 0.812f * dsqr(bm) + 3.7f * dpow_int(bm, 20));
  hc.v[1] = 0.25f * hc.v[0];
  hc.v[2] = 4.f * hc.v[0];
  hc.s = kSqrtPiOver8 * (0.265f * bn + 1.194f * dsqr(bn) + 5.372f * dpow_int(bn, 22));
  hc.v[3] = hc.s;
  hc.sin2k[0] = dsin(al);
  hc.cos2k[0] = dsqrt_safe(1.f - dsqr(hc.sin2k[0]));
  for (int i = 1; i < 3; ++i) {
    hc.sin2k[i] = 2.f * hc.cos2k[i - 1] * hc.sin2k[i - 1];
    hc.cos2k[i] = dsqr(hc.cos2k[i - 1]) - dsqr(hc.sin2k[i - 1]);
  }
  for (int c = 0; c < 3; ++c) hc.sigma_a[c] = dvar(sigma_a[c], c);
  for (int k = 0; k < 4; ++k) hc.gain[k] = gain[k];
  auto cdf = [&](float x) { return 1.f / (1.f + dexp(-x / hc.s)); };  // LogisticCDF :123-125
  hc.trim_den = cdf(kPi) - cdf(-kPi);
  return hc;
}

HM_D Dual bessel_i0_dual(const Dual& x) {  // disney_hair.cuh:54-67
  Dual val = dc(0.f), x2i = dc(1.f);
  float ifact = 1.f, i4 = 1.f;
  const Dual xx = x * x;
  for (int i = 0; i < 10; ++i) {
    if (i > 1) ifact *= (float)i;
    val = val + x2i / (i4 * ifact * ifact);
    x2i = x2i * xx;
    i4 *= 4.f;
  }
  return val;
}

HM_D Dual log_i0_dual(const Dual& x) {  // disney_hair.cuh:70-75
  if (x.v > 12.f) return x + 0.5f * ((-logf(2.f * kPi)) + dlog(1.f / x) + 1.f / (8.f * x));
  return dlog(bessel_i0_dual(x));
}

// M_p (disney_hair.cuh:78-88); cop may carry partials (through alpha).
HM_D Dual mp_dual(float cti, const Dual& cto, float sti, const Dual& sto, const Dual& v) {
  const Dual a = (cti * cto) / v;
  const Dual b = (sti * sto) / v;
  if (v.v <= 0.1f) return dexp(log_i0_dual(a) - b - 1.f / v + 0.6931f + dlog(1.f / (2.f * v)));
  return (dexp(-b) * bessel_i0_dual(a)) / (dsinh(1.f / v) * 2.f * v);
}

HM_D Dual np_dual(float phi, int p, float gamma_o, float gamma_t, const HairConstsD& hc) {
  float dphi = phi - phi_p(p, gamma_o, gamma_t);
  while (dphi > kPi) dphi -= 2.f * kPi;
  while (dphi < -kPi) dphi += 2.f * kPi;
  const Dual e = dexp(-fabsf(dphi) / hc.s);
  return (e / (hc.s * dsqr(1.f + e))) / hc.trim_den;
}

struct HairEvalD {
  Dual f[3];
  Dual pdf;
};

// hair_eval with derivatives; wo, wi in the hair frame, h = dot(Y, n).
HM_D HairEvalD hair_eval_dual(f3 wo, f3 wi, float h, const HairConstsD& hc) {
  const float sin_to = wo.x;
  const float cos_to = safe_sqrt(1.f - sqr(sin_to));
  const float phi_o = atan2f(wo.z, wo.y);
  const float sin_ti = wi.x;
  const float cos_ti = safe_sqrt(1.f - sqr(sin_ti));
  const float phi_i = atan2f(wi.z, wi.y);
  const float sin_tt = sin_to / kEta;
  const float cos_tt = safe_sqrt(1.f - sqr(sin_tt));
  const float gamma_o = asinf(h);
  const float cos_go = cosf(gamma_o);
  const float etap = sqrtf(kEta * kEta - sqr(sin_to)) / cos_to;
  const float sin_gt = h / etap;
  const float cos_gt = safe_sqrt(1.f - sqr(sin_gt));
  const float gamma_t = safe_asin(sin_gt);
  const float fac = (2.f * cos_gt / cos_tt);
  Dual T[3];
  for (int c = 0; c < 3; ++c) T[c] = dexp(-hc.sigma_a[c] * fac);
  const float F0 = sqr(1.f - kEta) / sqr(1.f + kEta);
  const float xd = 1.f - cos_to * cos_go;
  const float fr = F0 + (1.f - F0) * xd * xd * xd * xd * xd;
  Dual a1[3], a2[3], a3[3];
  for (int c = 0; c < 3; ++c) {
    a1[c] = sqr(1.f - fr) * T[c];
    a2[c] = sqr(1.f - fr) * T[c] * T[c] * fr;
    a3[c] = a2[c] * fr * T[c] / (1.f - T[c] * fr);
  }
  const float phi = phi_i - phi_o;
  const Dual st = dc(sin_to), ct = dc(cos_to);

  Dual sop = st * hc.cos2k[1] - ct * hc.sin2k[1];
  Dual cop = dabs(ct * hc.cos2k[1] + st * hc.sin2k[1]);
  const Dual mp0 = mp_dual(cos_ti, cop, sin_ti, sop, hc.v[0]);
  const Dual np0 = np_dual(phi, 0, gamma_o, gamma_t, hc);

  sop = st * hc.cos2k[0] + ct * hc.sin2k[0];
  cop = dabs(ct * hc.cos2k[0] - st * hc.sin2k[0]);
  const Dual mp1 = mp_dual(cos_ti, cop, sin_ti, sop, hc.v[1]);
  const Dual np1 = np_dual(phi, 1, gamma_o, gamma_t, hc);

  sop = st * hc.cos2k[2] + ct * hc.sin2k[2];
  cop = dabs(ct * hc.cos2k[2] - st * hc.sin2k[2]);
  const Dual mp2 = mp_dual(cos_ti, cop, sin_ti, sop, hc.v[2]);
  const Dual np2 = np_dual(phi, 2, gamma_o, gamma_t, hc);

  const Dual mpm = mp_dual(cos_ti, ct, sin_ti, st, hc.v[2]);
  const float npm = 1.f / (2.f * kPi);

  HairEvalD out;
  for (int c = 0; c < 3; ++c) {
    Dual f = hc.gain[0] * mp0 * fr * np0;
    f = f + hc.gain[1] * mp1 * a1[c] * np1;
    f = f + hc.gain[2] * mp2 * a2[c] * np2;
    f = f + hc.gain[3] * mpm * a3[c] * npm;
    out.f[c] = f;
  }
  const Dual ap0 = dc((fr + fr + fr) / 3.f);
  const Dual ap1 = (a1[0] + a1[1] + a1[2]) / 3.f;
  const Dual ap2 = (a2[0] + a2[1] + a2[2]) / 3.f;
  const Dual ap3 = (a3[0] + a3[1] + a3[2]) / 3.f;
  const Dual sum = ap0 + ap1 + ap2 + ap3;
  Dual pdf = mp0 * (ap0 / sum) * np0;
  pdf = pdf + mp1 * (ap1 / sum) * np1;
  pdf = pdf + mp2 * (ap2 / sum) * np2;
  pdf = pdf + mpm * (ap3 / sum) * npm;
  out.pdf = pdf;
  return out;
}

}  // namespace hm
