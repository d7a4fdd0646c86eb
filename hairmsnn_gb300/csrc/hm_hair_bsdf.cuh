// Chiang 2016 / d'Eon hair BSDF ("disney_hair") for sm_103a.
//
// Same formulas, statement order and lobe layout as the reference's
// cuda_headers/disney_hair.cuh; what changes is where the work happens:
//  * everything that depends only on the material (setupHairShading
//    disney_hair.cuh:26-41, the trimmed-logistic normaliser, the per-lobe
//    1/v, log(1/2v), sinh(1/v)*2v and exp(-2/v) terms) is computed once on the
//    host into HairConsts (kernel-parameter / constant memory) instead of at
//    every closest hit;
//  * callers pass wo/wi already in the hair frame and h = dot(Y, n), not a
//    ~300-byte Interaction by value;
//  * for beta_m < 0.1 the log-space M_p branch (disney_hair.cuh:82-83) runs in
//    FP64, where the FP32 cancellation between LogI0(a) and 1/v loses digits.
#pragma once
#include "hm_common.cuh"

namespace hm {

struct HairConsts {
  float v[4];         // v[0..2] as setupHairShading; v[3] == s (see sample_disney_hair)
  float s;            // logistic scale
  float sin2k[3], cos2k[3];
  float sigma_a[3];
  float gain[4];      // R, TT, TRT, TRRT
  float trim_den;     // LogisticCDF(pi, s) - LogisticCDF(-pi, s)
  float cdf_lo;       // LogisticCDF(-pi, s)
  float inv_v[3];     // 1 / v[k]
  float mp_logc[3];   // log(1 / (2 v[k]))
  float mp_den[3];    // sinh(1 / v[k]) * 2 * v[k]
  float exp_m2v[4];   // exp(-2 / v[p]), p = 0..3
  int fp64_mp;        // beta_m < 0.1
};

HM_HD float logistic_cdf_s(float x, float s) { return 1.f / (1.f + expf(-x / s)); }  // LogisticCDF :123-125

// setupHairShading (disney_hair.cuh:26-41) and every other material-only
// term, in the reference's single-precision order.  The library evaluates it
// once per material on the host (hair_consts_from_params); code that
// includes include/hairmsnn_device.cuh may also call it on the device.
HM_HD HairConsts hair_consts(const hm_hair_params& p) {
  HairConsts hc;
  const float bm = p.beta_m, bn = p.beta_n;
  hc.v[0] = sqr(0.726f * bm + 0.812f * sqr(bm) + 3.7f * powf(bm, 20.f));
  hc.v[1] = (float)(.25 * (double)hc.v[0]);
  hc.v[2] = 4.f * hc.v[0];
  hc.s = kSqrtPiOver8 * (0.265f * bn + 1.194f * sqr(bn) + 5.372f * powf(bn, 22.f));
  hc.v[3] = hc.s;
  hc.sin2k[0] = sinf(p.alpha);
  hc.cos2k[0] = safe_sqrt(1.f - sqr(hc.sin2k[0]));
  for (int i = 1; i < 3; ++i) {
    hc.sin2k[i] = 2.f * hc.cos2k[i - 1] * hc.sin2k[i - 1];
    hc.cos2k[i] = sqr(hc.cos2k[i - 1]) - sqr(hc.sin2k[i - 1]);
  }
  for (int i = 0; i < 3; ++i) hc.sigma_a[i] = p.sigma_a[i];
  hc.gain[0] = p.gain_r;
  hc.gain[1] = p.gain_tt;
  hc.gain[2] = p.gain_trt;
  hc.gain[3] = p.gain_trrt;
  hc.trim_den = logistic_cdf_s(kPi, hc.s) - logistic_cdf_s(-kPi, hc.s);
  hc.cdf_lo = logistic_cdf_s(-kPi, hc.s);
  for (int k = 0; k < 3; ++k) {
    hc.inv_v[k] = 1.f / hc.v[k];
    hc.mp_logc[k] = logf(1.f / (2.f * hc.v[k]));
    hc.mp_den[k] = sinhf(1.f / hc.v[k]) * 2.f * hc.v[k];
  }
  for (int k = 0; k < 4; ++k) hc.exp_m2v[k] = expf(-2.f / hc.v[k]);
  hc.fp64_mp = bm < 0.1f ? 1 : 0;
  return hc;
}

// Host-side precompute of hair_consts (see hm_bsdf.cu).
HairConsts hair_consts_from_params(const hm_hair_params& p);

HM_D float bessel_i0(float x) {  // disney_hair.cuh:54-67
  float val = 0.f, x2i = 1.f;
  float ifact = 1.f;  // i! for i <= 9 is exact in float (int64 in the reference)
  float i4 = 1.f;
#pragma unroll
  for (int i = 0; i < 10; ++i) {
    if (i > 1) ifact *= (float)i;
    val += x2i / (i4 * sqr(ifact));
    x2i *= x * x;
    i4 *= 4.f;
  }
  return val;
}

HM_D float log_i0(float x) {  // disney_hair.cuh:70-75; the `0.5 *` product is FP64
  if (x > 12.f)
    return (float)((double)x + 0.5 * (double)(-logf(2.f * kPi) + logf(1.f / x) + 1.f / (8.f * x)));
  return logf(bessel_i0(x));
}

HM_D double bessel_i0_d(double x) {
  double val = 0.0, x2i = 1.0, ifact = 1.0, i4 = 1.0;
#pragma unroll
  for (int i = 0; i < 10; ++i) {
    if (i > 1) ifact *= i;
    val += x2i / (i4 * ifact * ifact);
    x2i *= x * x;
    i4 *= 4.0;
  }
  return val;
}

// M_p (disney_hair.cuh:78-88) for lobe constants k; v = v[k].
HM_D float mp_lobe(float cti, float cto, float sti, float sto, const HairConsts& hc, int k) {
  const float v = hc.v[k];
  if (hc.fp64_mp && v <= 0.1f) {
    double dv = v;
    double a = (double)cti * (double)cto / dv;
    double b = (double)sti * (double)sto / dv;
    double li = a > 12.0 ? a + 0.5 * (-log(2.0 * (double)kPi) + log(1.0 / a) + 1.0 / (8.0 * a))
                         : log(bessel_i0_d(a));
    return (float)exp(li - b - 1.0 / dv + 0.6931 + log(1.0 / (2.0 * dv)));
  }
  float a = cti * cto / v;
  float b = sti * sto / v;
  if (v <= 0.1f) return expf(log_i0(a) - b - hc.inv_v[k] + 0.6931f + hc.mp_logc[k]);
  return (expf(-b) * bessel_i0(a)) / hc.mp_den[k];
}

HM_D float phi_p(int p, float gamma_o, float gamma_t) {  // disney_hair.cuh:112-114
  return (float)(2 * p) * gamma_t - 2.f * gamma_o + (float)p * kPi;
}

// TrimmedLogistic(dphi, s, -pi, pi) after wrapping dphi to [-pi, pi] (:117-139)
HM_D float np_lobe(float phi, int p, float gamma_o, float gamma_t, const HairConsts& hc) {
  float dphi = phi - phi_p(p, gamma_o, gamma_t);
  while (dphi > kPi) dphi -= 2.f * kPi;
  while (dphi < -kPi) dphi += 2.f * kPi;
  const float s = hc.s;
  float e = expf(-fabsf(dphi) / s);
  return (e / (s * sqr(1.f + e))) / hc.trim_den;
}

struct HairEval {
  f3 f;       // f * cos (the reference's disney_hair return value)
  float pdf;  // full 4-lobe mixture pdf
};

// disney_hair(si, &pdf), disney_hair.cuh:186-266.  wo, wi: hair-frame unit
// vectors (x along the fibre); h = dot(Y, n) in [-1, 1].
HM_D HairEval hair_eval(f3 wo, f3 wi, float h, const HairConsts& hc) {
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
  const f3 T = mk(expf(-hc.sigma_a[0] * fac), expf(-hc.sigma_a[1] * fac), expf(-hc.sigma_a[2] * fac));
  // Fresnel(Eta, cos_to * cos_go), disney_hair.cuh:46-51
  const float F0 = sqr(1.f - kEta) / sqr(1.f + kEta);
  const float xd = 1.f - cos_to * cos_go;
  const float fr = F0 + (1.f - F0) * xd * xd * xd * xd * xd;
  // A_p, :91-109
  const f3 a0 = splat(fr);
  const f3 a1 = sqr(1.f - fr) * T;
  const f3 a2 = sqr(1.f - fr) * T * T * fr;
  const f3 a3 = a2 * fr * T / (splat(1.f) - T * fr);
  const float phi = phi_i - phi_o;

  float sop = sin_to * hc.cos2k[1] - cos_to * hc.sin2k[1];
  float cop = fabsf(cos_to * hc.cos2k[1] + sin_to * hc.sin2k[1]);
  const float mp0 = mp_lobe(cos_ti, cop, sin_ti, sop, hc, 0);
  const float np0 = np_lobe(phi, 0, gamma_o, gamma_t, hc);
  f3 f = hc.gain[0] * mp0 * a0 * np0;

  sop = sin_to * hc.cos2k[0] + cos_to * hc.sin2k[0];
  cop = fabsf(cos_to * hc.cos2k[0] - sin_to * hc.sin2k[0]);
  const float mp1 = mp_lobe(cos_ti, cop, sin_ti, sop, hc, 1);
  const float np1 = np_lobe(phi, 1, gamma_o, gamma_t, hc);
  f = f + hc.gain[1] * mp1 * a1 * np1;

  sop = sin_to * hc.cos2k[2] + cos_to * hc.sin2k[2];
  cop = fabsf(cos_to * hc.cos2k[2] - sin_to * hc.sin2k[2]);
  const float mp2 = mp_lobe(cos_ti, cop, sin_ti, sop, hc, 2);
  const float np2 = np_lobe(phi, 2, gamma_o, gamma_t, hc);
  f = f + hc.gain[2] * mp2 * a2 * np2;

  const float mpm = mp_lobe(cos_ti, cos_to, sin_ti, sin_to, hc, 2);
  const float npm = 1.f / (2.f * kPi);
  f = f + hc.gain[3] * mpm * a3 * npm;

  // computeApPdf (:143-182): with eta = Eta it reuses the T and Fresnel above.
  float ap[4] = {(a0.x + a0.y + a0.z) / 3.f, (a1.x + a1.y + a1.z) / 3.f,
                 (a2.x + a2.y + a2.z) / 3.f, (a3.x + a3.y + a3.z) / 3.f};
  const float sum = ap[0] + ap[1] + ap[2] + ap[3];
  float pdf = 0.f;
  pdf = pdf + mp0 * (ap[0] / sum) * np0;
  pdf = pdf + mp1 * (ap[1] / sum) * np1;
  pdf = pdf + mp2 * (ap[2] / sum) * np2;
  pdf = pdf + mpm * (ap[3] / sum) * npm;
  return HairEval{f, pdf};
}

// Lobe-selection pmf (computeApPdf, disney_hair.cuh:143-182).
HM_D void hair_ap_pdf(float sin_to, float cos_to, float cos_go, float h, const HairConsts& hc,
                      float out[4]) {
  const float sin_tt = sin_to / kEta;
  const float cos_tt = safe_sqrt(1.f - sqr(sin_tt));
  const float etap = sqrtf(kEta * kEta - sqr(sin_to)) / cos_to;
  const float sin_gt = h / etap;
  const float cos_gt = safe_sqrt(1.f - sqr(sin_gt));
  const float fac = (2.f * cos_gt / cos_tt);
  const f3 T = mk(expf(-hc.sigma_a[0] * fac), expf(-hc.sigma_a[1] * fac), expf(-hc.sigma_a[2] * fac));
  const float F0 = sqr(1.f - kEta) / sqr(1.f + kEta);
  const float xd = 1.f - cos_to * cos_go;
  const float fr = F0 + (1.f - F0) * xd * xd * xd * xd * xd;
  const f3 a1 = sqr(1.f - fr) * T;
  const f3 a2 = sqr(1.f - fr) * T * T * fr;
  const f3 a3 = a2 * fr * T / (splat(1.f) - T * fr);
  out[0] = (fr + fr + fr) / 3.f;
  out[1] = (a1.x + a1.y + a1.z) / 3.f;
  out[2] = (a2.x + a2.y + a2.z) / 3.f;
  out[3] = (a3.x + a3.y + a3.z) / 3.f;
  const float sum = out[0] + out[1] + out[2] + out[3];
#pragma unroll
  for (int p = 0; p < 4; ++p) out[p] = out[p] / sum;
}

// sample_disney_hair(si, rand, &pdf), disney_hair.cuh:277-386.  Returns the
// hair-frame wi and the full eval at it.  The TRRT lobe (p = 3) uses
// v[3] == s: in the reference's HairInteraction the element after v[2] is s.
HM_D HairEval hair_sample(f3 wo, float h, float u0, float u1, float u2, float u3,
                          const HairConsts& hc, f3* wi_out) {
  const float sin_to = wo.x;
  const float cos_to = safe_sqrt(1.f - sqr(sin_to));
  const float phi_o = atan2f(wo.z, wo.y);
  const float gamma_o = asinf(h);
  const float cos_go = cosf(gamma_o);
  float ap[4];
  hair_ap_pdf(sin_to, cos_to, cos_go, h, hc, ap);
  int p = 0;
  float eps1 = u0;
  for (p = 0; p < 3; ++p) {
    if (eps1 < ap[p]) break;
    eps1 -= ap[p];
  }
  float sop, cop;
  if (p == 0) {
    sop = sin_to * hc.cos2k[1] - cos_to * hc.sin2k[1];
    cop = cos_to * hc.cos2k[1] + sin_to * hc.sin2k[1];
  } else if (p == 1) {
    sop = sin_to * hc.cos2k[0] + cos_to * hc.sin2k[0];
    cop = cos_to * hc.cos2k[0] - sin_to * hc.sin2k[0];
  } else if (p == 2) {
    sop = sin_to * hc.cos2k[2] + cos_to * hc.sin2k[2];
    cop = cos_to * hc.cos2k[2] - sin_to * hc.sin2k[2];
  } else {
    sop = sin_to;
    cop = cos_to;
  }
  const float eps2 = fmaxf(u1, 1e-5f);
  const float vp = hc.v[p];
  const float cos_theta = 1.f + vp * logf(eps2 + (1.f - eps2) * hc.exp_m2v[p]);
  const float sin_theta = safe_sqrt(1.f - sqr(cos_theta));
  const float cos_phi = cosf(2.f * kPi * u2);
  const float sin_ti = -cos_theta * sop + sin_theta * cos_phi * cop;
  const float cos_ti = safe_sqrt(1.f - sqr(sin_ti));
  const float etap = sqrtf(kEta * kEta - sqr(sin_to)) / cos_to;
  const float gamma_t = safe_asin(h / etap);
  float dphi;
  if (p < 3) {
    // SampleTrimmedLogistic(u3, s, -pi, pi), :269-274
    float x = -hc.s * logf(1.f / (u3 * hc.trim_den + hc.cdf_lo) - 1.f);
    dphi = phi_p(p, gamma_o, gamma_t) + fminf(fmaxf(x, -kPi), kPi);
  } else {
    dphi = 2.f * kPi * u3;
  }
  const float phi_i = phi_o + dphi;
  const f3 wi = normalize(mk(sin_ti, cos_ti * cosf(phi_i), cos_ti * sinf(phi_i)));
  *wi_out = wi;
  return hair_eval(wo, wi, h, hc);
}

// Hair shading frame of the reference's closest-hit program
// (optix_common.cuh:571-583): X = tangent, Y = normalize(wo x X), Z = X x Y.
HM_D Frame hair_frame(f3 wo, f3 t) {
  Frame fr;
  fr.r0 = t;
  fr.r1 = normalize(cross(wo, t));
  fr.r2 = normalize(cross(t, fr.r1));
  return fr;
}

}  // namespace hm
