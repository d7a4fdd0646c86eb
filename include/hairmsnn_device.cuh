/* Device-side drop-in for the reference's hair BSDF API.
 *
 * The reference's OptiX programs call, per hit,
 *   void  setupHairShading(Interaction& si)                       disney_hair.cuh:26
 *   vec3f disney_hair(Interaction si, float* pdf)                 disney_hair.cuh:186
 *   vec3f sample_disney_hair(Interaction& si, vec4f& rand, float* pdf)  disney_hair.cuh:277
 * over a ~300-byte Interaction passed by value.  This header keeps those
 * names and argument meanings for CUDA code of one's own (a closest-hit
 * routine of another renderer, a test kernel) over a lean HairVertex: the
 * directions, the hair frame of hairCH (optix_common.cuh:571-583), the
 * surface normal and the material's precomputed terms.  The functions are
 * the library's own (hairmsnn_gb300/csrc/hm_hair_bsdf.cuh): the same code as
 * the batched hm_bsdf_eval / hm_bsdf_sample.
 *
 * Compile with  -I <repo>/include -I <repo>/hairmsnn_gb300/csrc  for sm_103a.
 * The library's batched kernels are built with -fmad=false (every operation
 * rounded like the reference's); build with the same flag to get their
 * results bit for bit.
 *
 * Like the reference, no function here has an error path: a NaN result is
 * the caller's to handle.
 */
#ifndef HAIRMSNN_DEVICE_CUH_
#define HAIRMSNN_DEVICE_CUH_

#include "hairmsnn.h"
#include "hm_hair_bsdf.cuh"

/* A hair hit, as much of the reference's Interaction as the BSDF reads. */
struct HairVertex {
  float3 wo, wi;             /* world directions, both pointing away from the hit */
  float3 wo_local, wi_local; /* in the hair frame (x along the fibre) */
  float3 to_local[3];        /* frame rows X = t, Y = normalize(wo x t), Z = X x Y */
  float3 n;                  /* surface normal at the hit: h = dot(Y, n) */
  hm::HairConsts hair;       /* the material's terms (setupHairShading) */
};

namespace hairmsnn_device_detail {
__device__ __forceinline__ hm::f3 f3_of(float3 v) { return hm::mk(v.x, v.y, v.z); }
__device__ __forceinline__ float3 float3_of(hm::f3 v) { return make_float3(v.x, v.y, v.z); }
__device__ __forceinline__ hm::Frame frame_of(const HairVertex& v) {
  return hm::Frame{f3_of(v.to_local[0]), f3_of(v.to_local[1]), f3_of(v.to_local[2])};
}
}  // namespace hairmsnn_device_detail

/* setupHairShading (disney_hair.cuh:26-41): the material's terms, here from
 * hm_hair_params (alpha in radians).  Material-only: compute it once per
 * material (on the host or the device) and copy it into each vertex. */
__host__ __device__ __forceinline__ void setupHairShading(HairVertex& v, const hm_hair_params& material) {
  v.hair = hm::hair_consts(material);
}

/* The hair frame of hairCH (optix_common.cuh:571-583) for outgoing direction
 * wo, fibre tangent t and surface normal n; sets wo_local. */
__device__ __forceinline__ void hairVertexFrame(HairVertex& v, float3 wo, float3 t, float3 n) {
  using namespace hairmsnn_device_detail;
  const hm::Frame fr = hm::hair_frame(f3_of(wo), f3_of(t));
  v.wo = wo;
  v.n = n;
  v.to_local[0] = float3_of(fr.r0);
  v.to_local[1] = float3_of(fr.r1);
  v.to_local[2] = float3_of(fr.r2);
  v.wo_local = float3_of(hm::normalize(hm::to_local(fr, f3_of(wo))));
}

/* disney_hair (disney_hair.cuh:186-266): f * cos for v.wo_local, v.wi_local
 * summed over the R, TT, TRT and TRRT lobes; *pdf = the four-lobe mixture
 * pdf of wi. */
__device__ __forceinline__ float3 disney_hair(const HairVertex& v, float* pdf) {
  using namespace hairmsnn_device_detail;
  const float h = hm::dot(f3_of(v.to_local[1]), f3_of(v.n));
  const hm::HairEval e = hm::hair_eval(f3_of(v.wo_local), f3_of(v.wi_local), h, v.hair);
  *pdf = e.pdf;
  return float3_of(e.f);
}

/* sample_disney_hair (disney_hair.cuh:277-386): picks a lobe with rand.x,
 * samples theta with rand.y, rand.z and phi with rand.w; writes v.wi_local
 * and v.wi and returns disney_hair at the sampled direction (*pdf its full
 * mixture pdf). */
__device__ __forceinline__ float3 sample_disney_hair(HairVertex& v, const float4& rand, float* pdf) {
  using namespace hairmsnn_device_detail;
  const hm::Frame fr = frame_of(v);
  const float h = hm::dot(fr.r1, f3_of(v.n));
  hm::f3 wil;
  const hm::HairEval e = hm::hair_sample(f3_of(v.wo_local), h, rand.x, rand.y, rand.z, rand.w, v.hair, &wil);
  v.wi_local = float3_of(wil);
  v.wi = float3_of(hm::normalize(hm::to_world(fr, wil)));
  *pdf = e.pdf;
  return float3_of(e.f);
}

#endif /* HAIRMSNN_DEVICE_CUH_ */
