// Shared device/host helpers for the HairMSNN GB300 library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/hairmsnn.h"

#define HM_HD __host__ __device__ __forceinline__
#define HM_D __device__ __forceinline__

namespace hm {

// utils.cuh:10-11 of the reference: two distinct pi literals.
constexpr float kPi = 3.1415926f;
constexpr float kTwoPiRef = 2.f * 3.14159f;
// disney_hair.cuh:10-11
constexpr float kEta = 1.55f;
constexpr float kSqrtPiOver8 = 0.626657069f;

struct f3 {
  float x, y, z;
};
HM_HD f3 mk(float x, float y, float z) { return f3{x, y, z}; }
HM_HD f3 splat(float s) { return f3{s, s, s}; }
HM_HD f3 operator+(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
HM_HD f3 operator-(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
HM_HD f3 operator*(f3 a, f3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
HM_HD f3 operator/(f3 a, f3 b) { return mk(a.x / b.x, a.y / b.y, a.z / b.z); }
HM_HD f3 operator*(float s, f3 a) { return mk(s * a.x, s * a.y, s * a.z); }
HM_HD f3 operator*(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
HM_HD f3 operator/(f3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
HM_HD f3 operator-(f3 a) { return mk(-a.x, -a.y, -a.z); }
HM_HD float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
HM_HD f3 cross(f3 a, f3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
HM_HD float length(f3 a) { return sqrtf(dot(a, a)); }
// v * (1/|v|) with an IEEE reciprocal and square root, the form used for
// every normalisation in the reference's vector library.
HM_HD f3 normalize(f3 a) { return a * (1.f / sqrtf(dot(a, a))); }
HM_HD float sqr(float v) { return v * v; }
HM_HD float safe_sqrt(float x) { return sqrtf(fmaxf(0.f, x)); }
HM_HD float safe_asin(float x) { return asinf(fminf(fmaxf(x, -1.f), 1.f)); }
HM_HD float luminance(f3 c) { return 0.212671f * c.x + 0.715160f * c.y + 0.072169f * c.z; }

// 3x3 frame stored as rows (to_local); to_world is its transpose.
struct Frame {
  f3 r0, r1, r2;
};
HM_HD f3 to_local(const Frame& m, f3 v) { return mk(dot(m.r0, v), dot(m.r1, v), dot(m.r2, v)); }
HM_HD f3 to_world(const Frame& m, f3 v) {
  return mk(dot(mk(m.r0.x, m.r1.x, m.r2.x), v), dot(mk(m.r0.y, m.r1.y, m.r2.y), v),
            dot(mk(m.r0.z, m.r1.z, m.r2.z), v));
}

// ------------------------------------------------------------------ RNG
// random.cuh:15-65 of the reference (ospray's murmur-hash seeded LCG).
HM_HD uint32_t murmur_mix(uint32_t hash, uint32_t k) {
  k *= 0xcc9e2d51u;
  k = (k << 15) | (k >> 17);
  k *= 0x1b873593u;
  hash ^= k;
  hash = ((hash << 13) | (hash >> 19)) * 5u + 0xe6546b64u;
  return hash;
}
HM_HD uint32_t murmur_finalize(uint32_t h) {
  h ^= h >> 16;
  h *= 0x85ebca6bu;
  h ^= h >> 13;
  h *= 0xc2b2ae35u;
  h ^= h >> 16;
  return h;
}
HM_HD uint32_t rng_seed(int frame_id, uint32_t pixel_index) {
  return murmur_finalize(murmur_mix(murmur_mix(0u, pixel_index), (uint32_t)frame_id));
}
// u32 -> float in [0,1): exact conversion of the rounded (float)u times 2^-32.
HM_HD float lcg_next(uint32_t& s) {
  s = s * 1664525u + 1013904223u;
  return (float)s * 2.3283064365386963e-10f;  // 2^-32 exactly
}

}  // namespace hm

// Error plumbing for the C ABI (thread-local message, hm_last_error()).
void hm_set_error(const char* fmt, ...);
int hm_cuda_status(cudaError_t e, const char* what);
#define HM_CHECK_LAUNCH(what)                                   \
  do {                                                          \
    cudaError_t _e = cudaGetLastError();                        \
    if (_e != cudaSuccess) return hm_cuda_status(_e, what);     \
  } while (0)
