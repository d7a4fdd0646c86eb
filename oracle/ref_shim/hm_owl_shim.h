// Host-side stand-ins for the OWL / OptiX / CUDA names that the reference's
// header-only device code uses, so that those headers compile unmodified with
// g++ on the CPU.  Test infrastructure only: this file and everything it
// supports are the checker, never part of the shipped library.
//
// What is emulated and how:
//  * owl::vec2f/vec2i/vec3f/vec3i/vec4f with the arithmetic the reference uses
//    (component-wise ops, dot, cross, length, normalize, clamp/min/max).
//    OWL itself is an absent submodule; normalize is written as
//    v * (1/sqrt(dot(v,v))) in single precision.
//  * CUDA qualifiers (__device__, __forceinline__, ...) expand to nothing.
//  * OptiX program macros become plain extern "C" functions; the OptiX query
//    intrinsics (optixGetPrimitiveIndex, optixGetCurveParameter, ...) read a
//    thread-local "hit context" that the harness fills before it calls a
//    closest-hit / any-hit / miss program.
//  * owl::traceRay forwards to a harness callback (hm_shim_trace_hook).
//  * tex2D<T>(obj, x, y) reads a harness-registered host table with CUDA's
//    normalized-coordinate, clamp-address semantics (nearest or linear).
#pragma once

#include <cmath>
#include <math.h>
#include <cstdint>
#include <cstring>

#define __device__
#define __host__
#define __global__
#define __constant__
#define __forceinline__ inline
#define __inline__ inline
#define __both__

// ---------------------------------------------------------------- CUDA types
struct uint2 { unsigned x, y; };
inline uint2 make_uint2(unsigned x, unsigned y) { uint2 r; r.x = x; r.y = y; return r; }
struct float2 { float x, y; };
struct float3 { float x, y, z; };
struct float4 { float x, y, z, w; };
struct int2 { int x, y; };
typedef unsigned long long cudaTextureObject_t;
typedef unsigned long long OptixTraversableHandle;

namespace owl {

template <class T> inline T abs(T x) { return x < T(0) ? -x : x; }
template <class T> inline T max(T a, T b) { return a < b ? b : a; }
template <class T> inline T min(T a, T b) { return a < b ? a : b; }
template <class T> inline T clamp(T x, T lo, T hi) { return min(max(x, lo), hi); }
// Templates, so that an unqualified call under `using namespace owl` prefers
// the global float overloads from <math.h> instead of being ambiguous.
template <class T> inline T sqrt(T x) { return (T)::sqrtf((float)x); }
template <class T> inline T cos(T x) { return (T)::cosf((float)x); }
template <class T> inline T sin(T x) { return (T)::sinf((float)x); }
inline float rsqrt_ref(float x) { return 1.f / ::sqrtf(x); }

struct vec2i {
  union { int x; int u; };
  union { int y; int v; };
  vec2i() : x(0), y(0) {}
  vec2i(int s) : x(s), y(s) {}  // broadcast, as OWL's
  vec2i(int a, int b) : x(a), y(b) {}
};
struct vec3i {
  int x, y, z;
  vec3i() : x(0), y(0), z(0) {}
  vec3i(int a, int b, int c) : x(a), y(b), z(c) {}
};

struct vec2f {
  union { float x; float u; };
  union { float y; float v; };
  vec2f() : x(0.f), y(0.f) {}
  explicit vec2f(float s) : x(s), y(s) {}
  vec2f(float a, float b) : x(a), y(b) {}
  explicit vec2f(const vec2i& o) : x((float)o.x), y((float)o.y) {}
};
inline vec2f operator+(vec2f a, vec2f b) { return vec2f(a.x + b.x, a.y + b.y); }
inline vec2f operator-(vec2f a, vec2f b) { return vec2f(a.x - b.x, a.y - b.y); }
inline vec2f operator*(vec2f a, vec2f b) { return vec2f(a.x * b.x, a.y * b.y); }
inline vec2f operator/(vec2f a, vec2f b) { return vec2f(a.x / b.x, a.y / b.y); }
inline vec2f operator*(float s, vec2f a) { return vec2f(s * a.x, s * a.y); }
inline vec2f operator*(vec2f a, float s) { return vec2f(a.x * s, a.y * s); }

struct vec4f;
struct vec3f {
  float x, y, z;
  vec3f() : x(0.f), y(0.f), z(0.f) {}
  vec3f(float s) : x(s), y(s), z(s) {}  // implicit like OWL's broadcast
  vec3f(float a, float b, float c) : x(a), y(b), z(c) {}
  explicit vec3f(const vec4f& o);
  vec3f(const float3& o) : x(o.x), y(o.y), z(o.z) {}
  vec3f(const float4& o) : x(o.x), y(o.y), z(o.z) {}  // implicit, as OWL's
  float& operator[](int i) { return (&x)[i]; }
  const float& operator[](int i) const { return (&x)[i]; }
  operator float3() const { float3 r; r.x = x; r.y = y; r.z = z; return r; }  // as OWL's
};
struct vec4f {
  float x, y, z, w;
  vec4f() : x(0.f), y(0.f), z(0.f), w(0.f) {}
  vec4f(float s) : x(s), y(s), z(s), w(s) {}
  vec4f(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
  vec4f(const vec3f& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
  float& operator[](int i) { return (&x)[i]; }
  const float& operator[](int i) const { return (&x)[i]; }
  operator float4() const { float4 r; r.x = x; r.y = y; r.z = z; r.w = w; return r; }
};
inline vec3f::vec3f(const vec4f& o) : x(o.x), y(o.y), z(o.z) {}

inline vec3f operator+(vec3f a, vec3f b) { return vec3f(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3f operator-(vec3f a, vec3f b) { return vec3f(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3f operator*(vec3f a, vec3f b) { return vec3f(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3f operator/(vec3f a, vec3f b) { return vec3f(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3f operator*(float s, vec3f a) { return vec3f(s * a.x, s * a.y, s * a.z); }
inline vec3f operator*(vec3f a, float s) { return vec3f(a.x * s, a.y * s, a.z * s); }
inline vec3f operator/(vec3f a, float s) { return vec3f(a.x / s, a.y / s, a.z / s); }
inline vec3f operator-(vec3f a) { return vec3f(-a.x, -a.y, -a.z); }
inline vec3f& operator+=(vec3f& a, vec3f b) { a = a + b; return a; }
inline vec3f& operator-=(vec3f& a, vec3f b) { a = a - b; return a; }
inline vec3f& operator*=(vec3f& a, float s) { a = a * s; return a; }
inline bool operator==(vec3f a, vec3f b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline bool operator!=(vec3f a, vec3f b) { return !(a == b); }

inline vec4f operator+(vec4f a, vec4f b) { return vec4f(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4f operator-(vec4f a, vec4f b) { return vec4f(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline vec4f operator*(float s, vec4f a) { return vec4f(s * a.x, s * a.y, s * a.z, s * a.w); }
inline vec4f operator*(vec4f a, float s) { return vec4f(a.x * s, a.y * s, a.z * s, a.w * s); }
inline vec4f operator*(vec4f a, vec4f b) { return vec4f(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
inline vec4f operator/(vec4f a, float s) { return vec4f(a.x / s, a.y / s, a.z / s, a.w / s); }

inline float dot(vec3f a, vec3f b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3f cross(vec3f a, vec3f b) {
  return vec3f(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float length(vec3f a) { return ::sqrtf(dot(a, a)); }
inline vec3f normalize(vec3f a) { return a * rsqrt_ref(dot(a, a)); }
inline vec3f min(vec3f a, vec3f b) { return vec3f(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline vec3f max(vec3f a, vec3f b) { return vec3f(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }

inline uint32_t make_rgba(vec3f c) {
  auto q = [](float v) { int i = (int)(v * 255.9f); return (uint32_t)(i < 0 ? 0 : (i > 255 ? 255 : i)); };
  return q(c.x) | (q(c.y) << 8) | (q(c.z) << 16) | (0xffu << 24);
}

// axis-aligned box (OWL's box3f: lower / upper), for the reference's host
// headers (Model::bounds)
struct box3f {
  vec3f lower = vec3f(1e30f), upper = vec3f(-1e30f);
};

// ----------------------------------------------------------- ray + traceRay
template <int RAY_TYPE, int NUM_RAY_TYPES>
struct RayT {
  vec3f origin, direction;
  float tmin = 0.f, tmax = 1e30f;
};

}  // namespace owl

inline float linear_to_srgb(float x) {
  if (x <= 0.0031308f) return 12.92f * x;
  return 1.055f * ::powf(x, 1.f / 2.4f) - 0.055f;
}

// ----------------------------------------------------- harness hit context
struct HmShimHitContext {
  int primitive_index = 0;
  float curve_u = 0.f;
  float ray_tmax = 0.f;
  float3 ray_origin{0.f, 0.f, 0.f};
  float3 ray_dir{0.f, 0.f, 1.f};
  float2 barycentrics{0.f, 0.f};
  float4 cps[4];
  const void* program_data = nullptr;
  void* prd = nullptr;
  int launch_x = 0, launch_y = 0;
  int terminated = 0;
};
extern thread_local HmShimHitContext hm_shim_ctx;
// Implemented by the harness: trace one ray of the given type; it calls the
// reference's closest-hit / any-hit / miss programs with hm_shim_ctx set.
extern "C" void hm_shim_trace_hook(int ray_type, const float* org, const float* dir,
                                   float tmin, float tmax, void* prd);

namespace owl {
template <int T, int N> inline int ray_type_of(const RayT<T, N>*) { return T; }
template <class RayType, class PRD>
inline void traceRay(OptixTraversableHandle, const RayType& ray, PRD& prd) {
  float o[3] = {ray.origin.x, ray.origin.y, ray.origin.z};
  float d[3] = {ray.direction.x, ray.direction.y, ray.direction.z};
  hm_shim_trace_hook(ray_type_of((const RayType*)nullptr), o, d, ray.tmin, ray.tmax, (void*)&prd);
}
template <class T> inline T& getPRD() { return *(T*)hm_shim_ctx.prd; }
template <class T> inline const T& getProgramData() { return *(const T*)hm_shim_ctx.program_data; }
inline vec2i getLaunchIndex() { return vec2i(hm_shim_ctx.launch_x, hm_shim_ctx.launch_y); }
}  // namespace owl

inline unsigned optixGetPrimitiveIndex() { return (unsigned)hm_shim_ctx.primitive_index; }
inline float optixGetCurveParameter() { return hm_shim_ctx.curve_u; }
inline float optixGetRayTmax() { return hm_shim_ctx.ray_tmax; }
inline float3 optixGetWorldRayOrigin() { return hm_shim_ctx.ray_origin; }
inline float3 optixGetWorldRayDirection() { return hm_shim_ctx.ray_dir; }
inline float2 optixGetTriangleBarycentrics() { return hm_shim_ctx.barycentrics; }
inline OptixTraversableHandle optixGetGASTraversableHandle() { return 0; }
inline unsigned optixGetSbtGASIndex() { return 0; }
// The reference passes a vec4f array cast to float4* (curve_utils.cuh:230):
// written with memcpy, which may store into objects of any type (the build
// also uses -fno-strict-aliasing for the reference's casts).
inline void optixGetCatmullRomVertexData(OptixTraversableHandle, unsigned, unsigned, float, float4* out) {
  memcpy((void*)out, hm_shim_ctx.cps, 4 * sizeof(float4));
}
inline void optixGetLinearCurveVertexData(OptixTraversableHandle, unsigned, unsigned, float, float4* out) {
  memcpy((void*)out, hm_shim_ctx.cps, 2 * sizeof(float4));
}
inline void optixTerminateRay() { hm_shim_ctx.terminated = 1; }
inline void optixIgnoreIntersection() {}

#define OPTIX_RAYGEN_PROGRAM(name) extern "C" void __raygen__##name
#define OPTIX_CLOSEST_HIT_PROGRAM(name) extern "C" void __closesthit__##name
#define OPTIX_ANY_HIT_PROGRAM(name) extern "C" void __anyhit__##name
#define OPTIX_MISS_PROGRAM(name) extern "C" void __miss__##name

// ------------------------------------------------------------- texture emu
// A registered host table: width x height texels of `channels` floats,
// normalized coordinates, clamp addressing.  filter 0 = nearest, 1 = linear
// (exact fractional weights: the 1/256 fixed-point weight quantisation of the
// hardware texture unit is not modelled).
struct HmShimTexture {
  const float* data = nullptr;
  int width = 0, height = 0, channels = 1, filter = 0;
};
extern HmShimTexture hm_shim_textures[16];

inline void hm_shim_tex_fetch(const HmShimTexture& t, int x, int y, float* out) {
  x = x < 0 ? 0 : (x >= t.width ? t.width - 1 : x);
  y = y < 0 ? 0 : (y >= t.height ? t.height - 1 : y);
  const float* p = t.data + ((size_t)y * t.width + x) * t.channels;
  for (int c = 0; c < t.channels; ++c) out[c] = p[c];
}
inline void hm_shim_tex_sample(cudaTextureObject_t obj, float u, float v, float* out) {
  const HmShimTexture& t = hm_shim_textures[obj];
  float x = u * (float)t.width, y = v * (float)t.height;
  if (t.filter == 0) {
    hm_shim_tex_fetch(t, (int)floorf(x), (int)floorf(y), out);
    return;
  }
  float xb = x - 0.5f, yb = y - 0.5f;
  float fx = floorf(xb), fy = floorf(yb);
  float ax = xb - fx, ay = yb - fy;
  int ix = (int)fx, iy = (int)fy;
  float a[4], b[4], c[4], d[4];
  hm_shim_tex_fetch(t, ix, iy, a);
  hm_shim_tex_fetch(t, ix + 1, iy, b);
  hm_shim_tex_fetch(t, ix, iy + 1, c);
  hm_shim_tex_fetch(t, ix + 1, iy + 1, d);
  for (int k = 0; k < t.channels; ++k)
    out[k] = (1.f - ay) * ((1.f - ax) * a[k] + ax * b[k]) + ay * ((1.f - ax) * c[k] + ax * d[k]);
}
template <class T> T tex2D(cudaTextureObject_t obj, float u, float v);
template <> inline float tex2D<float>(cudaTextureObject_t obj, float u, float v) {
  float r[4];
  hm_shim_tex_sample(obj, u, v, r);
  return r[0];
}
template <> inline float4 tex2D<float4>(cudaTextureObject_t obj, float u, float v) {
  float r[4] = {0.f, 0.f, 0.f, 0.f};
  hm_shim_tex_sample(obj, u, v, r);
  float4 o;
  o.x = r[0]; o.y = r[1]; o.z = r[2]; o.w = r[3];
  return o;
}
