// HairMSNN hot-path ORACLE — test infrastructure only.
//
// A scalar CPU restatement of the reference's per-path-vertex algorithm, used
// by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg as
// the checker.  The shipped library (hairmsnn_gb300/) never includes, links
// or calls anything in oracle/.
//
// Pinning: the RNG, hair BSDF, GGX, curve and utility functions are checked
// bit-for-bit against the reference's own headers compiled on the host
// (oracle/build.py build_ref -> oracle/_ref, golden vectors in tests/golden/).
// The integrator is checked against the reference's own rayGenCam /
// msnnPathTrace / directLighting compiled the same way, with this oracle's
// BVH standing in for OptiX traversal (which is closed driver code).  The MLP
// restates tiny-cuda-nn's documented semantics (tiny-cuda-nn is an empty
// submodule in the reference checkout): parity against tiny-cuda-nn itself is
// unpinned.
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// Hair material block used throughout: sigma_a[3], beta_m, beta_n,
// alpha (radians), gain R, gain TT, gain TRT, gain TRRT  (10 floats).
enum { HMO_HAIR_PARAMS = 10 };

// ---- RNG (random.cuh:15-65)
uint32_t hmo_get_rng(int frame_id, uint32_t px, uint32_t py, uint32_t dimx, uint32_t dimy);
uint32_t hmo_lcg_stream(uint32_t state, int n, float* out);
// Synthetic-input stream: query index i, seed s -> state get_rng(s, (i,0),(2^31,1)).
uint32_t hmo_query_rng(uint32_t seed, uint32_t index);

// ---- hair BSDF (disney_hair.cuh:26-386), frame as in hairCH (optix_common.cuh:571-583)
void hmo_setup_hair(const float* hp, float* out10);
// 1: keep the M_p log branch in FP32 for every beta_m (bit-for-bit the
// reference); 0 (default): FP64 for that branch when beta_m < 0.1.
void hmo_set_mp_force_fp32(int on);
// 0 (default): libm's transcendental functions; +1 / -1: each result moved
// one ulp up / down; k >= 2: each result moved by a pseudo-random -2..+2 ulps
// (stream k, reseeded per pixel): the sensitivity of a path to last-ulp
// differences of its transcendental functions.
void hmo_set_ulp_perturb(int k);
// wo, wi, t: [n][3] world vectors; h: [n]; f: [n][3]; pdf: [n]
void hmo_hair_eval(int64_t n, const float* wo, const float* wi, const float* t, const float* h,
                   const float* hp, float* f, float* pdf);
// u: [n][4]; wi_out: [n][3] world; margin (optional, may be NULL): distance of
// u.x to the nearest lobe-selection boundary (queries with a tiny margin may
// legitimately pick another lobe under last-ulp differences in the lobe pmf).
void hmo_hair_sample(int64_t n, const float* wo, const float* t, const float* h, const float* u,
                     const float* hp, float* wi_out, float* f, float* pdf, float* margin);
// Same, multithreaded over `threads` host threads (CPU baseline timing).
void hmo_hair_eval_mt(int64_t n, const float* wo, const float* wi, const float* t, const float* h,
                      const float* hp, float* f, float* pdf, int threads);
void hmo_hair_sample_mt(int64_t n, const float* wo, const float* t, const float* h, const float* u,
                        const float* hp, float* wi_out, float* f, float* pdf, int threads);

// ---- synthetic BSDF workload (2^18 queries): planar [3][n] layouts like the GPU API
void hmo_gen_bsdf_queries(uint32_t seed, int64_t n, float* wo, float* wi, float* t, float* h,
                          float* u);

// ---- head BRDF (frostbite_anisotropic.cuh:17-157), local-frame vectors
void hmo_frostbite_ggx(const float* wo, const float* wi, const float* color, float alpha, float* out);
void hmo_sample_ggx(const float* rand2, float alpha, const float* v, float* l_out, float* pdf);
float hmo_pdf_ggx(float alpha, const float* v, const float* ne);

// ---- curves (curve_utils.cuh:57-214).  basis 0 = uniform cubic B-spline,
// 1 = Catmull-Rom.  out: pos4, vel4, acc4, tangent3, normal3, projected ps3.
void hmo_curve_eval(int basis, const float* q, float u, const float* ps_in, float* out24);

// ---- utils.cuh
void hmo_orthonormal_basis(const float* n, float* out18);
void hmo_uniform_sample_sphere(const float* u2, float* out3);
float hmo_power_heuristic(float f, float g);
float hmo_luminance(const float* rgb);
float hmo_spherical_theta(const float* v);
float hmo_spherical_phi(const float* v);

#ifdef __cplusplus
}
#endif
