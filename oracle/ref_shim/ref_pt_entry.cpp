// The reference's plain path tracer, compiled unmodified on the host (test
// infrastructure only; built by oracle/build.py into oracle/_ref/, never
// committed, never shipped).
//
// Reference files included verbatim: cuda/path_tracing.cu (rayGenCam +
// writePixel), which includes cuda_headers/path_tracing.cuh, utils.cuh,
// curve_utils.cuh, disney_hair.cuh, frostbite_anisotropic.cuh and
// optix_common.cuh (pathTrace, nextPathVertex, directLighting and the hit /
// miss programs).  The launch and traceRay are emulated by ref_harness.h.
#include "hm_owl_shim.h"

thread_local HmShimHitContext hm_shim_ctx;
HmShimTexture hm_shim_textures[16];

#include "ref_eval_order.h"
#include "path_tracing.cu"

#include "ref_harness.h"

extern "C" {

void* hmr_pt_scene_new(void* trace_scene, const float* cp, int n_cp, const int* seg, int n_seg, const float* vtx,
                       const float* nrm, int n_vtx, const int* tri, int n_tri, const float* env, int env_w,
                       int env_h, const float* cpdf, const float* ccdf, const float* mpdf, const float* mcdf,
                       const float* dl, int n_dl, const float* mat16, const int* settings9) {
  return hmref::new_scene(trace_scene, cp, n_cp, seg, n_seg, vtx, nrm, n_vtx, tri, n_tri, env, env_w, env_h, cpdf,
                          ccdf, mpdf, mcdf, dl, n_dl, mat16, settings9);
}

void hmr_pt_scene_free(void* h) { delete (hmref::Scene*)h; }

// One launch of the path tracer's rayGenCam (path_tracing.cu:19-66): accum
// [P][4] is read (accum_id > 0) and written, avg [P][4] written; ev / n_ev:
// per-pixel ray logs (may be NULL).
void hmr_pt_frame(void* h, const float* camera12, const float* mat16, const int* settings9, float scene_scale,
                  int accum_id, float* accum, float* avg, float* ev, int* n_ev, int max_ev, int threads) {
  hmref::Scene* s = (hmref::Scene*)h;
  LaunchParams& lp = optixLaunchParams;
  lp = LaunchParams();
  hmref::set_scene_params(lp, *s, camera12, mat16, settings9, scene_scale);
  lp.pathV1 = settings9[2];
  lp.pathV2 = settings9[3];
  lp.accumId = accum_id;
  lp.accumBuffer = (float4*)accum;
  lp.averageBuffer = (float4*)avg;
  hmref::launch(s, threads, ev, n_ev, max_ev, [&](int) { __raygen__rayGenCam(); });
}

}  // extern "C"
