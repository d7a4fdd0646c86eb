// The reference's own HairMSNN integrator, compiled unmodified on the host
// (test infrastructure only; built by oracle/build.py into oracle/_ref/,
// never committed, never shipped).
//
// Reference files included verbatim: cuda/hair_msnn.cu, which includes
// cuda_headers/hair_msnn.cuh, utils.cuh, curve_utils.cuh, disney_hair.cuh,
// frostbite_anisotropic.cuh and optix_common.cuh (directLighting,
// sampleLights, sampleBSDF, the environment light, hairCH, triangleMeshCH,
// miss).  The OptiX launch and traceRay are emulated by ref_harness.h; the
// closest/any hit itself comes from the oracle's LBVH.
#include "hm_owl_shim.h"

thread_local HmShimHitContext hm_shim_ctx;
HmShimTexture hm_shim_textures[16];

#include "ref_eval_order.h"
#include "hair_msnn.cu"

#include "ref_harness.h"

namespace {

// GBuffer (hair_msnn.cuh:31-35) <-> 8 floats: hit, isSurface, p[3], shortPathColor[3]
void gbuf_to_f(const GBuffer& g, float* o) {
  o[0] = g.hit ? 1.f : 0.f;
  o[1] = g.isSurface ? 1.f : 0.f;
  o[2] = g.p.x; o[3] = g.p.y; o[4] = g.p.z;
  o[5] = g.shortPathColor.x; o[6] = g.shortPathColor.y; o[7] = g.shortPathColor.z;
}
GBuffer gbuf_from_f(const float* o) {
  GBuffer g;
  g.hit = o[0] != 0.f;
  g.isSurface = o[1] != 0.f;
  g.p = vec3f(o[2], o[3], o[4]);
  g.shortPathColor = vec3f(o[5], o[6], o[7]);
  return g;
}

}  // namespace

extern "C" {

// The scene's geometry, environment tables and lights (the same arrays as
// hmo_scene_new); trace_scene: the oracle scene whose BVH answers traceRay.
void* hmr_scene_new(void* trace_scene, const float* cp, int n_cp, const int* seg, int n_seg, const float* vtx,
                    const float* nrm, int n_vtx, const int* tri, int n_tri, const float* env, int env_w, int env_h,
                    const float* cpdf, const float* ccdf, const float* mpdf, const float* mcdf, const float* dl,
                    int n_dl, const float* mat16, const int* settings9) {
  return hmref::new_scene(trace_scene, cp, n_cp, seg, n_seg, vtx, nrm, n_vtx, tri, n_tri, env, env_w, env_h, cpdf,
                          ccdf, mpdf, mcdf, dl, n_dl, mat16, settings9);
}

void hmr_scene_free(void* h) { delete (hmref::Scene*)h; }

// One G_BUFFER launch of rayGenCam (hair_msnn.cu:187-312) over the whole
// frame.  train_idx [n_train_idx] is the trainIdxs table; beta_knob is the
// command line's BETA (the launch's beta is BETA - 1, render_hair_msnn.cu:1170).
// Outputs: gbuf [P][8] (hit, isSurface, p, shortPathColor), nn_in [P][12]
// (nnFrameInput), train_in [R][12] / train_out [R][3] (nnTrainInput /
// nnTrainOutput at trOfs); ev / n_ev: per-pixel ray logs (may be NULL).
void hmr_msnn_gbuffer(void* h, const float* camera12, const float* mat16, const int* settings9, float scene_scale,
                      int beta_knob, int accum_id, int every_nth, const int* train_idx, int n_train_idx, float* gbuf,
                      float* nn_in, float* train_in, float* train_out, float* ev, int* n_ev, int max_ev,
                      int threads) {
  hmref::Scene* s = (hmref::Scene*)h;
  const int P = s->width * s->height;
  LaunchParams& lp = optixLaunchParams;
  lp = LaunchParams();
  hmref::set_scene_params(lp, *s, camera12, mat16, settings9, scene_scale);
  lp.pathV1 = settings9[2];
  lp.pathV2 = settings9[3];
  std::vector<GBuffer> gb(P);
  std::vector<int> tidx(train_idx, train_idx + n_train_idx);
  lp.pass = G_BUFFER;
  lp.accumId = accum_id;
  lp.everyNth = every_nth;
  lp.trainIdxs = tidx.data();
  lp.gBuffer = gb.data();
  lp.mlpInputCh = 12;
  lp.mlpOutputCh = 3;
  lp.nnFrameInput = nn_in;
  lp.nnTrainInput = train_in;
  lp.nnTrainOutput = train_out;
  lp.beta = beta_knob - 1;
  hmref::launch(s, threads, ev, n_ev, max_ev, [&](int) { __raygen__rayGenCam(); });
  for (int i = 0; i < P; ++i) gbuf_to_f(gb[i], gbuf + 8 * (size_t)i);
}

// One TRAIN_DATA_GEN launch of rayGenCam (hair_msnn.cu:187-275,
// render_hair_msnn.cu:654-662) over a rec_x x rec_y grid: record trOfs =
// x + rec_x * y aims at points3[scene_indices[trOfs]] and writes
// nnTrainInput / nnTrainOutput [rec_x * rec_y][12] / [..][3] at trOfs.
void hmr_msnn_traingen(void* h, const float* camera12, const float* mat16, const int* settings9, float scene_scale,
                       int beta_knob, int accum_id, int rec_x, int rec_y, const int* scene_indices,
                       const float* points3, int n_points, float* train_in, float* train_out, float* ev, int* n_ev,
                       int max_ev, int threads) {
  hmref::Scene* s = (hmref::Scene*)h;
  LaunchParams& lp = optixLaunchParams;
  lp = LaunchParams();
  hmref::set_scene_params(lp, *s, camera12, mat16, settings9, scene_scale);
  lp.pathV1 = settings9[2];
  lp.pathV2 = settings9[3];
  std::vector<int> sidx(scene_indices, scene_indices + (size_t)rec_x * rec_y);
  std::vector<float3> pts(n_points);
  for (int i = 0; i < n_points; ++i) pts[i] = float3{points3[3 * i], points3[3 * i + 1], points3[3 * i + 2]};
  lp.pass = TRAIN_DATA_GEN;
  lp.accumId = accum_id;
  lp.numTrainRecordsX = rec_x;
  lp.numTrainRecordsY = rec_y;
  lp.numSamples = n_points;
  lp.sceneIndices = sidx.data();
  lp.sampledPoints = pts.data();
  lp.mlpInputCh = 12;
  lp.mlpOutputCh = 3;
  lp.nnTrainInput = train_in;
  lp.nnTrainOutput = train_out;
  lp.beta = beta_knob - 1;
  hmref::launch_grid(s, rec_x, rec_y, threads, ev, n_ev, max_ev, [&](int) { __raygen__rayGenCam(); });
}

// One RENDER launch (hair_msnn.cu:314-356): gbuf_in [P][8] and nn_out [P][3]
// in; the three accumulation buffers [P][4] are read (accum_id > 0) and
// written; the three average buffers [P][4] are written.
void hmr_msnn_render(void* h, int accum_id, const float* gbuf_in, const float* nn_out, float* pt_acc, float* nn_acc,
                     float* final_acc, float* pt_avg, float* nn_avg, float* final_avg, int threads) {
  hmref::Scene* s = (hmref::Scene*)h;
  const int P = s->width * s->height;
  LaunchParams& lp = optixLaunchParams;
  std::vector<GBuffer> gb(P);
  for (int i = 0; i < P; ++i) gb[i] = gbuf_from_f(gbuf_in + 8 * (size_t)i);
  lp.pass = RENDER;
  lp.accumId = accum_id;
  lp.gBuffer = gb.data();
  lp.mlpOutputCh = 3;
  lp.nnFrameOutput = const_cast<float*>(nn_out);
  lp.ptAccumBuffer = (float4*)pt_acc;
  lp.nnAccumBuffer = (float4*)nn_acc;
  lp.finalAccumBuffer = (float4*)final_acc;
  lp.ptAverageBuffer = (float4*)pt_avg;
  lp.nnAverageBuffer = (float4*)nn_avg;
  lp.finalAverageBuffer = (float4*)final_avg;
  hmref::launch(s, threads, nullptr, nullptr, 0, [&](int) { __raygen__rayGenCam(); });
}

}  // extern "C"
