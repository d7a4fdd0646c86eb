// The reference's NRC comparison renderer, compiled unmodified on the host
// (test infrastructure only; built by oracle/build.py into oracle/_ref/,
// never committed, never shipped).
//
// Reference files included verbatim: cuda/nrc.cu (rayGenCam, nrcTracePaths,
// nextPathVertexNRC, nrcGenerateTrainingData), which includes
// cuda_headers/nrc.cuh, utils.cuh, curve_utils.cuh, disney_hair.cuh,
// frostbite_anisotropic.cuh and optix_common.cuh.  The launch and traceRay
// are emulated by ref_harness.h.
//
// One departure, for a defined result: every pixel of the reference writes
// tBuffer[trOfs].bounces / .hit when its path ends (nrc.cu:211-222), so the
// pixels that share a training record race on it on the GPU.  Here each
// pixel writes a train buffer of its own (the pixel loop runs on one thread
// and points tBuffer[trOfs] at the pixel's buffer), which is the training
// pixel's own result.
#include "hm_owl_shim.h"

thread_local HmShimHitContext hm_shim_ctx;
HmShimTexture hm_shim_textures[16];

#include "ref_eval_order.h"
#include "nrc.cu"

#include "ref_harness.h"

extern "C" {

void* hmr_nrc_scene_new(void* trace_scene, const float* cp, int n_cp, const int* seg, int n_seg, const float* vtx,
                        const float* nrm, int n_vtx, const int* tri, int n_tri, const float* env, int env_w,
                        int env_h, const float* cpdf, const float* ccdf, const float* mpdf, const float* mcdf,
                        const float* dl, int n_dl, const float* mat16, const int* settings9) {
  return hmref::new_scene(trace_scene, cp, n_cp, seg, n_seg, vtx, nrm, n_vtx, tri, n_tri, env, env_w, env_h, cpdf,
                          ccdf, mpdf, mcdf, dl, n_dl, mat16, settings9);
}

void hmr_nrc_scene_free(void* h) { delete (hmref::Scene*)h; }

// One G_BUFFER launch of the NRC rayGenCam (nrc.cu:312-356) over the whole
// frame, c the spread threshold (render_nrc.h).  train_idx [n_train_idx]:
// the trainIdxs table.  Outputs per pixel: gbuf [P][8] (hit, pathRadiance,
// beta, bounces), query [(P + n_train_idx)][9] (nnFrameInput: the pixels'
// cache queries, then the training suffixes'), train [P][40][15] (the
// pixel's own train buffer: vert, wo, n, vertRadiance, vertBeta) and
// tinfo [P][2] (bounces, hit of its train buffer); ev / n_ev: ray logs.
void hmr_nrc_gbuffer(void* h, const float* camera12, const float* mat16, const int* settings9, float scene_scale,
                     int accum_id, int every_nth, const int* train_idx, int n_train_idx, float c, int all_unbiased,
                     float* gbuf, float* query, float* train, int* tinfo, float* ev, int* n_ev, int max_ev) {
  hmref::Scene* s = (hmref::Scene*)h;
  const int P = s->width * s->height;
  LaunchParams& lp = optixLaunchParams;
  lp = LaunchParams();
  hmref::set_scene_params(lp, *s, camera12, mat16, settings9, scene_scale);
  std::vector<GBuffer> gb(P);
  std::vector<TrainBuffer> tb(P);
  std::vector<int> tidx(train_idx, train_idx + n_train_idx);
  lp.pass = G_BUFFER;
  lp.accumId = accum_id;
  lp.everyNth = every_nth;
  lp.trainIdxs = tidx.data();
  lp.gBuffer = gb.data();
  lp.mlpInputCh = 9;
  lp.mlpOutputCh = 3;
  lp.nnFrameInput = query;
  lp.c = c;
  lp.allUnbiased = all_unbiased != 0;
  hmref::launch(s, 1, ev, n_ev, max_ev, [&](int pid) {
    const int tr = pid / every_nth;
    lp.tBuffer = tb.data() + pid - tr;  // tBuffer[trOfs] is this pixel's own buffer
    __raygen__rayGenCam();
  });
  for (int i = 0; i < P; ++i) {
    const GBuffer& g = gb[i];
    float* o = gbuf + 8 * (size_t)i;
    o[0] = g.hit ? 1.f : 0.f;
    o[1] = g.pathRadiance.x; o[2] = g.pathRadiance.y; o[3] = g.pathRadiance.z;
    o[4] = g.beta.x; o[5] = g.beta.y; o[6] = g.beta.z;
    o[7] = (float)g.bounces;
    const TrainBuffer& t = tb[i];
    for (int b = 0; b < MAX_BOUNCES; ++b) {
      float* r = train + ((size_t)i * MAX_BOUNCES + b) * 15;
      const vec3f* v[5] = {&t.vert[b], &t.wo[b], &t.n[b], &t.vertRadiance[b], &t.vertBeta[b]};
      for (int k = 0; k < 5; ++k) {
        r[3 * k] = v[k]->x;
        r[3 * k + 1] = v[k]->y;
        r[3 * k + 2] = v[k]->z;
      }
    }
    tinfo[2 * i] = t.bounces;
    tinfo[2 * i + 1] = t.hit ? 1 : 0;
  }
}

// One RENDER launch of the NRC rayGenCam (nrc.cu:365-380): per pixel the
// composed colour through writePixel (accum [P][4] read when accum_id > 0 and
// written; avg [P][4]); per training pixel nrcGenerateTrainingData
// (nrc.cu:70-133): train_in [n_train_idx][40][9] and train_gt
// [n_train_idx][40][3] at trOfs.  gbuf [P][8] and train [P][40][15] / tinfo
// [P][2] in the layouts hmr_nrc_gbuffer returns (each pixel's own train
// buffer stands at tBuffer[trOfs]); nn_out [(P + n_train_idx)][3] the cache
// outputs (pixels' queries, then the training suffixes').
void hmr_nrc_render(void* h, int accum_id, int every_nth, const int* train_idx, int n_train_idx, int all_unbiased,
                    const float* gbuf, const float* train, const int* tinfo, const float* nn_out, float* accum,
                    float* avg, float* train_in, float* train_gt) {
  hmref::Scene* s = (hmref::Scene*)h;
  const int P = s->width * s->height;
  LaunchParams& lp = optixLaunchParams;
  std::vector<GBuffer> gb(P);
  std::vector<TrainBuffer> tb(P);
  for (int i = 0; i < P; ++i) {
    const float* g = gbuf + 8 * (size_t)i;
    gb[i].hit = g[0] != 0.f;
    gb[i].pathRadiance = vec3f(g[1], g[2], g[3]);
    gb[i].beta = vec3f(g[4], g[5], g[6]);
    gb[i].bounces = (int)g[7];
    for (int b = 0; b < MAX_BOUNCES; ++b) {
      const float* r = train + ((size_t)i * MAX_BOUNCES + b) * 15;
      tb[i].vert[b] = vec3f(r[0], r[1], r[2]);
      tb[i].wo[b] = vec3f(r[3], r[4], r[5]);
      tb[i].n[b] = vec3f(r[6], r[7], r[8]);
      tb[i].vertRadiance[b] = vec3f(r[9], r[10], r[11]);
      tb[i].vertBeta[b] = vec3f(r[12], r[13], r[14]);
    }
    tb[i].bounces = tinfo[2 * i];
    tb[i].hit = tinfo[2 * i + 1] != 0;
  }
  std::vector<int> tidx(train_idx, train_idx + n_train_idx);
  std::vector<float3> gt((size_t)n_train_idx * MAX_BOUNCES, float3{0.f, 0.f, 0.f});
  lp.pass = RENDER;
  lp.accumId = accum_id;
  lp.everyNth = every_nth;
  lp.trainIdxs = tidx.data();
  lp.allUnbiased = all_unbiased != 0;
  lp.gBuffer = gb.data();
  lp.mlpInputCh = 9;
  lp.mlpOutputCh = 3;
  lp.nnFrameOutput = (float3*)const_cast<float*>(nn_out);
  lp.accumBuffer = (float4*)accum;
  lp.averageBuffer = (float4*)avg;
  lp.trainInput = train_in;
  lp.trainGT = gt.data();
  hmref::launch(s, 1, nullptr, nullptr, 0, [&](int pid) {
    const int tr = pid / every_nth;
    lp.tBuffer = tb.data() + pid - tr;  // tBuffer[trOfs] is this pixel's own buffer
    __raygen__rayGenCam();
  });
  for (size_t k = 0; k < gt.size(); ++k) {
    train_gt[3 * k] = gt[k].x;
    train_gt[3 * k + 1] = gt[k].y;
    train_gt[3 * k + 2] = gt[k].z;
  }
}

}  // extern "C"
