// Host harness for the reference's own OptiX programs (test infrastructure
// only).  Included by ref_path_entry.cpp, ref_pt_entry.cpp and
// ref_nrc_entry.cpp after the reference's raygen source, so that
// `LaunchParams` and `optixLaunchParams` are the reference's own
// (hair_msnn.cuh, path_tracing.cuh or nrc.cuh).
//
// What it emulates:
//  * owl::traceRay (hm_shim_trace_hook): the ray is answered by the oracle's
//    LBVH (hmo_trace_rays in oracle/_build/libhmoracle.so, the one closed
//    piece of the path: OptiX's curve intersector), and the hit is handed to
//    the reference's own programs exactly as OptiX would: hairCH /
//    triangleMeshCH for the closest radiance hit, miss for a radiance miss,
//    hairAHShadow / triangleMeshAHShadow for a shadow-ray hit.  OWL creates
//    one miss program, for ray type 0 (render_hair_msnn.cu:602), so a shadow
//    miss calls nothing.
//  * tex2D on the environment map (linear filter) and the four sampling
//    tables (nearest), clamp addressing, as created in
//    render_hair_msnn.cu:163-198.
//  * the launch: rayGenCam is called once per pixel with the launch index
//    set, on a few host threads.
// Every ray the programs trace is also logged per pixel in the oracle's
// event format (kind, result, t, u, origin, direction), so the tests can
// compare the two integrators ray by ray.
#pragma once

#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <thread>
#include <vector>

extern "C" void hmo_trace_rays(void* h, const float* org, const float* dir, int n, float tmin, float tmax, int any,
                               float* hits);

namespace hmref {

constexpr int kEvFloats = 12;

struct Scene {
  void* trace_scene = nullptr;  // the oracle's scene (its BVH answers traceRay)
  std::vector<float> cp;        // [n_cp][4]
  std::vector<int> seg;
  std::vector<vec3f> vtx, nrm;
  std::vector<vec3i> tri;
  std::vector<vec2f> uv;
  std::vector<float> env, cpdf, ccdf, mpdf, mcdf;
  std::vector<DirectionalLight> dl;
  TriangleMeshData tri_data;
  HairData hair_data;
  MissProgData miss_data;
  RayGenData raygen;
  std::vector<uint32_t> frame_buffer;
  int width = 0, height = 0, env_w = 0, env_h = 0;
  int n_seg() const { return (int)seg.size(); }
};

Scene* g_scene = nullptr;  // the scene of the running launch

struct EvLog {
  float* ev = nullptr;
  int cap = 0, n = 0;
};
thread_local EvLog* tl_log = nullptr;

inline void log_event(int kind, int result, float t, float u, const float* o, const float* d) {
  EvLog* L = tl_log;
  if (!L) return;
  if (L->n < L->cap) {
    float* e = L->ev + (size_t)L->n * kEvFloats;
    memcpy(e + 0, &kind, 4);
    memcpy(e + 1, &result, 4);
    e[2] = t;
    e[3] = u;
    for (int i = 0; i < 3; ++i) {
      e[4 + i] = o[i];
      e[7 + i] = d[i];
    }
    e[10] = 0.f;
    e[11] = 0.f;
  }
  ++L->n;
}

// Fills optixLaunchParams' scene fields (shared by the MSNN, PT and NRC
// launch parameter blocks) and the texture registry.
template <class LP>
void set_scene_params(LP& lp, const Scene& s, const float* camera12, const float* mat16, const int* settings9,
                      float scene_scale) {
  lp.hasEnvLight = settings9[6] != 0;
  lp.envPdfSampling = settings9[5] != 0;
  lp.envScale = mat16[14];
  lp.envRotPhi = mat16[15];
  lp.envWidth = s.env_w;
  lp.envHeight = s.env_h;
  // texture handles index hm_shim_textures
  lp.env = 0;
  lp.conditionalPdf = 1;
  lp.conditionalCdf = 2;
  lp.marginalPdf = 3;
  lp.marginalCdf = 4;
  lp.hasDirectionalLights = !s.dl.empty();
  lp.dLights = const_cast<DirectionalLight*>(s.dl.data());
  lp.num_dlights = (int)s.dl.size();
  lp.num_total_lights = lp.num_dlights + (lp.hasEnvLight ? 1 : 0);
  lp.camera.pos = vec3f(camera12[0], camera12[1], camera12[2]);
  lp.camera.dir_00 = vec3f(camera12[3], camera12[4], camera12[5]);
  lp.camera.dir_du = vec3f(camera12[6], camera12[7], camera12[8]);
  lp.camera.dir_dv = vec3f(camera12[9], camera12[10], camera12[11]);
  lp.hairData.sig_a = vec3f(mat16[0], mat16[1], mat16[2]);
  lp.hairData.beta_m = mat16[3];
  lp.hairData.beta_n = mat16[4];
  lp.hairData.alpha = mat16[5];
  lp.hairData.R_G = mat16[6];
  lp.hairData.TT_G = mat16[7];
  lp.hairData.TRT_G = mat16[8];
  lp.hairData.TRRT_G = mat16[9];
  lp.MIS = settings9[4] != 0;
  lp.sceneScale = scene_scale;
  if (lp.hasEnvLight) {
    const int w = lp.envWidth, h = lp.envHeight;
    hm_shim_textures[0] = HmShimTexture{s.env.data(), w, h, 4, 1};
    hm_shim_textures[1] = HmShimTexture{s.cpdf.data(), w + 1, h, 1, 0};
    hm_shim_textures[2] = HmShimTexture{s.ccdf.data(), w + 1, h, 1, 0};
    hm_shim_textures[3] = HmShimTexture{s.mpdf.data(), h + 1, 1, 1, 0};
    hm_shim_textures[4] = HmShimTexture{s.mcdf.data(), h + 1, 1, 1, 0};
  }
}

inline Scene* new_scene(void* trace_scene, const float* cp, int n_cp, const int* seg, int n_seg, const float* vtx,
                        const float* nrm, int n_vtx, const int* tri, int n_tri, const float* env, int env_w,
                        int env_h, const float* cpdf, const float* ccdf, const float* mpdf, const float* mcdf,
                        const float* dl, int n_dl, const float* mat16, const int* settings9) {
  Scene* s = new Scene();
  s->trace_scene = trace_scene;
  s->cp.assign(cp, cp + 4 * (size_t)n_cp);
  s->seg.assign(seg, seg + n_seg);
  for (int i = 0; i < n_vtx; ++i) {
    s->vtx.push_back(vec3f(vtx[3 * i], vtx[3 * i + 1], vtx[3 * i + 2]));
    s->nrm.push_back(vec3f(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]));
    s->uv.push_back(vec2f(0.f, 0.f));
  }
  for (int i = 0; i < n_tri; ++i) s->tri.push_back(vec3i(tri[3 * i], tri[3 * i + 1], tri[3 * i + 2]));
  s->env_w = env_w;
  s->env_h = env_h;
  if (env_w > 0) {
    s->env.assign(env, env + 4 * (size_t)env_w * env_h);
    s->cpdf.assign(cpdf, cpdf + (size_t)(env_w + 1) * env_h);
    s->ccdf.assign(ccdf, ccdf + (size_t)(env_w + 1) * env_h);
    s->mpdf.assign(mpdf, mpdf + env_h + 1);
    s->mcdf.assign(mcdf, mcdf + env_h + 1);
  }
  for (int i = 0; i < n_dl; ++i) {
    DirectionalLight L;
    L.from = vec3f(dl[6 * i], dl[6 * i + 1], dl[6 * i + 2]);
    L.emit = vec3f(dl[6 * i + 3], dl[6 * i + 4], dl[6 * i + 5]);
    s->dl.push_back(L);
  }
  s->tri_data.vertex = s->vtx.data();
  s->tri_data.normal = s->nrm.data();
  s->tri_data.index = s->tri.data();
  s->tri_data.texCoord = s->uv.data();
  s->tri_data.diffuse = vec3f(mat16[10], mat16[11], mat16[12]);
  s->tri_data.hasDiffuseTexture = false;
  s->tri_data.alpha = mat16[13];  // the mesh's own alpha; triangleMeshCH clamps and squares it
  s->tri_data.hasAlphaTexture = false;
  s->width = settings9[0];
  s->height = settings9[1];
  s->raygen.frameBufferSize = vec2i(s->width, s->height);
  s->frame_buffer.assign((size_t)s->width * s->height, 0u);
  s->raygen.frameBuffer = s->frame_buffer.data();
  return s;
}

// Runs fn(index) for every index of an lw x lh launch grid with the launch
// index and the raygen's program data (whose frameBufferSize stays the
// frame's) set; ev/n_ev/max_ev: optional per-index event logs.
template <class Fn>
void launch_grid(Scene* s, int lw, int lh, int threads, float* ev, int* n_ev, int max_ev, Fn fn) {
  g_scene = s;
  const int P = lw * lh;
  auto work = [&](int b, int e) {
    EvLog log;
    for (int pid = b; pid < e; ++pid) {
      if (ev) {
        log.ev = ev + (size_t)pid * max_ev * kEvFloats;
        log.cap = max_ev;
        log.n = 0;
        tl_log = &log;
      }
      hm_shim_ctx = HmShimHitContext();
      hm_shim_ctx.launch_x = pid % lw;
      hm_shim_ctx.launch_y = pid / lw;
      hm_shim_ctx.program_data = &s->raygen;
      fn(pid);
      if (n_ev) n_ev[pid] = log.n;
    }
    tl_log = nullptr;
  };
  threads = std::max(1, threads);
  if (threads == 1) {
    work(0, P);
    return;
  }
  std::vector<std::thread> pool;
  const int chunk = (P + threads - 1) / threads;
  for (int k = 0; k < threads; ++k) {
    const int b = k * chunk, e = std::min(P, b + chunk);
    if (b < e) pool.emplace_back(work, b, e);
  }
  for (auto& t : pool) t.join();
}

// The frame-sized launch: fn(pixel) for every pixel.
template <class Fn>
void launch(Scene* s, int threads, float* ev, int* n_ev, int max_ev, Fn fn) {
  launch_grid(s, s->width, s->height, threads, ev, n_ev, max_ev, fn);
}

}  // namespace hmref

// owl::traceRay: the oracle's BVH finds the hit, the reference's programs
// shade it (see the header comment).
extern "C" void hm_shim_trace_hook(int ray_type, const float* org, const float* dir, float tmin, float tmax,
                                   void* prd) {
  const hmref::Scene& s = *hmref::g_scene;
  float hit[4];
  hmo_trace_rays(s.trace_scene, org, dir, 1, tmin, tmax, ray_type == RADIANCE_RAY_TYPE ? 0 : 1, hit);
  int prim;
  memcpy(&prim, hit + 1, 4);
  const HmShimHitContext saved = hm_shim_ctx;
  hm_shim_ctx.prd = prd;
  hm_shim_ctx.ray_origin = float3{org[0], org[1], org[2]};
  hm_shim_ctx.ray_dir = float3{dir[0], dir[1], dir[2]};
  hm_shim_ctx.ray_tmax = hit[0];
  hm_shim_ctx.terminated = 0;
  if (ray_type == RADIANCE_RAY_TYPE) {
    if (prim < 0) {
      hm_shim_ctx.program_data = &s.miss_data;
      __miss__miss();
    } else if (prim < s.n_seg()) {
      hm_shim_ctx.primitive_index = prim;
      hm_shim_ctx.curve_u = hit[2];
      const float* q = &s.cp[4 * (size_t)s.seg[prim]];
      for (int i = 0; i < 4; ++i) hm_shim_ctx.cps[i] = float4{q[4 * i], q[4 * i + 1], q[4 * i + 2], q[4 * i + 3]};
      hm_shim_ctx.program_data = &s.hair_data;
      __closesthit__hairCH();
    } else {
      hm_shim_ctx.primitive_index = prim - s.n_seg();
      hm_shim_ctx.barycentrics = float2{hit[2], hit[3]};
      hm_shim_ctx.program_data = &s.tri_data;
      __closesthit__triangleMeshCH();
    }
    hmref::log_event(0, prim < 0 ? -1 : prim, prim < 0 ? 0.f : hit[0], prim < 0 ? 0.f : hit[2], org, dir);
  } else if (ray_type == SHADOW_RAY_TYPE) {
    if (prim >= 0) {
      if (prim < s.n_seg())
        __anyhit__hairAHShadow();
      else
        __anyhit__triangleMeshAHShadow();
    }
    hmref::log_event(1, prim < 0 ? 1 : 0, 0.f, 0.f, org, dir);
  }
  const int lx = saved.launch_x, ly = saved.launch_y;
  hm_shim_ctx = saved;
  hm_shim_ctx.launch_x = lx;
  hm_shim_ctx.launch_y = ly;
}
