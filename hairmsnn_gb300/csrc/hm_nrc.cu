// Neural radiance caching, the comparison integrator of the reference
// (Müller et al. 2021 as cuda/nrc.cu:17-397 and render_nrc.cu:640-701
// implement it), on the wavefront.  Compiled with -fmad=false, like the
// other shading units.
//
//   nrc_shade_kernel     one path vertex of nrcTracePaths (nrc.cu:136-310):
//                        the spread test against the previous vertex, the
//                        cache query where the spread passes c * a0 (and,
//                        for training pixels, the training suffix), direct
//                        lighting (shadow rays resolved later), the next
//                        vertex (nextPathVertexNRC, nrc.cu:17-66); no Russian
//                        roulette, at most 40 vertices (MAX_BOUNCES)
//   nrc_finalize_kernel  G-buffer of the paths that ended without a snapshot
//   nrc_compose_kernel   RENDER pass: radiance + beta * max(cache, 0), FP64
//                        accumulation (writePixel)
//   nrc_train_data_kernel  nrcGenerateTrainingData (nrc.cu:67-133): one
//                        record per vertex of each training pixel's path
#include "hm_render.h"
#include "hm_shading.cuh"

namespace hm {

HM_D f3 ld4(const float4* p, int i) {
  const float4 v = p[i];
  return mk(v.x, v.y, v.z);
}
HM_D void st4(float4* p, int i, f3 v, float w = 0.f) { p[i] = make_float4(v.x, v.y, v.z, w); }

// Cache query row: position / scene scale, wo, n (nrc.cu:236-250).
HM_D void nrc_query(float* row, const SceneDev& s, const Vertex& v) {
  const f3 q = v.p / s.scene_scale;
  row[0] = q.x; row[1] = q.y; row[2] = q.z;
  row[3] = v.wo.x; row[4] = v.wo.y; row[5] = v.wo.z;
  row[6] = v.n.x; row[7] = v.n.y; row[8] = v.n.z;
}

// Camera rays with the NRC per-frame reset of the pixel's G-buffer, cache
// query rows and (training pixels) train buffer (RESET pass, nrc.cu:371-386,
// and the buffer clears of render_nrc.cu:683-687).
__global__ void __launch_bounds__(256) nrc_camera_kernel(const __grid_constant__ SceneDev s, FrameParams fp,
                                                         PathState ps, FrameBufs fb, NrcBufs nb, int* queue,
                                                         int* count) {
  const int P = s.width * s.height;
  const int pid = blockIdx.x * blockDim.x + threadIdx.x;
  if (pid == 0) *count = P;
  if (pid >= P) return;
  const int x = pid % s.width, y = pid / s.width;
  const int accum_id = fp.d_frame ? *fp.d_frame : fp.accum_id;
  uint32_t rng = rng_seed(fp.d_frame ? accum_id + 10007 : fp.frame_seed, (uint32_t)pid);
  uint32_t flags = 0;
  const int tr = pid / fp.every_nth;
  if (tr < fp.n_train) {
    const uint32_t pick = feistel_perm((uint32_t)tr, (uint32_t)fp.n_train, (uint32_t)accum_id) % fp.every_nth;
    if ((uint32_t)(pid % fp.every_nth) == pick) {
      flags |= F_TRAIN;
      if (tr % 16 == 0 || nb.all_unbiased) flags |= F_NRC_UNBIASED;  // rayGenCam, nrc.cu:327
      nb.tinfo[tr] = make_int4(0, 0, (flags & F_NRC_UNBIASED) ? 1 : 0, 0);
      float* row = fb.nn_frame_in + ((size_t)P + tr) * fp.in_ch;
      for (int c = 0; c < fp.in_ch; ++c) row[c] = 0.f;
    }
  }
  float* row = fb.nn_frame_in + (size_t)pid * fp.in_ch;
  for (int c = 0; c < fp.in_ch; ++c) row[c] = 0.f;
  nb.gbeta[pid] = make_float4(0.f, 0.f, 0.f, 0.f);
  const float ox = lcg_next(rng), oy = lcg_next(rng);
  const float su = ((float)x + ox) / (float)s.width, sv = ((float)y + oy) / (float)s.height;
  const f3 dir = normalize(s.cam_d00 + su * s.cam_du + sv * s.cam_dv);
  ps.rng[pid] = rng;
  ps.flags[pid] = flags;
  ps.bounce[pid] = 0;
  st4(ps.ray_o, pid, s.cam_pos);
  st4(ps.ray_d, pid, dir);
  st4(ps.beta, pid, splat(1.f));
  st4(ps.col, pid, splat(0.f));
  nb.dl_rec[pid] = -1;
  queue[pid] = pid;
}

// The end of a path: the training pixel's bounce count (records 0..bounces-1
// are used) and whether its suffix ended at a cache query.
HM_D void nrc_end_train(const NrcBufs& nb, int tr, int bounces, int hit) {
  int4 t = nb.tinfo[tr];
  t.x = bounces;
  t.y = hit;
  t.w = 1;  // primary hit: the records are valid
  nb.tinfo[tr] = t;
}

__global__ void __launch_bounds__(128) nrc_shade_kernel(const __grid_constant__ SceneDev s, FrameParams fp,
                                                        PathState ps, FrameBufs fb, NrcBufs nb,
                                                        const int* __restrict__ queue, const int* __restrict__ count,
                                                        int* __restrict__ keep) {
  const int n = *count;
  const int P = s.width * s.height;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int pid = queue[i];
    uint32_t flags = ps.flags[pid];
    const int k = ps.bounce[pid];
    const float4 h = ps.hit[pid];
    const bool hit = __float_as_int(h.y) >= 0;
    const bool train = flags & F_TRAIN;
    const int tr = pid / fp.every_nth;
    const f3 ro = ld4(ps.ray_o, pid), rd = ld4(ps.ray_d, pid);
    const float4 hr = hit ? refit_hit(s, ro, rd, h) : h;
    if (fp.log.ev)
      log_ray(fp.log, pid, 3 * k, 0, hit ? __float_as_int(hr.y) : -1, hit ? hr.x : 0.f, hit ? hr.z : 0.f,
              ps.rng[pid], ro, rd);
    nb.dl_rec[pid] = -1;
    if (k == 0 && !hit) {  // camera ray missed: G-buffer = Le, no cache (rayGenCam, nrc.cu:343-350)
      st4(fb.gbuf, pid, env_radiance(s, rd), 0.f);
      ps.flags[pid] = flags | F_NRC_GSNAP;
      keep[i] = 0;
      continue;
    }
    if (!hit) {  // si.hit == false after the last vertex: the path ends with beta 0
      if (train) nrc_end_train(nb, tr, k - 1, 0);
      ps.flags[pid] = flags;
      keep[i] = 0;
      continue;
    }
    const Vertex v = setup_vertex(s, ro, rd, hr);
    float4 sp = nb.spread[pid];  // spread, a0
    f3 beta = ld4(ps.beta, pid);
    if (k == 0) {
      if (v.surface && v.wo_local.z < 0.f) {  // back of the head: treated as a miss, Le = 0
        st4(fb.gbuf, pid, splat(0.f), 0.f);
        ps.flags[pid] = flags | F_NRC_GSNAP;
        keep[i] = 0;
        continue;
      }
      flags |= F_PRIM_HIT;
      const float l = length(v.p - s.cam_pos);
      sp = make_float4(0.f, l * l / (4.f * kPi) / fabsf(v.wo_local.z), 0.f, 0.f);
    } else {
      // nrcSpread (utils.cuh:86-90) from the previous vertex, then the end
      // tests of the reference's iteration k - 1 (nrc.cu:207-303)
      const float4 prev = nb.prev[pid];
      const f3 pp = mk(prev.x, prev.y, prev.z);
      const float l = length(v.p - pp);
      if (flags & F_NRC_RECALC) {  // a0 of a training suffix (nrc.cu:192-195)
        sp.y = l * l / (4.f * kPi) / fabsf(v.wo_local.z);
        flags &= ~F_NRC_RECALC;
      }
      sp.x = sp.x + sqrtf(l * l / prev.w / fabsf(v.wo_local.z));
      const float c = (flags & F_NRC_NOSPREAD) ? 1e30f : nb.c;
      const bool spread_cond = sp.x * sp.x > c * sp.y;
      if (spread_cond && !(flags & F_NRC_SUFFIX)) {
        // the pixel's path stops here and takes the cache (nrc.cu:225-270)
        nrc_query(fb.nn_frame_in + (size_t)pid * fp.in_ch, s, v);
        st4(nb.gbeta, pid, beta);
        if (train) {
          st4(fb.gbuf, pid, ld4(ps.col, pid), 1.f);  // the G-buffer keeps the prefix
          flags |= F_NRC_GSNAP | F_NRC_SUFFIX | F_NRC_RECALC;
          sp.x = 0.f;
        } else {
          ps.flags[pid] = flags;
          keep[i] = 0;
          continue;
        }
      } else if (spread_cond && (flags & F_NRC_SUFFIX)) {
        // the training suffix ends at a cache query (nrc.cu:271-302)
        nrc_query(fb.nn_frame_in + ((size_t)P + tr) * fp.in_ch, s, v);
        nrc_end_train(nb, tr, k - 1, 1);
        if (!(flags & F_NRC_UNBIASED)) {
          ps.flags[pid] = flags;
          keep[i] = 0;
          continue;
        }
        flags |= F_NRC_NOSPREAD;  // unbiased pixels trace on (c = 1e30)
      }
    }
    uint32_t rng = ps.rng[pid];
    // ---- direct lighting at this vertex
    ShadowSample ss[2];
    direct_lighting(s, v, rng, ss);
    if (fp.log.ev) {
      fp.log.vcur[pid] = k;
      for (int j = 0; j < 2; ++j)
        if (ss[j].valid) log_ray(fp.log, pid, 3 * k + 1 + j, 1 + j, kLogPending, 0.f, 0.f, 0u, ss[j].o, ss[j].d);
    }
    st4(ps.sh_o0, pid, ss[0].o, ss[0].valid ? 1.f : 0.f);
    st4(ps.sh_d0, pid, ss[0].d);
    st4(ps.sh_c0, pid, ss[0].c);
    st4(ps.sh_o1, pid, ss[1].o, ss[1].valid ? 1.f : 0.f);
    st4(ps.sh_d1, pid, ss[1].d);
    st4(ps.sh_c1, pid, ss[1].c);
    st4(ps.dl_w, pid, beta);
    flags |= F_DL;
    float4* rec = nb.rec + ((size_t)tr * kNrcMaxBounces + k) * kNrcRecordF4;
    if (train) {
      nb.dl_rec[pid] = tr * kNrcMaxBounces + k;  // the resolve writes the vertex's direct light
      const f3 q = v.p / s.scene_scale;
      rec[0] = make_float4(q.x, q.y, q.z, 0.f);
      st4(rec + 1, 0, v.wo);
      st4(rec + 2, 0, v.n);
    }
    // ---- next vertex (nextPathVertexNRC); the last vertex ends the path
    int k_keep = 0;
    if (k == kNrcMaxBounces - 1) {
      if (train) nrc_end_train(nb, tr, k, 0);
    } else {
      f3 o, d;
      float pdf = 1.f;
      const f3 mul = next_vertex(s, v, rng, &o, &d, nullptr, nullptr, nullptr, &pdf);
      if (train) st4(rec + 4, 0, mul);
      beta = beta * mul;
      nb.prev[pid] = make_float4(v.p.x, v.p.y, v.p.z, pdf);
      st4(ps.ray_o, pid, o);
      st4(ps.ray_d, pid, d);
      ps.bounce[pid] = k + 1;
      k_keep = 1;
    }
    nb.spread[pid] = sp;
    st4(ps.beta, pid, beta);
    ps.rng[pid] = rng;
    ps.flags[pid] = flags;
    keep[i] = k_keep;
  }
}

// G-buffer of the paths that ended without a snapshot: their whole radiance
// (nrc.cu:211-222; a cache query, if any, was recorded with its beta).
__global__ void __launch_bounds__(256) nrc_finalize_kernel(int P, PathState ps, FrameBufs fb, float4* col_out) {
  const int pid = blockIdx.x * blockDim.x + threadIdx.x;
  if (pid >= P) return;
  const uint32_t flags = ps.flags[pid];
  if (col_out) col_out[pid] = ps.col[pid];
  if (flags & F_NRC_GSNAP) return;
  const float4 c = ps.col[pid];
  fb.gbuf[pid] = make_float4(c.x, c.y, c.z, 1.f);
}

HM_D bool nan3(f3 c) { return isnan(c.x) || isnan(c.y) || isnan(c.z); }

// RENDER pass (nrc.cu:357-369): color = radiance + beta * max(cache, 0), a
// NaN cache read as 0; writePixel's FP64 accumulation (utils.cuh:13-35).
__global__ void __launch_bounds__(256) nrc_compose_kernel(int P, FrameParams fp, FrameBufs fb, NrcBufs nb) {
  const int pid = blockIdx.x * blockDim.x + threadIdx.x;
  if (pid >= P) return;
  const float4 g = fb.gbuf[pid];
  const float4 b = nb.gbeta[pid];
  f3 cache = mk(fb.nn_frame_out[3 * (size_t)pid], fb.nn_frame_out[3 * (size_t)pid + 1],
                fb.nn_frame_out[3 * (size_t)pid + 2]);
  if (nan3(cache)) cache = splat(0.f);
  cache = mk(fmaxf(cache.x, 0.f), fmaxf(cache.y, 0.f), fmaxf(cache.z, 0.f));
  f3 color = mk(g.x, g.y, g.z) + mk(b.x, b.y, b.z) * cache;
  if (nan3(color)) color = splat(0.f);
  double* a = fb.acc_final + 3 * (size_t)pid;
  if (fp.accum_id == 0) {
    a[0] = color.x; a[1] = color.y; a[2] = color.z;
  } else {
    a[0] += color.x; a[1] += color.y; a[2] += color.z;
  }
}

// nrcGenerateTrainingData (nrc.cu:67-133): record b of training pixel tr is
// the vertex's (position, wo, n) with target = sum over later recorded
// vertices of their direct light times the factors in between, plus the
// suffix's cache (if it ended at one and the pixel is not unbiased) times all
// the factors.  As in the reference, the vertex at which the path ended is
// not among the records (sub < bounces), and records past the end are 0.
__global__ void __launch_bounds__(64) nrc_train_data_kernel(int P, int n_pix, FrameParams fp, FrameBufs fb,
                                                            NrcBufs nb) {
  const int tr = blockIdx.x * blockDim.x + threadIdx.x;
  if (tr >= n_pix) return;
  const int4 info = nb.tinfo[tr];
  const int bounces = info.w ? info.x : 0;
  f3 cache = splat(0.f);
  if (info.w && info.y && !info.z)
    cache = mk(fb.nn_frame_out[3 * ((size_t)P + tr)], fb.nn_frame_out[3 * ((size_t)P + tr) + 1],
               fb.nn_frame_out[3 * ((size_t)P + tr) + 2]);
  const float4* rec = nb.rec + (size_t)tr * kNrcMaxBounces * kNrcRecordF4;
  for (int b = 0; b < kNrcMaxBounces; ++b) {
    float* in = fb.nn_train_in + ((size_t)tr * kNrcMaxBounces + b) * fp.in_ch;
    float* out = fb.nn_train_out + ((size_t)tr * kNrcMaxBounces + b) * 3;
    if (b >= bounces) {
      for (int c = 0; c < fp.in_ch; ++c) in[c] = 0.f;
      out[0] = out[1] = out[2] = 0.f;
      continue;
    }
    f3 color = splat(0.f), beta = splat(1.f);
    for (int sub = b; sub < bounces; ++sub) {
      const float4* r = rec + (size_t)sub * kNrcRecordF4;
      color = color + beta * mk(r[3].x, r[3].y, r[3].z);
      beta = beta * mk(r[4].x, r[4].y, r[4].z);
    }
    const float4* r = rec + (size_t)b * kNrcRecordF4;
    in[0] = r[0].x; in[1] = r[0].y; in[2] = r[0].z;
    in[3] = r[1].x; in[4] = r[1].y; in[5] = r[1].z;
    in[6] = r[2].x; in[7] = r[2].y; in[8] = r[2].z;
    for (int c = 9; c < fp.in_ch; ++c) in[c] = 0.f;
    f3 t = color + beta * cache;
    if (nan3(t)) t = splat(0.f);
    out[0] = t.x; out[1] = t.y; out[2] = t.z;
  }
}

int launch_nrc_camera(const SceneDev& s, const FrameParams& fp, const PathState& ps, const FrameBufs& fb,
                      const NrcBufs& nb, int* queue, int* count, cudaStream_t st) {
  const int P = s.width * s.height;
  nrc_camera_kernel<<<(P + 255) / 256, 256, 0, st>>>(s, fp, ps, fb, nb, queue, count);
  HM_CHECK_LAUNCH("nrc_camera_kernel");
  return HM_OK;
}

int launch_nrc_shade(const SceneDev& s, const FrameParams& fp, const PathState& ps, const FrameBufs& fb,
                     const NrcBufs& nb, const int* queue, const int* count, int* keep, int grid, cudaStream_t st) {
  nrc_shade_kernel<<<grid, 128, 0, st>>>(s, fp, ps, fb, nb, queue, count, keep);
  HM_CHECK_LAUNCH("nrc_shade_kernel");
  return HM_OK;
}

int launch_nrc_finalize(int P, const PathState& ps, const FrameBufs& fb, float4* col_out, cudaStream_t st) {
  nrc_finalize_kernel<<<(P + 255) / 256, 256, 0, st>>>(P, ps, fb, col_out);
  HM_CHECK_LAUNCH("nrc_finalize_kernel");
  return HM_OK;
}

int launch_nrc_compose(int P, int n_pix, const FrameParams& fp, const FrameBufs& fb, const NrcBufs& nb,
                       cudaStream_t st) {
  nrc_compose_kernel<<<(P + 255) / 256, 256, 0, st>>>(P, fp, fb, nb);
  HM_CHECK_LAUNCH("nrc_compose_kernel");
  nrc_train_data_kernel<<<(n_pix + 63) / 64, 64, 0, st>>>(P, n_pix, fp, fb, nb);
  HM_CHECK_LAUNCH("nrc_train_data_kernel");
  return HM_OK;
}

}  // namespace hm
