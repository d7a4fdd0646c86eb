// Wavefront shading kernels (compiled with -fmad=false: every
// non-transcendental operation is rounded like the reference's formulas).
//
//   camera_kernel    rayGenCam's camera ray and path set-up (hair_msnn.cu:187-221,
//                    path_tracing.cu:19-45)
//   shade_kernel     one path vertex: closest-hit set-up, directLighting's two
//                    samples (shadow rays resolved later), Russian roulette /
//                    BETA cut, next-vertex sample (msnnPathTrace hair_msnn.cu:135-185,
//                    msnnTrainingPath :68-132, pathTrace optix_common.cuh:363-409)
//   finalize_kernel  G-buffer, cache inputs and training targets with the
//                    reference's NaN/Inf scrubbing (hair_msnn.cu:242-312)
//   compose_kernel   RENDER pass: short path + cache on hair pixels, FP64
//                    accumulation (hair_msnn.cu:314-356; utils.cuh:13-35 for PT)
#include "hm_hair_grad.cuh"
#include "hm_render.h"
#include "hm_shading.cuh"

namespace hm {

HM_D f3 ld3(const float4* p, int i) {
  float4 v = p[i];
  return mk(v.x, v.y, v.z);
}
HM_D void st3(float4* p, int i, f3 v, float w = 0.f) { p[i] = make_float4(v.x, v.y, v.z, w); }

// Camera rays of one frame, or (fp.pretrain) the rays of the scene-sample
// training pass: record r aims from the camera at sample perm(r) (the
// reference's sceneIndices[trOfs], a shuffled index, hair_msnn.cu:222-233)
// with the RNG of its launch index (r % 128, r / 128) over the frame's
// width (get_rng with the frame buffer's size, hair_msnn.cu:193-194).
template <bool MULTI>
__global__ void __launch_bounds__(256) camera_kernel(const __grid_constant__ SceneDev s0, FrameParams fp, Batch b,
                                                     PathState ps, int* queue, int* count) {
  const int P = fp.pretrain ? fp.n_train : (MULTI ? b.n_paths : s0.width * s0.height);
  const int pid = blockIdx.x * blockDim.x + threadIdx.x;
  if (pid == 0) *count = P;
  if (pid >= P) return;
  if (fp.pretrain) {
    const uint32_t si = feistel_perm((uint32_t)pid, (uint32_t)fp.n_samples, fp.sample_key);
    const float4 sp = fp.samples[si];
    const uint32_t lx = (uint32_t)pid % kTrainRecordsX, ly = (uint32_t)pid / kTrainRecordsX;
    ps.rng[pid] = rng_seed(fp.frame_seed, lx + ly * (uint32_t)s0.width);
    ps.flags[pid] = F_TRAIN;
    ps.bounce[pid] = 0;
    st3(ps.ray_o, pid, s0.cam_pos);
    st3(ps.ray_d, pid, normalize(mk(sp.x, sp.y, sp.z) - s0.cam_pos));
    st3(ps.beta, pid, splat(1.f));
    st3(ps.beta_s, pid, splat(1.f));
    st3(ps.col, pid, splat(0.f));
    st3(ps.col_s, pid, splat(0.f));
    queue[pid] = pid;
    return;
  }
  const PathCtx c = path_ctx<MULTI>(s0, fp, b, pid);
  const SceneDev& s = *c.s;
  const int x = c.local % s.width, y = c.local / s.width;
  const int accum_id = fp.d_frame ? *fp.d_frame : fp.accum_id;
  uint32_t rng = rng_seed(fp.d_frame ? accum_id + 10007 : fp.frame_seed, (uint32_t)c.local);
  uint32_t flags = 0;
  if (fp.mode == MODE_MSNN && !fp.no_train) {
    const int tr = c.local / c.every_nth;
    if (tr < c.n_train) {
      const uint32_t pick = feistel_perm((uint32_t)tr, (uint32_t)c.n_train, (uint32_t)accum_id) % c.every_nth;
      if ((uint32_t)(c.local % c.every_nth) == pick) flags |= F_TRAIN;
    }
  }
  const float ox = lcg_next(rng), oy = lcg_next(rng);
  const float su = ((float)x + ox) / (float)s.width, sv = ((float)y + oy) / (float)s.height;
  const f3 dir = normalize(s.cam_d00 + su * s.cam_du + sv * s.cam_dv);
  ps.rng[pid] = rng;
  ps.flags[pid] = flags;
  ps.bounce[pid] = 0;
  st3(ps.ray_o, pid, s.cam_pos);
  st3(ps.ray_d, pid, dir);
  st3(ps.beta, pid, splat(1.f));
  st3(ps.beta_s, pid, splat(1.f));
  st3(ps.col, pid, splat(0.f));
  st3(ps.col_s, pid, splat(0.f));
  if (fp.eval_hc) st3(ps.beta_d, pid, splat(1.f));
  queue[pid] = pid;
}

HM_D void write_cache_input(float* dst, int in_ch, f3 p, f3 wo, f3 t) {
  dst[0] = p.x; dst[1] = p.y; dst[2] = p.z;
  dst[3] = wo.x; dst[4] = wo.y; dst[5] = wo.z;
  dst[6] = t.x; dst[7] = t.y; dst[8] = t.z;
  for (int c = 9; c < in_ch; ++c) dst[c] = 0.f;
}

HM_D float comp(f3 v, int c) { return c == 0 ? v.x : (c == 1 ? v.y : v.z); }

// Path-replay terms of one hair vertex (material derivatives, adjoint A,
// throughput bw at the vertex, R = the path's total radiance minus what it
// gathered before the vertex).
//  * Its own direct lighting: a sample's contribution c = f * (emitted
//    radiance, MIS weight, 1 / pdf), with f the BSDF value at the sample's
//    direction; the weight and the pdf are held fixed (detached sampling),
//    so d c = c * (d f) / f.  E[k] gets A . (bw * d c_k), counted only if
//    the shadow ray finds the light.
//  * The continuation: the throughput factor f / pdf of the sampled
//    direction scales all the radiance gathered after the vertex, R minus
//    this vertex's own direct lighting, so T gets A . ((d f) / f * R) and
//    E[k] loses A . ((d f) / f * bw * c_k), the part of R that is the
//    sample's (if visible).
// Non-finite terms (a NaN path, f = 0) are left out.
HM_D void replay_vertex(const HairConstsD& hcd, const Vertex& v, f3 A, f3 bw, f3 R, const ShadowSample ss[2],
                        bool dl, bool cont, f3 wl_next, float E[2][kNd], float T[kNd]) {
  const float h = dot(v.fr.r1, v.n);
#pragma unroll
  for (int i = 0; i < kNd; ++i) {
    E[0][i] = 0.f;
    E[1][i] = 0.f;
    T[i] = 0.f;
  }
  for (int k = 0; k < 2; ++k) {
    if (!dl || !ss[k].valid) continue;
    const HairEvalD e = hair_eval_dual(v.wo_local, ss[k].wl, h, hcd);
    for (int c = 0; c < 3; ++c) {
      const float f = e.f[c].v;
      const float w = comp(A, c) * comp(bw, c) * comp(ss[k].c, c) / f;
      if (f == 0.f || !isfinite(w)) continue;
#pragma unroll
      for (int i = 0; i < kNd; ++i) E[k][i] += w * e.f[c].d[i];
    }
  }
  if (!cont) return;
  const HairEvalD e = hair_eval_dual(v.wo_local, wl_next, h, hcd);
  for (int c = 0; c < 3; ++c) {
    const float f = e.f[c].v;
    if (f == 0.f) continue;
    const float a = comp(A, c) / f;
    const float t = a * comp(R, c);
    const float u0 = dl && ss[0].valid ? a * comp(bw, c) * comp(ss[0].c, c) : 0.f;
    const float u1 = dl && ss[1].valid ? a * comp(bw, c) * comp(ss[1].c, c) : 0.f;
    if (!isfinite(t) || !isfinite(u0) || !isfinite(u1)) continue;
#pragma unroll
    for (int i = 0; i < kNd; ++i) {
      const float d = e.f[c].d[i];
      T[i] += t * d;
      E[0][i] -= u0 * d;
      E[1][i] -= u1 * d;
    }
  }
}

// Shades every path of `queue`; keep[i] = 1 if path queue[i] continues.
// REPLAY: the same shading (same random numbers, same results) plus the
// path-replay terms of each hair vertex (single-scene frames).
template <bool MULTI, bool REPLAY>
__global__ void __launch_bounds__(128) shade_kernel(const __grid_constant__ SceneDev s0, FrameParams fp, Batch b,
                                                    PathState ps, FrameBufs fb, const int* __restrict__ queue,
                                                    const int* __restrict__ count, int* __restrict__ keep,
                                                    DiffParams dp) {
  const int n = *count;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int pid = queue[i];
    const PathCtx c = path_ctx<MULTI>(s0, fp, b, pid);
    const SceneDev& s = *c.s;
    const int v2_stop = s.path_v2 - 1;  // hair_msnn.cu:201 / path_tracing.cu:54
    const int v1_stop = s.path_v1 - 1;
    const int rec = c.train_base + c.local / c.every_nth;  // training record of a training path
    uint32_t flags = ps.flags[pid];
    const int k = ps.bounce[pid];
    const float4 h_trav = ps.hit[pid];
    const bool hit = __float_as_int(h_trav.y) >= 0;
    const bool train = flags & F_TRAIN;
    const f3 ro = ld3(ps.ray_o, pid), rd = ld3(ps.ray_d, pid);
    const float4 h = hit ? refit_hit(s, ro, rd, h_trav) : h_trav;
    if (fp.log.ev)
      log_ray(fp.log, pid, 3 * k, 0, hit ? __float_as_int(h.y) : -1, hit ? h.x : 0.f, hit ? h.z : 0.f, ps.rng[pid],
              ro, rd);
    int k_keep = 0;
    if (k == 0 && !hit) {
      // miss program (optix_common.cuh:604-616): Le of the camera ray
      st3(ps.col, pid, env_radiance(s, rd));
      if (fp.mode == MODE_MSNN) {
        write_cache_input(fb.nn_frame_in + (size_t)pid * fp.in_ch, fp.in_ch, splat(0.f), -1.f * rd, splat(0.f));
        if (train)
          write_cache_input(fb.nn_train_in + (size_t)rec * fp.in_ch, fp.in_ch, splat(0.f), -1.f * rd, splat(0.f));
      }
      ps.flags[pid] = flags;
      keep[i] = 0;
      continue;
    }
    if (!hit) {  // escaped after a bounce: the path ends with no contribution
      keep[i] = 0;
      continue;
    }
    Vertex v = setup_vertex(s, ro, rd, h);
    if (fp.eval_hc && !v.surface) v.hc_eval = fp.eval_hc + v.group;
    if (k == 0) {
      flags |= F_PRIM_HIT | (v.surface ? F_PRIM_SURF : 0u);
      if (fp.mode == MODE_MSNN) {
        const f3 pn = v.p / s.scene_scale;
        write_cache_input(fb.nn_frame_in + (size_t)pid * fp.in_ch, fp.in_ch, pn, v.wo, v.t);
        if (train)
          write_cache_input(fb.nn_train_in + (size_t)rec * fp.in_ch, fp.in_ch, pn, v.wo, v.t);
      }
    }
    uint32_t rng = ps.rng[pid];
    f3 beta = ld3(ps.beta, pid);
    f3 beta_s = ld3(ps.beta_s, pid);
    // detached renders: Russian roulette on the sampling material's throughput
    const bool detached = fp.eval_hc != nullptr;
    f3 beta_d = detached ? ld3(ps.beta_d, pid) : beta;
    const f3 beta_v = beta;  // throughput at the vertex
    // ---- direct lighting at this vertex
    const bool do_dl = fp.mode == MODE_MSNN || (k == 0 ? v1_stop == 0 : k >= v1_stop);
    ShadowSample ss[2];
    ss[0].valid = ss[1].valid = 0;
    if (do_dl) {
      direct_lighting(s, v, rng, ss);
      if (fp.log.ev) {
        fp.log.vcur[pid] = k;
        for (int j = 0; j < 2; ++j)
          if (ss[j].valid) log_ray(fp.log, pid, 3 * k + 1 + j, 1 + j, kLogPending, 0.f, 0.f, 0u, ss[j].o, ss[j].d);
      }
      st3(ps.sh_o0, pid, ss[0].o, ss[0].valid ? 1.f : 0.f);
      st3(ps.sh_d0, pid, ss[0].d);
      st3(ps.sh_c0, pid, ss[0].c);
      st3(ps.sh_o1, pid, ss[1].o, ss[1].valid ? 1.f : 0.f);
      st3(ps.sh_d1, pid, ss[1].d);
      st3(ps.sh_c1, pid, ss[1].c);
      st3(ps.dl_w, pid, beta);
      st3(ps.dl_ws, pid, 1.f * beta_s);
      flags |= F_DL;
    }
    // ---- Russian roulette (from the first bounce on)
    bool done = false;
    if (k >= 1) {
      const float q = fmaxf(0.05f, 1.f - luminance(beta));
      if (fp.mode == MODE_MSNN && train) {
        const float qs = fmaxf(0.05f, 1.f - luminance(beta_s));
        const float eps = lcg_next(rng);
        if (eps < qs || k > c.beta) beta_s = splat(0.f);
        if (eps < q) {
          done = true;
        } else {
          beta = beta / (1.f - q);
          if (beta_s.x != 0.f || beta_s.y != 0.f || beta_s.z != 0.f) beta_s = beta_s / (1.f - qs);
        }
      } else {
        const float qd = detached ? fmaxf(0.05f, 1.f - luminance(beta_d)) : q;
        const float eps = lcg_next(rng);
        if (eps < qd || (fp.mode == MODE_MSNN && k > c.beta)) {
          done = true;
        } else {
          beta = beta / (1.f - qd);
          if (detached) beta_d = beta_d / (1.f - qd);
        }
      }
    }
    // ---- next vertex
    bool cont = false;
    f3 wl_next = splat(0.f);
    if (!done && k + 1 <= v2_stop) {
      f3 o, d, mul_s;
      bool mul_nan = false;
      const f3 mul = next_vertex(s, v, rng, &o, &d, &mul_s, &wl_next, &mul_nan);
      beta = beta * mul;
      beta_s = beta_s * mul;
      if (detached) beta_d = beta_d * mul_s;
      st3(ps.ray_o, pid, o);
      st3(ps.ray_d, pid, d);
      ps.bounce[pid] = k + 1;
      k_keep = 1;
      cont = !mul_nan;
    }
    if constexpr (REPLAY) {
      float E[2][kNd], T[kNd];
      if (!v.surface) {
        const float* ad = dp.adjoint + 3 * (size_t)c.local;
        const f3 A = dp.adj_scale * mk(ad[0], ad[1], ad[2]);
        const f3 R = ld3(dp.col_total, pid) - ld3(ps.col, pid);
        replay_vertex(dp.group_dual[v.group], v, A, beta_v, R, ss, do_dl, cont, wl_next, E, T);
        float* g = dp.gacc + (size_t)v.group * kNd * dp.P + pid;
#pragma unroll
        for (int i = 0; i < kNd; ++i) g[(size_t)i * dp.P] += T[i];
      } else {
#pragma unroll
        for (int i = 0; i < kNd; ++i) E[0][i] = E[1][i] = 0.f;
      }
      if (do_dl) {
#pragma unroll
        for (int i = 0; i < kNd; ++i) {
          dp.stash[(size_t)i * dp.P + pid] = E[0][i];
          dp.stash[(size_t)(kNd + i) * dp.P + pid] = E[1][i];
        }
        dp.stash[(size_t)(2 * kNd) * dp.P + pid] = __int_as_float(v.group);
      }
    }
    st3(ps.beta, pid, beta);
    st3(ps.beta_s, pid, beta_s);
    if (detached) st3(ps.beta_d, pid, beta_d);
    ps.rng[pid] = rng;
    ps.flags[pid] = flags;
    keep[i] = k_keep;
  }
}

HM_D bool anynan(f3 c) { return isnan(c.x) || isnan(c.y) || isnan(c.z); }
HM_D bool anyinf(f3 c) { return isinf(c.x) || isinf(c.y) || isinf(c.z); }

template <bool MULTI>
__global__ void __launch_bounds__(256) finalize_kernel(const __grid_constant__ SceneDev s0, FrameParams fp, Batch b,
                                                       PathState ps, FrameBufs fb) {
  const int P = fp.pretrain ? fp.n_train : (MULTI ? b.n_paths : s0.width * s0.height);
  const int pid = blockIdx.x * blockDim.x + threadIdx.x;
  if (pid >= P) return;
  const uint32_t flags = ps.flags[pid];
  const bool hit = flags & F_PRIM_HIT;
  f3 color = ld3(ps.col, pid);
  if (fb.col_out) fb.col_out[pid] = ps.col[pid];  // differentiable renders: the path's radiance
  if (fp.mode == MODE_PT) {
    // writePixel (utils.cuh:13-35), FP64 accumulation
    if (anynan(color)) color = splat(0.f);
    double* a = fb.acc_final + 3 * (size_t)pid;
    if (fp.accum_id == 0) {
      a[0] = color.x; a[1] = color.y; a[2] = color.z;
    } else {
      a[0] += color.x; a[1] += color.y; a[2] += color.z;
    }
    return;
  }
  if (flags & F_TRAIN) {
    f3 c = hit ? color : splat(0.f);
    f3 sc = hit ? ld3(ps.col_s, pid) : splat(0.f);
    if (anynan(c)) c = splat(0.f);
    if (anyinf(c)) c = splat(1e5f);
    if (anynan(sc)) sc = splat(0.01f);
    if (anyinf(sc)) sc = splat(1e5f);
    const PathCtx pc = path_ctx<MULTI>(s0, fp, b, pid);
    float* t = fb.nn_train_out + (size_t)(pc.train_base + pc.local / pc.every_nth) * 3;
    t[0] = c.x - sc.x;
    t[1] = c.y - sc.y;
    t[2] = c.z - sc.z;
    color = hit ? c : color;  // a miss keeps Le
  }
  if (fp.pretrain) return;  // training records only
  const float w = (hit ? 1.f : 0.f) + ((flags & F_PRIM_SURF) ? 2.f : 0.f);
  fb.gbuf[pid] = make_float4(color.x, color.y, color.z, w);
}

__global__ void __launch_bounds__(256) compose_kernel(int P, FrameParams fp, FrameBufs fb) {
  const int pid = blockIdx.x * blockDim.x + threadIdx.x;
  if (pid >= P) return;
  const float4 g = fb.gbuf[pid];
  const int gf = (int)g.w;
  const f3 sc = mk(g.x, g.y, g.z);
  f3 nn = mk(fb.nn_frame_out[3 * pid], fb.nn_frame_out[3 * pid + 1], fb.nn_frame_out[3 * pid + 2]);
  f3 color;
  if (!(gf & 1) || (gf & 2)) {
    color = sc;
    nn = color;
  } else {
    color = sc + nn;
  }
  double* apt = fb.acc_pt + 3 * (size_t)pid;
  double* ann = fb.acc_nn + 3 * (size_t)pid;
  double* afi = fb.acc_final + 3 * (size_t)pid;
  if (fp.accum_id == 0) {
    apt[0] = sc.x; apt[1] = sc.y; apt[2] = sc.z;
    ann[0] = nn.x; ann[1] = nn.y; ann[2] = nn.z;
    afi[0] = color.x; afi[1] = color.y; afi[2] = color.z;
  } else {
    apt[0] += sc.x; apt[1] += sc.y; apt[2] += sc.z;
    ann[0] += nn.x; ann[1] += nn.y; ann[2] += nn.z;
    afi[0] += color.x; afi[1] += color.y; afi[2] += color.z;
  }
}

int launch_camera(const SceneDev& s, const FrameParams& fp, const Batch& b, const PathState& ps, int* queue,
                  int* count, cudaStream_t st) {
  const int P = fp.pretrain ? fp.n_train : (b.scenes ? b.n_paths : s.width * s.height);
  if (b.scenes)
    camera_kernel<true><<<(P + 255) / 256, 256, 0, st>>>(s, fp, b, ps, queue, count);
  else
    camera_kernel<false><<<(P + 255) / 256, 256, 0, st>>>(s, fp, b, ps, queue, count);
  HM_CHECK_LAUNCH("camera_kernel");
  return HM_OK;
}

int launch_shade(const SceneDev& s, const FrameParams& fp, const Batch& b, const PathState& ps, const FrameBufs& fb,
                 const int* queue, const int* count, int* keep, int grid, cudaStream_t st, const DiffParams* dp) {
  if (dp) {
    if (b.scenes) return hm_set_error("path replay: single-scene renders only"), HM_EINVAL;
    shade_kernel<false, true><<<grid, 128, 0, st>>>(s, fp, b, ps, fb, queue, count, keep, *dp);
  } else if (b.scenes) {
    shade_kernel<true, false><<<grid, 128, 0, st>>>(s, fp, b, ps, fb, queue, count, keep, DiffParams{});
  } else {
    shade_kernel<false, false><<<grid, 128, 0, st>>>(s, fp, b, ps, fb, queue, count, keep, DiffParams{});
  }
  HM_CHECK_LAUNCH("shade_kernel");
  return HM_OK;
}

// Materials with their partials, one per strand group (the scene's own
// material when it has no groups).
__global__ void group_dual_kernel(const __grid_constant__ SceneDev s, HairConstsD* out, int n) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  const hm_hair_params& m = s.n_groups ? s.group_raw[g] : s.hair_raw;
  const float gain[4] = {m.gain_r, m.gain_tt, m.gain_trt, m.gain_trrt};
  out[g] = hair_consts_dual(m.sigma_a, m.beta_m, m.beta_n, m.alpha, gain);
}

int launch_group_dual(const SceneDev& s, void* out, int n, cudaStream_t st) {
  group_dual_kernel<<<1, 64, 0, st>>>(s, (HairConstsD*)out, n);
  HM_CHECK_LAUNCH("group_dual_kernel");
  return HM_OK;
}
size_t group_dual_bytes() { return sizeof(HairConstsD); }

// dL/d(cache output) of a replayed frame: the adjoint of the pixels whose
// image took the cache (hair at the primary hit), 0 elsewhere.
__global__ void __launch_bounds__(256) replay_cache_grad_kernel(int P, PathState ps, DiffParams dp, float* dy) {
  const int pid = blockIdx.x * blockDim.x + threadIdx.x;
  if (pid >= P) return;
  const uint32_t flags = ps.flags[pid];
  const bool nn = (flags & F_PRIM_HIT) && !(flags & F_PRIM_SURF);
  for (int c = 0; c < 3; ++c) dy[3 * (size_t)pid + c] = nn ? dp.adj_scale * dp.adjoint[3 * (size_t)pid + c] : 0.f;
}

int launch_replay_cache_grad(int P, const PathState& ps, const DiffParams& dp, float* dy, cudaStream_t st) {
  replay_cache_grad_kernel<<<(P + 255) / 256, 256, 0, st>>>(P, ps, dp, dy);
  HM_CHECK_LAUNCH("replay_cache_grad_kernel");
  return HM_OK;
}

int launch_finalize(const SceneDev& s, const FrameParams& fp, const Batch& b, const PathState& ps,
                    const FrameBufs& fb, cudaStream_t st) {
  const int P = fp.pretrain ? fp.n_train : (b.scenes ? b.n_paths : s.width * s.height);
  if (b.scenes)
    finalize_kernel<true><<<(P + 255) / 256, 256, 0, st>>>(s, fp, b, ps, fb);
  else
    finalize_kernel<false><<<(P + 255) / 256, 256, 0, st>>>(s, fp, b, ps, fb);
  HM_CHECK_LAUNCH("finalize_kernel");
  return HM_OK;
}

int launch_compose(int P, const FrameParams& fp, const FrameBufs& fb, cudaStream_t st) {
  compose_kernel<<<(P + 255) / 256, 256, 0, st>>>(P, fp, fb);
  HM_CHECK_LAUNCH("compose_kernel");
  return HM_OK;
}

}  // namespace hm
