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
// reference's sceneIndices[trOfs], a shuffled index, hair_msnn.cu:222-233).
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
    ps.rng[pid] = rng_seed(fp.frame_seed, (uint32_t)pid);
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
  uint32_t rng = rng_seed(fp.frame_seed, (uint32_t)c.local);
  uint32_t flags = 0;
  if (fp.mode == MODE_MSNN) {
    const int tr = c.local / c.every_nth;
    if (tr < c.n_train) {
      const uint32_t pick = feistel_perm((uint32_t)tr, (uint32_t)c.n_train, (uint32_t)fp.accum_id) % c.every_nth;
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
  queue[pid] = pid;
}

HM_D void write_cache_input(float* dst, int in_ch, f3 p, f3 wo, f3 t) {
  dst[0] = p.x; dst[1] = p.y; dst[2] = p.z;
  dst[3] = wo.x; dst[4] = wo.y; dst[5] = wo.z;
  dst[6] = t.x; dst[7] = t.y; dst[8] = t.z;
  for (int c = 9; c < in_ch; ++c) dst[c] = 0.f;
}

// Shades every path of `queue`; keep[i] = 1 if path queue[i] continues.
template <bool MULTI>
__global__ void __launch_bounds__(128) shade_kernel(const __grid_constant__ SceneDev s0, FrameParams fp, Batch b,
                                                    PathState ps, FrameBufs fb, const int* __restrict__ queue,
                                                    const int* __restrict__ count, int* __restrict__ keep) {
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
    const float4 h = ps.hit[pid];
    const bool hit = __float_as_int(h.y) >= 0;
    const bool train = flags & F_TRAIN;
    const f3 ro = ld3(ps.ray_o, pid), rd = ld3(ps.ray_d, pid);
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
    const Vertex v = setup_vertex(s, ro, rd, h);
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
    // ---- direct lighting at this vertex
    const bool do_dl = fp.mode == MODE_MSNN || (k == 0 ? v1_stop == 0 : k >= v1_stop);
    if (do_dl) {
      ShadowSample ss[2];
      direct_lighting(s, v, rng, ss);
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
      } else if (fp.mode == MODE_MSNN) {
        const float eps = lcg_next(rng);
        if (eps < q || k > c.beta) done = true;
        else beta = beta / (1.f - q);
      } else {
        const float eps = lcg_next(rng);
        if (eps < q) done = true;
        else beta = beta / (1.f - q);
      }
    }
    // ---- next vertex
    if (!done && k + 1 <= v2_stop) {
      f3 o, d;
      const f3 mul = next_vertex(s, v, rng, &o, &d);
      beta = beta * mul;
      beta_s = beta_s * mul;
      st3(ps.ray_o, pid, o);
      st3(ps.ray_d, pid, d);
      ps.bounce[pid] = k + 1;
      k_keep = 1;
    }
    st3(ps.beta, pid, beta);
    st3(ps.beta_s, pid, beta_s);
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
                 const int* queue, const int* count, int* keep, int grid, cudaStream_t st) {
  if (b.scenes)
    shade_kernel<true><<<grid, 128, 0, st>>>(s, fp, b, ps, fb, queue, count, keep);
  else
    shade_kernel<false><<<grid, 128, 0, st>>>(s, fp, b, ps, fb, queue, count, keep);
  HM_CHECK_LAUNCH("shade_kernel");
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
