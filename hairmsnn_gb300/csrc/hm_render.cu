// Wavefront frame driver and trace kernels.
//
// Per frame (one sample per pixel, as the reference's render loop,
// render_hair_msnn.cu:699-771):
//   camera -> [extend -> shade -> shadow -> compact] x bounces -> finalize
//   MSNN: -> cache training step on the frame's records -> cache inference on
//   every pixel -> compose (FP64 accumulation)
// Queues are compacted with a deterministic block scan, so the order of the
// surviving paths (and therefore every result) does not depend on timing.
#include <algorithm>
#include <string>
#include <vector>

#include "hm_hair_grad.cuh"
#include "hm_mlp.cuh"
#include "hm_render.h"
#include "hm_trace.cuh"

namespace hm {

int launch_camera(const SceneDev& s, const FrameParams& fp, const Batch& b, const PathState& ps, int* queue,
                  int* count, cudaStream_t st);
int launch_shade(const SceneDev& s, const FrameParams& fp, const Batch& b, const PathState& ps, const FrameBufs& fb,
                 const int* queue, const int* count, int* keep, int grid, cudaStream_t st,
                 const DiffParams* dp = nullptr);
int launch_group_dual(const SceneDev& s, void* out, int n, cudaStream_t st);
size_t group_dual_bytes();
int launch_replay_cache_grad(int P, const PathState& ps, const DiffParams& dp, float* dy, cudaStream_t st);
int launch_nrc_camera(const SceneDev& s, const FrameParams& fp, const PathState& ps, const FrameBufs& fb,
                      const NrcBufs& nb, int* queue, int* count, cudaStream_t st);
int launch_nrc_shade(const SceneDev& s, const FrameParams& fp, const PathState& ps, const FrameBufs& fb,
                     const NrcBufs& nb, const int* queue, const int* count, int* keep, int grid, cudaStream_t st);
int launch_nrc_finalize(int P, const PathState& ps, const FrameBufs& fb, float4* col_out, cudaStream_t st);
int launch_nrc_compose(int P, int n_pix, const FrameParams& fp, const FrameBufs& fb, const NrcBufs& nb,
                       cudaStream_t st);
int launch_finalize(const SceneDev& s, const FrameParams& fp, const Batch& b, const PathState& ps,
                    const FrameBufs& fb, cudaStream_t st);
int launch_compose(int P, const FrameParams& fp, const FrameBufs& fb, cudaStream_t st);

// ---- persistent traversal with warp-aggregated dynamic ray fetching
// Ray sources: extension rays (one per queued path), shadow rays (two slots
// per queued path, empty slots finish at once), and plain ray batches.
struct ExtendRays {
  PathState ps;
  const int* queue;
  const int* count;
  HM_D int n() const { return *count; }
  HM_D int path(int i) const { return queue[i]; }
  HM_D bool ray(int i, f3* o, f3* d) const {
    const int pid = queue[i];
    const float4 a = ps.ray_o[pid], b = ps.ray_d[pid];
    *o = mk(a.x, a.y, a.z);
    *d = mk(b.x, b.y, b.z);
    return true;
  }
  HM_D void write(int i, const Hit& h) const {
    ps.hit[queue[i]] = make_float4(h.t, __int_as_float(h.prim), h.u, h.v);
  }
};

struct ShadowRays {
  PathState ps;
  const int* queue;
  const int* count;
  uint8_t* vis;  // [P][2]: 1 = unoccluded
  // ray i < count: the light sample of queued path i; ray count + i: its
  // BSDF sample.  Light samples share few directions (the directional
  // lights, the bright part of the sky), so keeping the two kinds apart
  // keeps a warp's rays alike.
  HM_D int n() const { return 2 * *count; }
  HM_D int entry(int i, int* slot) const {
    const int c = *count;
    *slot = i >= c ? 1 : 0;
    return *slot ? i - c : i;
  }
  HM_D int path(int i) const {
    int slot;
    return queue[entry(i, &slot)];
  }
  HM_D bool ray(int i, f3* o, f3* d) const {
    int slot;
    const int pid = queue[entry(i, &slot)];
    if (!(ps.flags[pid] & F_DL)) return false;
    const float4 a = slot ? ps.sh_o1[pid] : ps.sh_o0[pid];
    if (a.w == 0.f) return false;
    const float4 b = slot ? ps.sh_d1[pid] : ps.sh_d0[pid];
    *o = mk(a.x, a.y, a.z);
    *d = mk(b.x, b.y, b.z);
    return true;
  }
  HM_D void write(int i, const Hit& h) const {
    int slot;
    const int pid = queue[entry(i, &slot)];
    vis[2 * pid + slot] = h.prim < 0 ? 1 : 0;
  }
};

struct BatchRays {
  const float* org;
  const float* dir;
  int64_t count;
  float tmin, tmax;
  float4* out;
  HM_D int n() const { return (int)count; }
  HM_D int path(int i) const { return i; }
  HM_D bool ray(int i, f3* o, f3* d) const {
    *o = mk(org[3 * i], org[3 * i + 1], org[3 * i + 2]);
    *d = mk(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]);
    return true;
  }
  HM_D void write(int i, const Hit& h) const { out[i] = make_float4(h.t, __int_as_float(h.prim), h.u, h.v); }
};

constexpr int kStragglersAnyHit = 12;   // lanes a warp does not wait for before its leaf phase: shadow rays
constexpr int kStragglersClosest = 12;  // ... extension rays
constexpr int kParkAnyHit = 2;        // leaves a lane parks before the leaf phase: shadow rays
constexpr int kParkClosest = 2;       // ... extension rays
constexpr bool kAnyHitNearest = false;  // shadow rays walk the first inner child hit next (true: the nearest)
constexpr int kMaxRounds = 1 << 22;   // per-warp round cap (~6k rounds per warp at 512x512)

// COUNT: accumulate BVH nodes visited / primitives tested (and rays) into
// cnt[0..2] (an untimed instrumentation pass; timed frames use COUNT = false).
// MULTI: the rays belong to the scenes of a batch (b.path_scene of the ray's
// path selects the tree each lane walks).
template <class Src, bool ANY_HIT, bool COUNT, bool MULTI>
__global__ void __launch_bounds__(128) persistent_trace_kernel(Src src, const __grid_constant__ SceneDev s0,
                                                               Batch b, float tmin, float tmax,
                                                               int* __restrict__ fetch, int* err,
                                                               unsigned long long* cnt) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int n = src.n();
  if (n <= 0) return;  // an empty bounce: no ray-fetch atomics at all
  int2 stack[kStack];
  TravState t;
  const SceneDev* sp = &s0;
  TraceCount tc{0, 0};
  uint32_t rays = 0;
  int cur = -1;
  bool exhausted = false;
  int rounds = 0;
  for (;;) {
    // refill idle lanes; a lane whose entry holds no ray (a shadow slot
    // left empty) fetches again at once instead of idling for a round
    unsigned idle = __ballot_sync(FULL, cur < 0);
    while (idle && !exhausted) {
      const int leader = __ffs(idle) - 1;
      const int want = __popc(idle);
      int base = 0;
      if (lane == leader) base = atomicAdd(fetch, want);
      base = __shfl_sync(FULL, base, leader);
      exhausted = base + want >= n;
      if (cur < 0) {
        const int my = base + __popc(idle & ((1u << lane) - 1u));
        if (my < n) {
          f3 o, d;
          if (src.ray(my, &o, &d)) {
            if (MULTI) sp = &b.scenes[b.path_scene[src.path(my)]].s;
            trav_init(t, o, d, tmin, tmax);
            cur = my;
            if (COUNT) ++rays;
          } else {
            src.write(my, Hit{tmax, -1, 0.f, 0.f});
          }
        }
      }
      idle = __ballot_sync(FULL, cur < 0);
    }
    if (exhausted && __all_sync(FULL, cur < 0)) break;
    if (++rounds > kMaxRounds) {  // safety net: never spin on a logic error
      if (lane == 0) atomicOr(err, TRACE_ERR_STEPS);
      break;
    }
    // box phase: walk inner nodes until every lane has parked two leaves or
    // finished; once some lane has a leaf parked, up to kStragglers* lanes
    // that still need steps are not waited for (they continue next round).
    // Every iteration advances at least one lane, so the phase terminates.
    for (int guard = 0; guard < kMaxVisits; ++guard) {
      const bool need = cur >= 0 && trav_needs_step<(ANY_HIT ? kParkAnyHit : kParkClosest)>(t);
      const unsigned needm = __ballot_sync(FULL, need);
      if (needm == 0) break;
      const unsigned parked = __ballot_sync(FULL, cur >= 0 && t.np > 0);
      if (parked != 0 && __popc(needm) <= (ANY_HIT ? kStragglersAnyHit : kStragglersClosest)) break;
      if (need) {
        if (ANY_HIT)
          trav_inner_step_any<COUNT, kParkAnyHit, kAnyHitNearest>(*sp, t, stack, err, &tc);
        else
          trav_inner_step<COUNT>(*sp, t, stack, err, &tc);
      }
    }
    // leaf phase: the parked curve / triangle tests run together
    if (cur >= 0) {
      const bool done = trav_leaf<ANY_HIT, COUNT>(*sp, t, &tc);
      if (done || trav_finished(t)) {
        src.write(cur, t.h);
        cur = -1;
      }
    }
  }
  if (COUNT) {
    atomicAdd(cnt + 0, (unsigned long long)tc.nodes);
    atomicAdd(cnt + 1, (unsigned long long)tc.prims);
    atomicAdd(cnt + 2, (unsigned long long)rays);
  }
}

template <class Src, bool ANY_HIT>
static int launch_persistent(const Src& src, const SceneDev& s, const Batch& b, float tmin, float tmax, int* fetch,
                             int* err, unsigned long long* cnt, bool counting, int max_blocks, cudaStream_t st) {
  // the traversal reads nodes with 32-byte loads (batch scenes: checked when the batch is built)
  if (((uintptr_t)s.wnodes & 31) != 0) return hm_set_error("traversal: wide nodes not 32-byte aligned"), HM_EINVAL;
  if (b.scenes) {
    if (counting)
      persistent_trace_kernel<Src, ANY_HIT, true, true><<<max_blocks, 128, 0, st>>>(src, s, b, tmin, tmax, fetch,
                                                                                    err, cnt);
    else
      persistent_trace_kernel<Src, ANY_HIT, false, true><<<max_blocks, 128, 0, st>>>(src, s, b, tmin, tmax, fetch,
                                                                                     err, cnt);
  } else {
    if (counting)
      persistent_trace_kernel<Src, ANY_HIT, true, false><<<max_blocks, 128, 0, st>>>(src, s, b, tmin, tmax, fetch,
                                                                                     err, cnt);
    else
      persistent_trace_kernel<Src, ANY_HIT, false, false><<<max_blocks, 128, 0, st>>>(src, s, b, tmin, tmax, fetch,
                                                                                      err, cnt);
  }
  HM_CHECK_LAUNCH("persistent_trace_kernel");
  return HM_OK;
}

template <class Src, bool ANY_HIT>
static int persistent_blocks() {
  int dev = 0, sms = 152, per_sm = 4;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, persistent_trace_kernel<Src, ANY_HIT, false, false>, 128,
                                                0);
  return sms * std::max(1, per_sm);
}

// Resolves the pending direct-lighting samples of each queued path: visible
// sum, NaN check (directLighting, optix_common.cuh:296-308), weighted add to
// the path radiance.  Explicitly rounded operations: no contraction.
// REPLAY: the stashed gradient terms of the visible samples join the path's
// gradient sums (none when the sum was a NaN and was dropped).
// rec_idx / rec (NRC frames, else NULL): the visible sum is also the
// vertex's direct light in the training pixel's train buffer.
template <bool REPLAY>
__global__ void __launch_bounds__(256) shadow_resolve_kernel(PathState ps, const int* __restrict__ queue,
                                                             const int* __restrict__ count,
                                                             const uint8_t* __restrict__ vis, DiffParams dp,
                                                             const int* __restrict__ rec_idx = nullptr,
                                                             float4* __restrict__ rec = nullptr,
                                                             PathLog log = PathLog{}) {
  const int n = *count;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int pid = queue[i];
    const uint32_t flags = ps.flags[pid];
    if (!(flags & F_DL)) continue;
    if (log.ev) {  // the shadow rays' results into the path's ray log
      const int k = log.vcur[pid];
      for (int j = 0; j < 2; ++j) {
        const int slot = 3 * k + 1 + j;
        if ((j ? ps.sh_o1[pid].w : ps.sh_o0[pid].w) != 0.f && slot < log.slots)
          log.ev[((size_t)pid * log.slots + slot) * 3].x = __int_as_float(vis[2 * pid + j] ? 1 : 0);
      }
    }
    float c0x = 0.f, c0y = 0.f, c0z = 0.f, c1x = 0.f, c1y = 0.f, c1z = 0.f;
    bool use0 = false, use1 = false;
    if (ps.sh_o0[pid].w != 0.f && vis[2 * pid]) {
      const float4 c = ps.sh_c0[pid];
      c0x = c.x; c0y = c.y; c0z = c.z;
      use0 = true;
    }
    if (ps.sh_o1[pid].w != 0.f && vis[2 * pid + 1]) {
      const float4 c = ps.sh_c1[pid];
      c1x = c.x; c1y = c.y; c1z = c.z;
      use1 = true;
    }
    float sx = __fadd_rn(0.f, __fadd_rn(c0x, c1x));
    float sy = __fadd_rn(0.f, __fadd_rn(c0y, c1y));
    float sz = __fadd_rn(0.f, __fadd_rn(c0z, c1z));
    if (isnan(sx) || isnan(sy) || isnan(sz)) {
      sx = sy = sz = 0.f;
      use0 = use1 = false;
    }
    if (rec_idx) {
      const int ri = rec_idx[pid];
      if (ri >= 0) rec[(size_t)ri * kNrcRecordF4 + 3] = make_float4(sx, sy, sz, 0.f);
    }
    if constexpr (REPLAY) {
      if (use0 || use1) {
        const size_t P = (size_t)dp.P;
        const int g = __float_as_int(dp.stash[2 * kNd * P + pid]);
        float* acc = dp.gacc + (size_t)g * kNd * P + pid;
#pragma unroll
        for (int k = 0; k < kNd; ++k) {
          const float a = (use0 ? dp.stash[k * P + pid] : 0.f) + (use1 ? dp.stash[(kNd + k) * P + pid] : 0.f);
          acc[k * P] += a;
        }
      }
    }
    const float4 w = ps.dl_w[pid];
    float4 c = ps.col[pid];
    c.x = __fadd_rn(c.x, __fmul_rn(w.x, sx));
    c.y = __fadd_rn(c.y, __fmul_rn(w.y, sy));
    c.z = __fadd_rn(c.z, __fmul_rn(w.z, sz));
    ps.col[pid] = c;
    if ((flags & F_TRAIN) && !rec_idx) {
      const float4 ws = ps.dl_ws[pid];
      float4 cs = ps.col_s[pid];
      cs.x = __fadd_rn(cs.x, __fmul_rn(ws.x, sx));
      cs.y = __fadd_rn(cs.y, __fmul_rn(ws.y, sy));
      cs.z = __fadd_rn(cs.z, __fmul_rn(ws.z, sz));
      ps.col_s[pid] = cs;
    }
    ps.flags[pid] = flags & ~F_DL;
  }
}

// ---- path-replay gradient sums (fixed order: results do not depend on timing)
// Block b sums paths [b * per, (b + 1) * per) of every row in FP64.
__global__ void __launch_bounds__(256) grad_block_sum_kernel(const float* __restrict__ gacc, int P, int rows,
                                                             double* __restrict__ partial) {
  __shared__ double red[256];
  const int per = (P + gridDim.x - 1) / gridDim.x;
  const int lo = blockIdx.x * per, hi = min(P, lo + per);
  for (int row = 0; row < rows; ++row) {
    double a = 0.0;
    for (int i = lo + threadIdx.x; i < hi; i += 256) a += (double)gacc[(size_t)row * P + i];
    red[threadIdx.x] = a;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) partial[(size_t)blockIdx.x * rows + row] = red[0];
    __syncthreads();
  }
}
// out[row] = sum over n_parts parts (in order) of part[part][row]
__global__ void grad_parts_sum_kernel(const double* __restrict__ part, int n_parts, int rows,
                                      double* __restrict__ out) {
  for (int row = threadIdx.x; row < rows; row += blockDim.x) {
    double a = 0.0;
    for (int b = 0; b < n_parts; ++b) a += part[(size_t)b * rows + row];
    out[row] = a;
  }
}

// ---- deterministic compaction: keep[] over count entries -> next queue
constexpr int kScanBlock = 1024;

__global__ void __launch_bounds__(kScanBlock) scan_count_kernel(const int* __restrict__ keep, const int* __restrict__ count,
                                                                int* __restrict__ block_sums, int n_blocks_max) {
  const int n = *count;
  const int nb = min(n_blocks_max, (n + kScanBlock - 1) / kScanBlock);
  __shared__ int warp_sums[kScanBlock / 32];
  for (int b = blockIdx.x; b < nb; b += gridDim.x) {
    const int i = b * kScanBlock + threadIdx.x;
    const int v = (i < n) ? keep[i] : 0;
    const int ws = __popc(__ballot_sync(0xffffffffu, v != 0));
    if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = ws;
    __syncthreads();
    if (threadIdx.x == 0) {
      int s = 0;
      for (int w = 0; w < kScanBlock / 32; ++w) s += warp_sums[w];
      block_sums[b] = s;
    }
    __syncthreads();
  }
}

__global__ void scan_blocks_kernel(int* __restrict__ block_sums, const int* __restrict__ count, int* __restrict__ out_count) {
  // single block: exclusive scan of ceil(count / kScanBlock) block sums
  const int n = *count;
  const int nb = (n + kScanBlock - 1) / kScanBlock;
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += blockDim.x) {
    const int i = base + threadIdx.x;
    int v = i < nb ? block_sums[i] : 0;
    // inclusive warp scan
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if ((threadIdx.x & 31) >= o) x += y;
    }
    __shared__ int wsum[32];
    if ((threadIdx.x & 31) == 31) wsum[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
      int w = threadIdx.x < (int)(blockDim.x >> 5) ? wsum[threadIdx.x] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, w, o);
        if (threadIdx.x >= o) w += y;
      }
      wsum[threadIdx.x] = w;
    }
    __syncthreads();
    const int warp_off = (threadIdx.x >> 5) ? wsum[(threadIdx.x >> 5) - 1] : 0;
    const int incl = x + warp_off;
    if (i < nb) block_sums[i] = carry + incl - v;  // exclusive
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) *out_count = carry;
}

__global__ void __launch_bounds__(kScanBlock) scatter_kernel(const int* __restrict__ keep, const int* __restrict__ queue,
                                                             const int* __restrict__ count,
                                                             const int* __restrict__ block_offsets,
                                                             int* __restrict__ next, int n_blocks_max) {
  const int n = *count;
  const int nb = min(n_blocks_max, (n + kScanBlock - 1) / kScanBlock);
  __shared__ int warp_off[kScanBlock / 32];
  for (int b = blockIdx.x; b < nb; b += gridDim.x) {
    const int i = b * kScanBlock + threadIdx.x;
    const int v = (i < n) ? keep[i] : 0;
    const unsigned m = __ballot_sync(0xffffffffu, v != 0);
    const int lane = threadIdx.x & 31;
    if (lane == 0) warp_off[threadIdx.x >> 5] = __popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
      int s = 0;
      for (int w = 0; w < kScanBlock / 32; ++w) {
        int t = warp_off[w];
        warp_off[w] = s;
        s += t;
      }
    }
    __syncthreads();
    if (v) next[block_offsets[b] + warp_off[threadIdx.x >> 5] + __popc(m & ((1u << lane) - 1u))] = queue[i];
    __syncthreads();
  }
}

// ---- render object
// Frames are pipelined: up to `depth` frames are in flight on their own
// streams with their own path state.  Frame k+1's path tracing never reads the
// cache (the reference's G_BUFFER pass, hair_msnn.cu:206-312), so it overlaps
// with the latency-bound tail of frame k's long training paths; only the cache
// step (train -> infer) and the FP64 accumulation (compose) are chained across
// frames with events, in frame order, so results are bit-identical to running
// the frames one after another.  Bounce counts stay on the device: every
// bounce's kernels read the queue length from device memory and do nothing
// once it is zero, so no frame needs a host round trip.
struct Slot {
  PathState ps{};
  FrameBufs fb{};
  int *q_a = nullptr, *q_b = nullptr, *keep = nullptr, *block_sums = nullptr, *counts = nullptr;
  int *err = nullptr, *fetch = nullptr;
  uint8_t* vis = nullptr;
  float* d_loss = nullptr;
  int* h_err = nullptr;  // pinned copy of err, read once the frame is done
  cudaStream_t st = nullptr;
  cudaEvent_t done = nullptr;
  bool in_flight = false;
  // the frame's path tracing (camera + bounce rounds) as a CUDA graph,
  // replayed every frame of this slot; the frame number comes from d_frame
  int* d_frame = nullptr;
  cudaGraphExec_t trace_exec = nullptr;
  int64_t trace_key[10] = {};
  NrcBufs nrc{};  // NRC renderers
  // path replay (allocated by the first differentiable forward)
  float* gacc = nullptr;       // [groups * 6][P]
  int gacc_rows = 0;
  float* stash = nullptr;      // [13][P]
  double* partial = nullptr;   // [kGradBlocks][groups * 6]
};

constexpr int kGradBlocks = 304;  // blocks of the per-frame gradient sum

struct Render {
  Scene* scene = nullptr;
  int mode = MODE_MSNN;
  int beta_knob = 1;
  int accum_id = 0;
  int n_train = 16384;  // training records per frame (NRC: training pixels)
  int every_nth = 1;
  int in_ch = 12;
  int nn_rows = 0;        // cache queries per frame (NRC: pixels + training suffixes)
  int nrc_records = 0;    // NRC: training records per frame (numTrainingRecords)
  float nrc_c = 0.01f;
  bool train = true;
  bool graphs = true;  // replay each slot's path tracing as a CUDA graph
  uint32_t seed = 0;
  hm_mlp* mlp = nullptr;
  // batch of scenes (hm_render_create_batch): the frame's paths are the
  // scenes' pixels one scene after another; batch.scenes == nullptr otherwise
  std::vector<Scene*> bscenes;
  std::vector<int> bbeta;  // BETA - 1 per scene
  std::vector<BatchScene> bhost;
  Batch batch{nullptr, nullptr, 0};
  int max_path_v2 = 0;
  float4* d_samples = nullptr;  // scene-sample training pass: points on the hair
  int n_samples = 0;
  int pretrain_passes = 0;
  // differentiable rendering (hm_render_diff_forward / _backward)
  bool diff_fwd = false;          // frames being enqueued belong to a differentiable forward
  int diff_frames = 0;            // frames of the last differentiable forward
  int diff_groups = 0;            // material groups it was rendered with
  int diff_material_version = 0;  // the scene's materials it was rendered with
  bool diff_detached = false;     // ... with evaluation materials (no backward)
  int64_t diff_cap_frames = 0;    // capacity of the per-frame buffers
  float4* diff_col = nullptr;     // [frames][P] path radiance
  float* diff_in = nullptr;       // [frames][P][in_ch] cache inputs (replay)
  float* diff_dy = nullptr;       // [frames][P][3] dL/d(cache output)
  double* diff_gframe = nullptr;  // [frames][groups * 6]
  double* diff_gsum = nullptr;    // [groups * 6]
  double* h_gsum = nullptr;       // pinned copy
  void* diff_dual = nullptr;      // [kMaxStrandGroups] HairConstsD
  HairConsts* diff_eval = nullptr;  // [kMaxStrandGroups] evaluation materials (detached renders)
  int P = 0;
  int depth = 0;  // 0: chosen from the frame size in render_setup
  std::vector<Slot> slots;
  double *acc_pt = nullptr, *acc_nn = nullptr, *acc_final = nullptr;
  double* read_stage = nullptr;  // hm_render_read_async: device snapshot of the sums being read
  cudaEvent_t ev_submit = nullptr, ev_mlp = nullptr, ev_compose = nullptr, ev_read = nullptr,
              ev_staged = nullptr;
  bool have_mlp_ev = false, have_compose_ev = false, have_read_ev = false, have_staged_ev = false;
  int* h_count = nullptr;  // pinned (synchronous instrumented frames)
  std::vector<void*> allocs;
  int64_t rays_extend = 0;
  int last_bounces = 0;
  int sm_count = 152;
  int fetch_slots = 0;
  int blocks_extend = 0, blocks_shadow = 0;  // persistent traversal grids
  int blocks_extend_max = 0, blocks_shadow_max = 0;
  int shade_blocks_per_sm = 8;                // shading grid = SMs x this
  int last_error = 0;
  // per-path ray log of the last frame (hm_render_set_path_log; tests)
  float4* log_ev = nullptr;
  int* log_vcur = nullptr;
  int log_slots = 0;
  // instrumentation (synchronous frames)
  bool timing = false, counting = false;
  unsigned long long* d_cnt = nullptr;
  std::vector<cudaEvent_t> ev;
  hm_render_timings tm{};

  ~Render() {
    for (auto& s : slots) {
      if (s.st) cudaStreamSynchronize(s.st);
      if (s.st) cudaStreamDestroy(s.st);
      if (s.done) cudaEventDestroy(s.done);
      if (s.h_err) cudaFreeHost(s.h_err);
      for (void* p : {(void*)s.gacc, (void*)s.stash, (void*)s.partial, (void*)s.ps.beta_d}) cudaFree(p);
      if (s.trace_exec) cudaGraphExecDestroy(s.trace_exec);
    }
    for (void* p : allocs) cudaFree(p);
    if (d_samples) cudaFree(d_samples);
    for (void* p : {(void*)diff_col, (void*)diff_in, (void*)diff_dy, (void*)diff_gframe}) cudaFree(p);
    for (void* p : {(void*)log_ev, (void*)log_vcur}) cudaFree(p);
    if (h_gsum) cudaFreeHost(h_gsum);
    if (h_count) cudaFreeHost(h_count);
    if (mlp) hm_mlp_destroy(mlp);
    for (auto e : ev) cudaEventDestroy(e);
    for (cudaEvent_t e : {ev_submit, ev_mlp, ev_compose, ev_read, ev_staged})
      if (e) cudaEventDestroy(e);
  }
  cudaEvent_t event(size_t i) {
    while (ev.size() <= i) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      ev.push_back(e);
    }
    return ev[i];
  }
  template <class T>
  cudaError_t alloc(T** p, size_t n) {
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e == cudaSuccess) allocs.push_back((void*)*p);
    return e;
  }
};

static const char* kDefaultCacheConfig =
    "{\"loss\":{\"otype\":\"RelativeL2Luminance\"},"
    "\"optimizer\":{\"otype\":\"ExponentialDecay\",\"decay_start\":4000,\"decay_interval\":4000,\"decay_base\":0.33,"
    "\"nested\":{\"otype\":\"Adam\",\"learning_rate\":1e-2,\"beta1\":0.9,\"beta2\":0.99,\"epsilon\":1e-15,\"l2_reg\":1e-6}},"
    "\"encoding\":{\"otype\":\"Composite\",\"nested\":["
    "{\"n_dims_to_encode\":3,\"otype\":\"HashGrid\",\"per_level_scale\":2.0,\"log2_hashmap_size\":15,"
    "\"base_resolution\":16,\"n_levels\":16},"
    "{\"n_dims_to_encode\":6,\"otype\":\"OneBlob\",\"n_bins\":4},{\"otype\":\"Identity\"}]},"
    "\"network\":{\"otype\":\"FullyFusedMLP\",\"activation\":\"ReLU\",\"output_activation\":\"None\","
    "\"n_neurons\":64,\"n_hidden_layers\":2}}";

static cudaError_t slot_alloc(Render* r, Slot& sl) {
  const int P = r->P;
  cudaError_t e = cudaSuccess;
  auto A4 = [&](float4** p) { if (e == cudaSuccess) e = r->alloc(p, P); };
  if (e == cudaSuccess) e = r->alloc(&sl.ps.rng, P);
  if (e == cudaSuccess) e = r->alloc(&sl.ps.flags, P);
  if (e == cudaSuccess) e = r->alloc(&sl.ps.bounce, P);
  A4(&sl.ps.ray_o); A4(&sl.ps.ray_d); A4(&sl.ps.hit); A4(&sl.ps.beta); A4(&sl.ps.beta_s);
  A4(&sl.ps.col); A4(&sl.ps.col_s); A4(&sl.ps.sh_o0); A4(&sl.ps.sh_d0); A4(&sl.ps.sh_o1);
  A4(&sl.ps.sh_d1); A4(&sl.ps.sh_c0); A4(&sl.ps.sh_c1); A4(&sl.ps.dl_w); A4(&sl.ps.dl_ws);
  A4(&sl.fb.gbuf);
  const int nblocks = (P + kScanBlock - 1) / kScanBlock;
  if (e == cudaSuccess) e = r->alloc(&sl.q_a, P);
  if (e == cudaSuccess) e = r->alloc(&sl.q_b, P);
  if (e == cudaSuccess) e = r->alloc(&sl.keep, P);
  if (e == cudaSuccess) e = r->alloc(&sl.block_sums, nblocks + 1);
  if (e == cudaSuccess) e = r->alloc(&sl.counts, 4);
  if (e == cudaSuccess) e = r->alloc(&sl.err, 1);
  if (e == cudaSuccess) e = r->alloc(&sl.fetch, r->fetch_slots);
  if (e == cudaSuccess) e = r->alloc(&sl.vis, (size_t)P * 2);
  if (e == cudaSuccess) e = r->alloc(&sl.d_loss, 1);
  if (e == cudaSuccess) e = r->alloc(&sl.d_frame, 1);
  if (e == cudaSuccess) e = cudaMallocHost(&sl.h_err, sizeof(int));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sl.st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
  if (e != cudaSuccess) return e;
  *sl.h_err = 0;
  cudaMemset(sl.err, 0, sizeof(int));
  cudaMemset(sl.d_loss, 0, sizeof(float));
  sl.fb.acc_pt = r->acc_pt;
  sl.fb.acc_nn = r->acc_nn;
  sl.fb.acc_final = r->acc_final;
  if (r->mode == MODE_MSNN || r->mode == MODE_NRC) {
    const int64_t recs = r->mode == MODE_NRC ? r->nrc_records : r->n_train;
    if (e == cudaSuccess) e = r->alloc(&sl.fb.nn_frame_in, (size_t)r->nn_rows * r->in_ch);
    if (e == cudaSuccess) e = r->alloc(&sl.fb.nn_frame_out, (size_t)r->nn_rows * 3);
    if (e == cudaSuccess) e = r->alloc(&sl.fb.nn_train_in, (size_t)recs * r->in_ch);
    if (e == cudaSuccess) e = r->alloc(&sl.fb.nn_train_out, (size_t)recs * 3);
    if (e != cudaSuccess) return e;
    cudaMemset(sl.fb.nn_frame_in, 0, (size_t)r->nn_rows * r->in_ch * sizeof(float));
    cudaMemset(sl.fb.nn_train_in, 0, (size_t)recs * r->in_ch * sizeof(float));
    cudaMemset(sl.fb.nn_train_out, 0, (size_t)recs * 3 * sizeof(float));
  }
  if (r->mode == MODE_NRC) {
    NrcBufs& nb = sl.nrc;
    const int R = r->n_train;
    if (e == cudaSuccess) e = r->alloc(&nb.prev, (size_t)P);
    if (e == cudaSuccess) e = r->alloc(&nb.spread, (size_t)P);
    if (e == cudaSuccess) e = r->alloc(&nb.gbeta, (size_t)P);
    if (e == cudaSuccess) e = r->alloc(&nb.dl_rec, (size_t)P);
    if (e == cudaSuccess) e = r->alloc(&nb.rec, (size_t)R * kNrcMaxBounces * kNrcRecordF4);
    if (e == cudaSuccess) e = r->alloc(&nb.tinfo, (size_t)R);
    if (e != cudaSuccess) return e;
    cudaMemset(nb.rec, 0, (size_t)R * kNrcMaxBounces * kNrcRecordF4 * sizeof(float4));
    cudaMemset(nb.tinfo, 0, (size_t)R * sizeof(int4));
    nb.c = r->nrc_c;
    nb.all_unbiased = 0;
  }
  return e;
}

static int render_setup(Render* r, const hm_render_options* o) {
  Scene* s = r->scene;
  if (int st = s->ensure_built()) return st;
  r->P = s->width * s->height;
  r->max_path_v2 = s->path_v2;
  if (!r->bscenes.empty()) {
    int64_t total = 0;
    for (Scene* b : r->bscenes) {
      if (int st = b->ensure_built()) return st;
      total += (int64_t)b->width * b->height;
      r->max_path_v2 = std::max(r->max_path_v2, b->path_v2);
    }
    if (total > INT32_MAX / 4) return hm_set_error("hm_render_create_batch: too many pixels"), HM_ECAPACITY;
    r->P = (int)total;
  }
  const int P = r->P;
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = r->alloc(&r->acc_pt, (size_t)P * 3);
  if (e == cudaSuccess) e = r->alloc(&r->acc_nn, (size_t)P * 3);
  if (e == cudaSuccess) e = r->alloc(&r->acc_final, (size_t)P * 3);
  if (e == cudaSuccess) e = r->alloc(&r->d_cnt, 8);
  if (e == cudaSuccess) e = cudaMallocHost(&r->h_count, sizeof(int));
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->ev_submit, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->ev_mlp, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->ev_compose, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->ev_read, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->ev_staged, cudaEventDisableTiming);
  if (e != cudaSuccess) return hm_cuda_status(e, "render buffers");
  cudaMemset(r->acc_pt, 0, (size_t)P * 3 * sizeof(double));
  cudaMemset(r->acc_nn, 0, (size_t)P * 3 * sizeof(double));
  cudaMemset(r->acc_final, 0, (size_t)P * 3 * sizeof(double));
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&r->sm_count, cudaDevAttrMultiProcessorCount, dev);
  r->fetch_slots = 2 * (std::max(r->max_path_v2, kNrcMaxBounces) + 2);
  r->blocks_extend = r->blocks_extend_max = persistent_blocks<ExtendRays, false>();
  r->blocks_shadow = r->blocks_shadow_max = persistent_blocks<ShadowRays, true>();
  r->nn_rows = P;
  if (r->mode == MODE_MSNN) {
    r->n_train = o && o->train_records > 0 ? o->train_records : 16384;
    // everyNth = frameSize / numTrainRecords (integer division, render_hair_msnn.cu:106), at least 1
    r->every_nth = std::max(1, P / r->n_train);
    r->n_train = std::min(r->n_train, (P + r->every_nth - 1) / r->every_nth);
  } else if (r->mode == MODE_NRC) {
    // render_nrc.cu:124-146: numTrainingPixels = numTrainingRecords / MAX_BOUNCES,
    // everyNth = frameSize / numTrainingPixels; the cache queries are the
    // frame's pixels plus one per training suffix; cache inputs are 9
    // channels (render_nrc.h:123)
    r->nrc_records = o && o->train_records > 0 ? o->train_records : 65536;
    r->n_train = std::max(1, r->nrc_records / kNrcMaxBounces);
    r->every_nth = std::max(1, P / r->n_train);
    r->n_train = std::min(r->n_train, (P + r->every_nth - 1) / r->every_nth);
    r->nrc_records = std::max(r->nrc_records, r->n_train * kNrcMaxBounces);
    r->in_ch = 9;
    r->nn_rows = P + r->n_train;
    if (o && o->nrc_c > 0.f) r->nrc_c = o->nrc_c;
  }
  if (!r->bscenes.empty()) {
    // one shared cache: every scene gives one training record per every_nth
    // of its pixels, records stored scene after scene
    int pix = 0, rec = 0;
    r->bhost.clear();
    for (size_t k = 0; k < r->bscenes.size(); ++k) {
      Scene* b = r->bscenes[k];
      BatchScene bs{};
      bs.s = b->dev();
      if (((uintptr_t)bs.s.wnodes & 31) != 0)  // the traversal's 32-byte node loads
        return hm_set_error("batch scene %d: wide nodes not 32-byte aligned", (int)k), HM_EINVAL;
      bs.pix_off = pix;
      bs.n_pix = b->width * b->height;
      bs.every_nth = r->every_nth;
      bs.n_train = r->mode == MODE_MSNN ? (bs.n_pix + r->every_nth - 1) / r->every_nth : 0;
      bs.train_off = rec;
      bs.beta = r->bbeta[k];
      pix += bs.n_pix;
      rec += bs.n_train;
      r->bhost.push_back(bs);
    }
    if (r->mode == MODE_MSNN) r->n_train = rec;
    std::vector<int> owner(P);
    for (size_t k = 0; k < r->bhost.size(); ++k)
      std::fill(owner.begin() + r->bhost[k].pix_off, owner.begin() + r->bhost[k].pix_off + r->bhost[k].n_pix, (int)k);
    BatchScene* d_bs = nullptr;
    int* d_owner = nullptr;
    e = r->alloc(&d_bs, r->bhost.size());
    if (e == cudaSuccess) e = r->alloc(&d_owner, (size_t)P);
    if (e == cudaSuccess)
      e = cudaMemcpy(d_bs, r->bhost.data(), r->bhost.size() * sizeof(BatchScene), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_owner, owner.data(), (size_t)P * sizeof(int), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return hm_cuda_status(e, "batch tables");
    r->batch = Batch{d_bs, d_owner, P};
  }
  if (r->depth <= 0) {
    // default: up to 8 frames in flight (the measured optimum at 512x512:
    // 4.6 ms per frame against 4.7 ms with 6 and 4.9 ms with 5), keeping the
    // per-slot path state and queues under about 2 GB in total
    const int64_t slot_bytes = (int64_t)P * 360;
    r->depth = (int)std::max<int64_t>(2, std::min<int64_t>(8, ((int64_t)2 << 30) / std::max<int64_t>(1, slot_bytes)));
  }
  r->slots.resize(r->depth);
  for (auto& sl : r->slots) {
    e = slot_alloc(r, sl);
    if (e != cudaSuccess) return hm_cuda_status(e, "render frame slot");
  }
  if (r->mode == MODE_MSNN || r->mode == MODE_NRC) {
    std::string cfg = o && o->cache_config_json ? o->cache_config_json
                                                : (s->cache_config.empty() ? kDefaultCacheConfig : s->cache_config);
    int st = 0;
    r->mlp = hm_mlp_create(cfg.c_str(), r->in_ch, 3, o ? o->cache_precision : HM_PREC_FP32, r->seed, &st);
    if (!r->mlp) return st;
    // the scene's tcnn.init_weights (render_hair_msnn.cu:109-110)
    if (!s->cache_weights.empty())
      if (int e3 = hm_mlp_load(r->mlp, s->cache_weights.c_str())) return e3;
  }
  cudaError_t e2 = cudaDeviceSynchronize();
  return e2 == cudaSuccess ? HM_OK : hm_cuda_status(e2, "render setup");
}

// Waits for a slot's frame and reports its traversal error bits.
static int slot_finish(Render* r, Slot& sl) {
  if (!sl.in_flight) return HM_OK;
  cudaError_t e = cudaEventSynchronize(sl.done);
  sl.in_flight = false;
  if (e != cudaSuccess) return hm_cuda_status(e, "render frame");
  if (*sl.h_err) {
    int bits = *sl.h_err;
    *sl.h_err = 0;
    cudaMemset(sl.err, 0, sizeof(int));
    return hm_set_error("traversal gave up on some rays (error bits 0x%x)", bits), HM_ECAPACITY;
  }
  return HM_OK;
}

static int render_sync(Render* r) {
  int status = HM_OK;
  for (auto& sl : r->slots) {
    int s = slot_finish(r, sl);
    if (s && !status) status = s;
  }
  return status;
}

// Bounce rounds a frame enqueues: path_v2 + 1, or, for HairMSNN frames
// without training pixels, the short paths' BETA + 1 vertices (at least 2):
// vertex k > beta = BETA - 1 always ends the path.
static int bounce_rounds(const Render* r, const FrameParams& fp) {
  if (fp.mode == MODE_NRC) return kNrcMaxBounces;  // the 40th vertex ends every path
  const int full = r->max_path_v2 + 1;
  if (fp.mode == MODE_MSNN && fp.no_train && r->bscenes.empty())
    return std::min(full, std::max(2, r->beta_knob + 1));
  return full;
}

__global__ void set_frame_kernel(int* d_frame, int v) { *d_frame = v; }

// Enqueues one frame.  sync_bounces: read the queue length after every
// bounce (instrumented frames: per-stage events, early exit); otherwise the
// whole frame is enqueued without a host round trip.
static int render_frame(Render* r, cudaStream_t user, bool sync_bounces) {
  Scene* s = r->scene;
  SceneDev sd = s->dev();
  Slot& sl = r->slots[r->accum_id % r->depth];
  if (int e = slot_finish(r, sl)) return e;  // back-pressure: the slot's previous frame
  const cudaStream_t st = sl.st;
  cudaEventRecord(r->ev_submit, user);
  cudaStreamWaitEvent(st, r->ev_submit, 0);
  FrameParams fp{r->mode, r->beta_knob - 1, r->accum_id, r->accum_id + 10007, r->every_nth, r->n_train, r->in_ch,
                 0, nullptr, 0, 0u};
  FrameBufs fb = sl.fb;
  if (r->log_ev && !r->diff_fwd) {
    fp.log = PathLog{r->log_ev, r->log_vcur, r->log_slots};
    cudaMemsetAsync(r->log_ev, 0xff, (size_t)r->P * r->log_slots * 3 * sizeof(float4), st);
  }
  if (!r->diff_fwd) r->diff_frames = 0;  // a plain frame ends the replayable forward
  if (r->diff_fwd) {  // a frame of a differentiable forward
    fp.no_train = 1;
    fp.eval_hc = r->diff_detached ? r->diff_eval : nullptr;
    fb.col_out = r->diff_col + (size_t)r->accum_id * r->P;
  }
  // instrumentation: event pairs per stage (timing) / work counters (counting)
  size_t ne = 0;
  int cur_bounce = -1;
  std::vector<std::pair<int, size_t>> marks;  // (stage, event index)
  std::vector<int> mark_bounce;
  std::vector<int> paths_at;
  auto mark = [&](int stage) {
    if (!r->timing || !sync_bounces) return;
    cudaEventRecord(r->event(ne), st);
    marks.emplace_back(stage, ne++);
    mark_bounce.push_back(cur_bounce);
  };
  enum { S_CAMERA, S_EXTEND, S_SHADE, S_SHADOW, S_COMPACT, S_FINALIZE, S_TRAIN, S_INFER, S_COMPOSE, S_END };
  const bool counting = r->counting && sync_bounces;
  if (counting) cudaMemsetAsync(r->d_cnt, 0, 8 * sizeof(unsigned long long), st);
  const int grid = r->sm_count * r->shade_blocks_per_sm;
  const int nblocks = (r->P + kScanBlock - 1) / kScanBlock;
  int count = r->P;
  int bounces = 0;
  int64_t ext_rays = 0;
  const int rounds = bounce_rounds(r, fp);
  FrameBufs fb_trace = fb;
  fb_trace.col_out = nullptr;  // finalize's; keeps the traced launches identical across frames
  // camera + bounce rounds (extend -> shade -> shadow -> resolve -> compact)
  auto trace = [&](const FrameParams& tfp) -> int {
    int* q_cur = sl.q_a;
    int* q_next = sl.q_b;
    int* c_cur = sl.counts;
    int* c_next = sl.counts + 1;
    cudaMemsetAsync(sl.fetch, 0, r->fetch_slots * sizeof(int), st);
    mark(S_CAMERA);
    if (tfp.mode == MODE_NRC) {
      if (int e = launch_nrc_camera(sd, tfp, sl.ps, fb_trace, sl.nrc, q_cur, c_cur, st)) return e;
    } else {
      if (int e = launch_camera(sd, tfp, r->batch, sl.ps, q_cur, c_cur, st)) return e;
    }
    bounces = 0;
    for (int it = 0; it < rounds && count > 0; ++it) {
      cur_bounce = it;
      paths_at.push_back(count);
      mark(S_EXTEND);
      if (int e = launch_persistent<ExtendRays, false>(ExtendRays{sl.ps, q_cur, c_cur}, sd, r->batch, 0.f, 1e30f,
                                                       sl.fetch + 2 * it, sl.err, r->d_cnt, counting,
                                                       r->blocks_extend, st))
        return e;
      mark(S_SHADE);
      if (tfp.mode == MODE_NRC) {
        if (int e = launch_nrc_shade(sd, tfp, sl.ps, fb_trace, sl.nrc, q_cur, c_cur, sl.keep, grid, st)) return e;
      } else {
        if (int e = launch_shade(sd, tfp, r->batch, sl.ps, fb_trace, q_cur, c_cur, sl.keep, grid, st)) return e;
      }
      mark(S_SHADOW);
      if (int e = launch_persistent<ShadowRays, true>(ShadowRays{sl.ps, q_cur, c_cur, sl.vis}, sd, r->batch, 0.f,
                                                      1e30f, sl.fetch + 2 * it + 1, sl.err, r->d_cnt + 3, counting,
                                                      r->blocks_shadow, st))
        return e;
      shadow_resolve_kernel<false><<<grid, 256, 0, st>>>(sl.ps, q_cur, c_cur, sl.vis, DiffParams{},
                                                         tfp.mode == MODE_NRC ? sl.nrc.dl_rec : nullptr,
                                                         sl.nrc.rec, tfp.log);
      HM_CHECK_LAUNCH("shadow_resolve_kernel");
      mark(S_COMPACT);
      scan_count_kernel<<<std::min(nblocks, r->sm_count * 2), kScanBlock, 0, st>>>(sl.keep, c_cur, sl.block_sums,
                                                                                    nblocks);
      scan_blocks_kernel<<<1, 1024, 0, st>>>(sl.block_sums, c_cur, c_next);
      scatter_kernel<<<std::min(nblocks, r->sm_count * 2), kScanBlock, 0, st>>>(sl.keep, q_cur, c_cur,
                                                                                sl.block_sums, q_next, nblocks);
      HM_CHECK_LAUNCH("compaction");
      if (sync_bounces) {
        ext_rays += count;
        cudaError_t e = cudaMemcpyAsync(r->h_count, c_next, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return hm_cuda_status(e, "bounce count");
        count = *r->h_count;
      }
      std::swap(q_cur, q_next);
      std::swap(c_cur, c_next);
      ++bounces;
    }
    return HM_OK;
  };
  if (r->graphs && !sync_bounces) {
    // the same launches as a graph per slot, captured once and replayed;
    // the camera kernel reads the frame number from the slot's d_frame
    set_frame_kernel<<<1, 1, 0, st>>>(sl.d_frame, r->accum_id);
    HM_CHECK_LAUNCH("set_frame_kernel");
    FrameParams tfp = fp;
    tfp.d_frame = sl.d_frame;
    const int64_t key[10] = {rounds, r->blocks_extend, r->blocks_shadow, grid, s->material_version, tfp.no_train,
                             (int64_t)(uintptr_t)tfp.eval_hc, (int64_t)(uintptr_t)sl.ps.beta_d, r->mode,
                             (int64_t)(uintptr_t)tfp.log.ev};
    if (!sl.trace_exec || memcmp(key, sl.trace_key, sizeof(key)) != 0) {
      if (sl.trace_exec) cudaGraphExecDestroy(sl.trace_exec);
      sl.trace_exec = nullptr;
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed);
      if (e != cudaSuccess) return hm_cuda_status(e, "trace graph capture");
      const int te = trace(tfp);
      e = cudaStreamEndCapture(st, &g);
      if (te != HM_OK || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return te != HM_OK ? te : hm_cuda_status(e, "trace graph capture");
      }
      e = cudaGraphInstantiate(&sl.trace_exec, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return hm_cuda_status(e, "trace graph instantiate");
      memcpy(sl.trace_key, key, sizeof(key));
    }
    cudaError_t e = cudaGraphLaunch(sl.trace_exec, st);
    if (e != cudaSuccess) return hm_cuda_status(e, "trace graph launch");
    bounces = rounds;
  } else {
    if (int e = trace(fp)) return e;
  }
  r->rays_extend += ext_rays;
  r->last_bounces = bounces;
  cur_bounce = -1;
  int launches = 1 + 7 * bounces + 1;
  if (r->mode == MODE_NRC) {
    // G_BUFFER done; then inference, RENDER pass (compose + training data),
    // training step (render_nrc.cu:651-681)
    mark(S_FINALIZE);
    if (int e = launch_nrc_finalize(r->P, sl.ps, fb, nullptr, st)) return e;
    if (r->have_mlp_ev) cudaStreamWaitEvent(st, r->ev_mlp, 0);
    mark(S_INFER);
    if (int e = hm_mlp_inference(r->mlp, fb.nn_frame_in, fb.nn_frame_out, r->nn_rows, st)) return e;
    if (r->have_compose_ev) cudaStreamWaitEvent(st, r->ev_compose, 0);
    if (r->have_read_ev) cudaStreamWaitEvent(st, r->ev_read, 0);
    mark(S_COMPOSE);
    if (int e = launch_nrc_compose(r->P, r->n_train, fp, fb, sl.nrc, st)) return e;
    cudaEventRecord(r->ev_compose, st);
    r->have_compose_ev = true;
    mark(S_TRAIN);
    if (r->train) {
      if (int e = hm_mlp_training_step(r->mlp, fb.nn_train_in, fb.nn_train_out, r->nrc_records, sl.d_loss, st))
        return e;
    }
    cudaEventRecord(r->ev_mlp, st);
    r->have_mlp_ev = true;
    hm_mlp_desc md;
    hm_mlp_info(r->mlp, &md);
    const bool grid_enc = md.n_params > md.n_network_params;
    launches += (r->train ? 4 + 2 * (md.n_hidden_layers + 1) + (grid_enc ? 2 : 0) + 1 : 0) + 2 + 2;
  } else if (r->mode == MODE_PT) {
    // writePixel accumulates: frames in order, after any pending read-back
    if (r->have_compose_ev) cudaStreamWaitEvent(st, r->ev_compose, 0);
    if (r->have_read_ev) cudaStreamWaitEvent(st, r->ev_read, 0);
    mark(S_FINALIZE);
    if (int e = launch_finalize(sd, fp, r->batch, sl.ps, fb, st)) return e;
    cudaEventRecord(r->ev_compose, st);
    r->have_compose_ev = true;
  } else {
    mark(S_FINALIZE);
    if (int e = launch_finalize(sd, fp, r->batch, sl.ps, fb, st)) return e;
    // cache step: after the previous frame's inference (weights and workspace)
    if (r->have_mlp_ev) cudaStreamWaitEvent(st, r->ev_mlp, 0);
    mark(S_TRAIN);
    if (r->train && !r->diff_fwd) {
      if (int e = hm_mlp_training_step(r->mlp, fb.nn_train_in, fb.nn_train_out, r->n_train, sl.d_loss, st))
        return e;
    }
    mark(S_INFER);
    if (int e = hm_mlp_inference(r->mlp, fb.nn_frame_in, fb.nn_frame_out, r->P, st)) return e;
    cudaEventRecord(r->ev_mlp, st);
    r->have_mlp_ev = true;
    if (r->have_compose_ev) cudaStreamWaitEvent(st, r->ev_compose, 0);
    if (r->have_read_ev) cudaStreamWaitEvent(st, r->ev_read, 0);
    mark(S_COMPOSE);
    if (int e = launch_compose(r->P, fp, fb, st)) return e;
    cudaEventRecord(r->ev_compose, st);
    r->have_compose_ev = true;
    hm_mlp_desc md;
    hm_mlp_info(r->mlp, &md);
    const bool grid_enc = md.n_params > md.n_network_params;
    launches += (r->train && !r->diff_fwd ? 4 + 2 * (md.n_hidden_layers + 1) + (grid_enc ? 2 : 0) + 1 : 0) + 2 + 1;
  }
  mark(S_END);
  cudaMemcpyAsync(sl.h_err, sl.err, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaEventRecord(sl.done, st);
  sl.in_flight = true;
  r->accum_id += 1;
  hm_render_timings& tm = r->tm;
  memset(&tm, 0, sizeof(tm));
  tm.bounces = bounces;
  tm.extension_rays = ext_rays;
  tm.kernel_launches = launches;
  if (r->timing && sync_bounces) {
    cudaEventSynchronize(r->event(ne - 1));
    float* slot[] = {&tm.camera_ms, &tm.extend_ms, &tm.shade_ms, &tm.shadow_ms, &tm.compact_ms,
                     &tm.finalize_ms, &tm.train_ms, &tm.infer_ms, &tm.compose_ms};
    for (size_t k = 0; k + 1 < marks.size(); ++k) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, r->event(marks[k].second), r->event(marks[k + 1].second));
      *slot[marks[k].first] += ms;
      const int b = mark_bounce[k];
      if (b >= 0 && b < 48) {
        if (marks[k].first == S_EXTEND) tm.extend_ms_by_bounce[b] += ms;
        if (marks[k].first == S_SHADOW) tm.shadow_ms_by_bounce[b] += ms;
      }
    }
    for (size_t b = 0; b < paths_at.size() && b < 48; ++b) tm.paths_by_bounce[b] = paths_at[b];
    cudaEventElapsedTime(&tm.total_ms, r->event(marks.front().second), r->event(marks.back().second));
  }
  if (counting) {
    unsigned long long c[8];
    cudaMemcpyAsync(c, r->d_cnt, sizeof(c), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    tm.extend_nodes = (int64_t)c[0];
    tm.extend_prims = (int64_t)c[1];
    tm.shadow_nodes = (int64_t)c[3];
    tm.shadow_prims = (int64_t)c[4];
    tm.shadow_rays = (int64_t)c[5];
  }
  if (sync_bounces) return slot_finish(r, sl);
  return HM_OK;
}

}  // namespace hm

using namespace hm;

static hm_render* render_create(Scene* first, const std::vector<Scene*>& batch, const int* betas,
                                const hm_render_options* opt, int* status) {
  Render* r = new Render();
  r->scene = first;
  if (opt) {
    r->mode = opt->mode;
    r->beta_knob = opt->beta;
    r->train = opt->train != 0;
    r->seed = opt->seed;
    if (opt->frames_in_flight > 0) r->depth = std::min(opt->frames_in_flight, 8);
  } else {
    r->train = r->scene->cache_train;
  }
  auto fail = [&](int st, const char* msg) -> hm_render* {
    delete r;
    *status = st;
    if (msg) hm_set_error("%s", msg);
    return nullptr;
  };
  if (r->mode != MODE_PT && r->mode != MODE_MSNN && r->mode != MODE_NRC)
    return fail(HM_EINVAL, "hm_render_create: unknown mode");
  if (r->mode == MODE_NRC && !batch.empty())
    return fail(HM_EUNSUPPORTED, "hm_render_create_batch: NRC renders single scenes");
  // internal beta = BETA - 1 (render_hair_msnn.cu:1170); BETA = 0 stops the
  // short path at the first bounce
  if (r->beta_knob < 0) return fail(HM_EINVAL, "hm_render_create: BETA must be >= 0 (internal beta = BETA - 1)");
  if (!batch.empty()) {
    r->bscenes = batch;
    for (size_t k = 0; k < batch.size(); ++k) {
      const int bk = betas ? betas[k] : r->beta_knob;
      if (bk < 0) return fail(HM_EINVAL, "hm_render_create_batch: BETA must be >= 0");
      r->bbeta.push_back(bk - 1);
    }
  }
  int st = render_setup(r, opt);
  if (st != HM_OK) return fail(st, nullptr);
  *status = HM_OK;
  return (hm_render*)r;
}

extern "C" hm_render* hm_render_create(hm_scene* scene, const hm_render_options* opt, int* status) {
  int dummy;
  if (!status) status = &dummy;
  if (!scene) {
    *status = HM_EINVAL;
    hm_set_error("hm_render_create: NULL scene");
    return nullptr;
  }
  return render_create((Scene*)scene, {}, nullptr, opt, status);
}

extern "C" hm_render* hm_render_create_batch(hm_scene* const* scenes, const int* betas, int n_scenes,
                                             const hm_render_options* opt, int* status) {
  int dummy;
  if (!status) status = &dummy;
  if (!scenes || n_scenes < 1) {
    *status = HM_EINVAL;
    hm_set_error("hm_render_create_batch: no scenes");
    return nullptr;
  }
  std::vector<Scene*> v;
  for (int k = 0; k < n_scenes; ++k) {
    if (!scenes[k]) {
      *status = HM_EINVAL;
      hm_set_error("hm_render_create_batch: NULL scene %d", k);
      return nullptr;
    }
    v.push_back((Scene*)scenes[k]);
  }
  return render_create(v[0], v, betas, opt, status);
}

extern "C" int hm_render_batch_scene(const hm_render* h, int scene, int* pixel_offset, int* width, int* height) {
  const Render* r = (const Render*)h;
  if (!r) return hm_set_error("hm_render_batch_scene: NULL"), HM_EINVAL;
  const int n = r->bscenes.empty() ? 1 : (int)r->bscenes.size();
  if (scene < 0 || scene >= n) return hm_set_error("hm_render_batch_scene: scene %d of %d", scene, n), HM_EINVAL;
  const Scene* sc = r->bscenes.empty() ? r->scene : r->bscenes[scene];
  if (pixel_offset) *pixel_offset = r->bscenes.empty() ? 0 : r->bhost[scene].pix_off;
  if (width) *width = sc->width;
  if (height) *height = sc->height;
  return HM_OK;
}

extern "C" void hm_render_destroy(hm_render* h) { delete (Render*)h; }

extern "C" int hm_render_frame(hm_render* h, void* stream) {
  Render* r = (Render*)h;
  if (!r) return hm_set_error("hm_render_frame: NULL"), HM_EINVAL;
  // asynchronous unless instrumented: errors of a frame are reported when its
  // slot is reused or at the next synchronising call (read / stats / reset)
  return render_frame(r, (cudaStream_t)stream, r->timing || r->counting);
}

// Asynchronous read-back of the FP64 running sums (not averaged) of every
// frame enqueued so far into host_dst (pinned for a true async copy), on
// `stream`; the next frame's accumulation waits for the copy.
extern "C" int hm_render_read_async(hm_render* h, int which, double* host_dst, void* stream) {
  Render* r = (Render*)h;
  if (!r || !host_dst) return hm_set_error("hm_render_read_async: NULL"), HM_EINVAL;
  const double* src = which == HM_IMAGE_FINAL ? r->acc_final
                      : which == HM_IMAGE_SHORT ? r->acc_pt
                      : which == HM_IMAGE_CACHE ? r->acc_nn : nullptr;
  if (!src) return hm_set_error("hm_render_read_async: unknown image %d", which), HM_EINVAL;
  if (r->mode != MODE_MSNN && which != HM_IMAGE_FINAL)
    return hm_set_error("hm_render_read_async: PT and NRC renders have only the final image"), HM_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t bytes = (size_t)r->P * 3 * sizeof(double);
  cudaError_t e = cudaSuccess;
  if (!r->read_stage) e = r->alloc(&r->read_stage, (size_t)r->P * 3);
  // the sums are snapshotted on the device and the host copy is made from the
  // snapshot, so the next frame's accumulation waits only for the device copy
  if (r->have_compose_ev) cudaStreamWaitEvent(s, r->ev_compose, 0);
  if (r->have_staged_ev) cudaStreamWaitEvent(s, r->ev_staged, 0);  // the previous host copy is done
  if (e == cudaSuccess) e = cudaMemcpyAsync(r->read_stage, src, bytes, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaEventRecord(r->ev_read, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(host_dst, r->read_stage, bytes, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaEventRecord(r->ev_staged, s);
  if (e != cudaSuccess) return hm_cuda_status(e, "hm_render_read_async");
  r->have_read_ev = true;
  r->have_staged_ev = true;
  return HM_OK;
}

// ---- launch-shape autotuner
// Times pipelined frames for candidate launch shapes and keeps the fastest:
// the persistent traversal grids (resident blocks per SM, extension and
// shadow rays tuned together, then each alone) and the shading grid.  These
// shapes do not change any result (every ray and path is computed alone), and
// the tuning frames neither train the cache nor stay in the image: training
// is paused and the renderer is reset afterwards, so a tuned renderer renders
// exactly what an untuned one does.
static int render_autotune(Render* r, int frames, cudaStream_t user, hm_render_tuning* out) {
  if (int e = render_sync(r)) return e;
  const bool train = r->train;
  r->train = false;
  cudaEvent_t a = nullptr, b = nullptr;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  auto time_frames = [&](float* ms) -> int {
    cudaEventRecord(a, user);
    for (int k = 0; k < frames; ++k)
      if (int e = render_frame(r, user, false)) return e;
    for (auto& sl : r->slots)
      if (sl.in_flight) cudaStreamWaitEvent(user, sl.done, 0);
    cudaEventRecord(b, user);
    cudaError_t e = cudaEventSynchronize(b);
    if (e != cudaSuccess) return hm_cuda_status(e, "autotune");
    cudaEventElapsedTime(ms, a, b);
    return render_sync(r);
  };
  int status = HM_OK;
  float warm = 0.f;
  status = time_frames(&warm);  // warm-up at the current shapes
  const int sms = r->sm_count;
  const int ext_max = r->blocks_extend_max / sms, sh_max = r->blocks_shadow_max / sms;
  auto tune = [&](int* ext_per_sm, int* sh_per_sm, bool both, bool ext_only) {
    float best = 1e30f;
    int best_e = *ext_per_sm, best_s = *sh_per_sm;
    const int hi = std::max(ext_max, sh_max);
    for (int c = 2; c <= hi && status == HM_OK; ++c) {
      const int ce = both || ext_only ? std::min(c, ext_max) : *ext_per_sm;
      const int cs = both || !ext_only ? std::min(c, sh_max) : *sh_per_sm;
      r->blocks_extend = ce * sms;
      r->blocks_shadow = cs * sms;
      float ms = 0.f;
      status = time_frames(&ms);
      if (ms < best) {
        best = ms;
        best_e = ce;
        best_s = cs;
      }
    }
    *ext_per_sm = best_e;
    *sh_per_sm = best_s;
    r->blocks_extend = best_e * sms;
    r->blocks_shadow = best_s * sms;
    return best;
  };
  int e_per_sm = ext_max, s_per_sm = sh_max;
  tune(&e_per_sm, &s_per_sm, true, false);
  tune(&e_per_sm, &s_per_sm, false, true);
  float best_ms = tune(&e_per_sm, &s_per_sm, false, false);
  int best_grid = r->shade_blocks_per_sm;
  for (int g : {4, 8, 16}) {
    if (status != HM_OK) break;
    r->shade_blocks_per_sm = g;
    float ms = 0.f;
    status = time_frames(&ms);
    if (ms < best_ms) {
      best_ms = ms;
      best_grid = g;
    }
  }
  r->shade_blocks_per_sm = best_grid;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  r->train = train;
  // forget the tuning frames
  r->accum_id = 0;
  if (out) {
    out->extend_blocks_per_sm = e_per_sm;
    out->shadow_blocks_per_sm = s_per_sm;
    out->shade_blocks_per_sm = best_grid;
    out->ms_per_frame = best_ms / (float)std::max(1, frames);
  }
  return status;
}

extern "C" int hm_render_autotune(hm_render* h, int frames, void* stream, hm_render_tuning* out) {
  Render* r = (Render*)h;
  if (!r || frames < 1) return hm_set_error("hm_render_autotune: bad arguments"), HM_EINVAL;
  return render_autotune(r, frames, (cudaStream_t)stream, out);
}

extern "C" int hm_render_set_graphs(hm_render* h, int on) {
  Render* r = (Render*)h;
  if (!r) return hm_set_error("hm_render_set_graphs: NULL"), HM_EINVAL;
  if (int e = render_sync(r)) return e;
  r->graphs = on != 0;
  return HM_OK;
}

extern "C" int hm_render_frames_in_flight(const hm_render* h) {
  const Render* r = (const Render*)h;
  return r ? r->depth : 0;
}

extern "C" int hm_render_wait(hm_render* h, void* stream) {
  Render* r = (Render*)h;
  if (!r) return HM_EINVAL;
  for (auto& sl : r->slots)
    if (sl.in_flight) {
      cudaError_t e = cudaStreamWaitEvent((cudaStream_t)stream, sl.done, 0);
      if (e != cudaSuccess) return hm_cuda_status(e, "hm_render_wait");
    }
  return HM_OK;
}

// ---- scene-sample training pass (initialize(), render_hair_msnn.cu:641-650)
// Points on the hair: fetchSceneSamples (render_hair_msnn.cu:34-97) gives
// each segment int(length / total length * 1e6) uniform samples, at least
// one, with length = |p1 - p0| + |p2 - p1| + |p3 - p2| of its control points
// (:359-367).  The reference evaluates the points on the Catmull-Rom
// interpretation of the control points; they only aim the training rays,
// which then hit whatever hair lies that way, and here they are taken on
// the B-spline curve that is intersected.  (The reference also looks the
// lengths up by control-point index instead of segment number; each
// segment's own length is used here.)
static int build_scene_samples(Render* r) {
  const Scene* sc = r->scene;
  const int n_seg = (int)sc->seg.size();
  if (n_seg == 0) return hm_set_error("hm_render_pretrain: the scene has no hair"), HM_EINVAL;
  std::vector<float> len(n_seg);
  double total = 0.0;
  auto pt = [&](int i) { const float4 c = sc->cp[i]; return mk(c.x, c.y, c.z); };
  for (int k = 0; k < n_seg; ++k) {
    const int i = sc->seg[k];
    len[k] = length(pt(i) - pt(i + 1)) + length(pt(i + 2) - pt(i + 1)) + length(pt(i + 3) - pt(i + 2));
    total += len[k];
  }
  const double wanted = 1e6;
  std::vector<float4> samples;
  samples.reserve((size_t)wanted + n_seg);
  uint32_t st = rng_seed((int)r->seed, 0x5a3u);
  for (int k = 0; k < n_seg; ++k) {
    int m = (int)((double)len[k] / total * wanted);
    if (m == 0) m = 1;
    const int i = sc->seg[k];
    const f3 q0 = pt(i), q1 = pt(i + 1), q2 = pt(i + 2), q3 = pt(i + 3);
    for (int j = 0; j < m; ++j) {
      const float u = lcg_next(st), v = 1.f - u;
      // uniform cubic B-spline basis
      const float b0 = v * v * v / 6.f, b1 = (3.f * u * u * u - 6.f * u * u + 4.f) / 6.f;
      const float b2 = (-3.f * u * u * u + 3.f * u * u + 3.f * u + 1.f) / 6.f, b3 = u * u * u / 6.f;
      const f3 p = q0 * b0 + q1 * b1 + q2 * b2 + q3 * b3;
      samples.push_back(make_float4(p.x, p.y, p.z, 0.f));
    }
  }
  cudaError_t e = cudaMalloc(&r->d_samples, samples.size() * sizeof(float4));
  if (e == cudaSuccess)
    e = cudaMemcpy(r->d_samples, samples.data(), samples.size() * sizeof(float4), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return hm_cuda_status(e, "scene samples");
  r->n_samples = (int)samples.size();
  return HM_OK;
}

// `passes` rounds of: n_train training paths aimed at scene samples (the
// TRAIN_DATA_GEN pass, hair_msnn.cu:222-233, 240-272), then one training
// step (train(), render_hair_msnn.cu:666-697).  The reference repeats this
// for one second of wall time; here the count is explicit.  Each pass uses a
// new permutation of the samples and the RNG seed of its pass number, like
// the reference's accumId during initial training.
static int render_pretrain(Render* r, int passes, cudaStream_t user) {
  if (r->mode != MODE_MSNN) return hm_set_error("hm_render_pretrain: HairMSNN renderers only"), HM_EINVAL;
  if (!r->bscenes.empty()) return hm_set_error("hm_render_pretrain: not available for batches"), HM_EUNSUPPORTED;
  if (int e = render_sync(r)) return e;
  if (!r->d_samples)
    if (int e = build_scene_samples(r)) return e;
  Scene* s = r->scene;
  const SceneDev sd = s->dev();
  Slot& sl = r->slots[0];
  const cudaStream_t st = sl.st;
  cudaEventRecord(r->ev_submit, user);
  cudaStreamWaitEvent(st, r->ev_submit, 0);
  const int grid = r->sm_count * 8;
  const int nblocks = (r->n_train + kScanBlock - 1) / kScanBlock;
  for (int pass = 0; pass < passes; ++pass) {
    const int id = r->pretrain_passes++;
    FrameParams fp{r->mode, r->beta_knob - 1, id, id + 10007, 1, r->n_train, r->in_ch,
                   1, r->d_samples, r->n_samples, 0x9e37u + (uint32_t)id};
    if (r->log_ev && r->n_train <= r->P) {  // the log holds P paths
      fp.log = PathLog{r->log_ev, r->log_vcur, r->log_slots};
      cudaMemsetAsync(r->log_ev, 0xff, (size_t)r->P * r->log_slots * 3 * sizeof(float4), st);
    }
    int* q_cur = sl.q_a;
    int* q_next = sl.q_b;
    int* c_cur = sl.counts;
    int* c_next = sl.counts + 1;
    cudaMemsetAsync(sl.fetch, 0, r->fetch_slots * sizeof(int), st);
    const Batch nob{nullptr, nullptr, 0};
    if (int e = launch_camera(sd, fp, nob, sl.ps, q_cur, c_cur, st)) return e;
    for (int it = 0; it <= s->path_v2; ++it) {
      if (int e = launch_persistent<ExtendRays, false>(ExtendRays{sl.ps, q_cur, c_cur}, sd, nob, 0.f, 1e30f,
                                                       sl.fetch + 2 * it, sl.err, r->d_cnt, false,
                                                       r->blocks_extend, st))
        return e;
      if (int e = launch_shade(sd, fp, nob, sl.ps, sl.fb, q_cur, c_cur, sl.keep, grid, st)) return e;
      if (int e = launch_persistent<ShadowRays, true>(ShadowRays{sl.ps, q_cur, c_cur, sl.vis}, sd, nob, 0.f, 1e30f,
                                                      sl.fetch + 2 * it + 1, sl.err, r->d_cnt + 3, false,
                                                      r->blocks_shadow, st))
        return e;
      shadow_resolve_kernel<false><<<grid, 256, 0, st>>>(sl.ps, q_cur, c_cur, sl.vis, DiffParams{}, nullptr,
                                                         nullptr, fp.log);
      scan_count_kernel<<<std::min(nblocks, r->sm_count * 2), kScanBlock, 0, st>>>(sl.keep, c_cur, sl.block_sums,
                                                                                    nblocks);
      scan_blocks_kernel<<<1, 1024, 0, st>>>(sl.block_sums, c_cur, c_next);
      scatter_kernel<<<std::min(nblocks, r->sm_count * 2), kScanBlock, 0, st>>>(sl.keep, q_cur, c_cur,
                                                                                sl.block_sums, q_next, nblocks);
      HM_CHECK_LAUNCH("pretrain bounce");
      std::swap(q_cur, q_next);
      std::swap(c_cur, c_next);
    }
    if (int e = launch_finalize(sd, fp, nob, sl.ps, sl.fb, st)) return e;
    if (r->have_mlp_ev) cudaStreamWaitEvent(st, r->ev_mlp, 0);
    if (int e = hm_mlp_training_step(r->mlp, sl.fb.nn_train_in, sl.fb.nn_train_out, r->n_train, sl.d_loss, st))
      return e;
    cudaEventRecord(r->ev_mlp, st);
    r->have_mlp_ev = true;
  }
  cudaMemcpyAsync(sl.h_err, sl.err, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaEventRecord(sl.done, st);
  sl.in_flight = true;
  return slot_finish(r, sl);
}

extern "C" int hm_render_pretrain(hm_render* h, int passes, void* stream) {
  Render* r = (Render*)h;
  if (!r || passes < 0) return hm_set_error("hm_render_pretrain: bad arguments"), HM_EINVAL;
  if (passes == 0) return HM_OK;
  return render_pretrain(r, passes, (cudaStream_t)stream);
}

// ---- differentiable rendering: detached forward frames and path replay
// Buffers for `frames` frames with `groups` materials (grown on demand).
static int diff_setup(Render* r, int frames, int groups) {
  const int64_t P = r->P;
  const int rows = groups * kNd;
  cudaError_t e = cudaSuccess;
  if (frames > r->diff_cap_frames) {
    for (void* p : {(void*)r->diff_col, (void*)r->diff_in, (void*)r->diff_dy, (void*)r->diff_gframe}) cudaFree(p);
    r->diff_col = nullptr;
    r->diff_in = r->diff_dy = nullptr;
    r->diff_gframe = nullptr;
    r->diff_cap_frames = 0;
    e = cudaMalloc(&r->diff_col, (size_t)frames * P * sizeof(float4));
    if (e == cudaSuccess && r->mode == MODE_MSNN)
      e = cudaMalloc(&r->diff_in, (size_t)frames * P * r->in_ch * sizeof(float));
    if (e == cudaSuccess && r->mode == MODE_MSNN) e = cudaMalloc(&r->diff_dy, (size_t)frames * P * 3 * sizeof(float));
    if (e == cudaSuccess)
      e = cudaMalloc(&r->diff_gframe, (size_t)frames * kMaxStrandGroups * kNd * sizeof(double));
    if (e != cudaSuccess) return hm_cuda_status(e, "differentiable render buffers");
    r->diff_cap_frames = frames;
  }
  if (!r->diff_gsum) {
    if (e == cudaSuccess) e = r->alloc(&r->diff_gsum, kMaxStrandGroups * kNd);
    if (e == cudaSuccess) e = cudaMallocHost(&r->h_gsum, kMaxStrandGroups * kNd * sizeof(double));
    if (e == cudaSuccess) e = r->alloc((char**)&r->diff_dual, kMaxStrandGroups * group_dual_bytes());
    if (e == cudaSuccess) e = r->alloc(&r->diff_eval, kMaxStrandGroups);
    if (e != cudaSuccess) return hm_cuda_status(e, "differentiable render tables");
  }
  for (auto& sl : r->slots) {
    if (!sl.stash) {
      if (e == cudaSuccess) e = cudaMalloc(&sl.stash, (size_t)(2 * kNd + 1) * P * sizeof(float));
      if (e == cudaSuccess) e = cudaMalloc(&sl.partial, (size_t)kGradBlocks * kMaxStrandGroups * kNd * sizeof(double));
      if (e == cudaSuccess) e = cudaMalloc(&sl.ps.beta_d, (size_t)P * sizeof(float4));
    }
    if (e == cudaSuccess && sl.gacc_rows < rows) {
      cudaFree(sl.gacc);
      sl.gacc = nullptr;
      sl.gacc_rows = 0;
      e = cudaMalloc(&sl.gacc, (size_t)rows * P * sizeof(float));
      if (e == cudaSuccess) sl.gacc_rows = rows;
    }
    if (e != cudaSuccess) return hm_cuda_status(e, "replay slot buffers");
  }
  return HM_OK;
}

static int diff_forward(Render* r, int frames, const hm_hair_params* eval, int n_eval, cudaStream_t user) {
  if (!r->bscenes.empty()) return hm_set_error("hm_render_diff_forward: single-scene renders only"), HM_EUNSUPPORTED;
  if (r->mode == MODE_NRC) return hm_set_error("hm_render_diff_forward: HairMSNN and PT renders only"), HM_EUNSUPPORTED;
  if (frames < 1) return hm_set_error("hm_render_diff_forward: frames < 1"), HM_EINVAL;
  const int groups = r->scene->n_groups();
  if (eval && n_eval != groups)
    return hm_set_error("hm_render_diff_forward: %d evaluation materials for %d groups", n_eval, groups), HM_EINVAL;
  if (int e = render_sync(r)) return e;
  if (int e = diff_setup(r, frames, groups)) return e;
  if (eval) {
    std::vector<HairConsts> hc(groups);
    for (int g = 0; g < groups; ++g) hc[g] = hair_consts_from_params(eval[g]);
    cudaError_t e = cudaMemcpy(r->diff_eval, hc.data(), groups * sizeof(HairConsts), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return hm_cuda_status(e, "evaluation materials");
  }
  r->accum_id = 0;
  r->diff_frames = 0;
  r->diff_groups = groups;
  r->diff_material_version = r->scene->material_version;
  r->diff_detached = eval != nullptr;
  r->diff_fwd = true;
  int st = HM_OK;
  for (int f = 0; f < frames && st == HM_OK; ++f) st = render_frame(r, user, r->timing || r->counting);
  r->diff_fwd = false;
  if (st == HM_OK) r->diff_frames = frames;
  return st;
}

// Replays frame f of the last differentiable forward on its own slot.
static int replay_frame(Render* r, int f, const float* adjoint) {
  Scene* s = r->scene;
  const SceneDev sd = s->dev();
  Slot& sl = r->slots[f % r->depth];
  if (int e = slot_finish(r, sl)) return e;
  const cudaStream_t st = sl.st;
  FrameParams fp{r->mode, r->beta_knob - 1, f, f + 10007, r->every_nth, r->n_train, r->in_ch, 0, nullptr, 0, 0u};
  fp.no_train = 1;
  FrameBufs fb = sl.fb;
  if (r->mode == MODE_MSNN) fb.nn_frame_in = r->diff_in + (size_t)f * r->P * r->in_ch;
  const int rows = r->diff_groups * kNd;
  const DiffParams dp{r->diff_col + (size_t)f * r->P, adjoint, 1.f / (float)r->diff_frames, sl.gacc, sl.stash,
                      (const HairConstsD*)r->diff_dual, r->P};
  cudaMemsetAsync(sl.gacc, 0, (size_t)rows * r->P * sizeof(float), st);
  cudaMemsetAsync(sl.fetch, 0, r->fetch_slots * sizeof(int), st);
  int* q_cur = sl.q_a;
  int* q_next = sl.q_b;
  int* c_cur = sl.counts;
  int* c_next = sl.counts + 1;
  if (int e = launch_camera(sd, fp, r->batch, sl.ps, q_cur, c_cur, st)) return e;
  const int grid = r->sm_count * r->shade_blocks_per_sm;
  const int nblocks = (r->P + kScanBlock - 1) / kScanBlock;
  const int rounds = bounce_rounds(r, fp);
  for (int it = 0; it < rounds; ++it) {
    if (int e = launch_persistent<ExtendRays, false>(ExtendRays{sl.ps, q_cur, c_cur}, sd, r->batch, 0.f, 1e30f,
                                                     sl.fetch + 2 * it, sl.err, r->d_cnt, false, r->blocks_extend,
                                                     st))
      return e;
    if (int e = launch_shade(sd, fp, r->batch, sl.ps, fb, q_cur, c_cur, sl.keep, grid, st, &dp)) return e;
    if (int e = launch_persistent<ShadowRays, true>(ShadowRays{sl.ps, q_cur, c_cur, sl.vis}, sd, r->batch, 0.f, 1e30f,
                                                    sl.fetch + 2 * it + 1, sl.err, r->d_cnt + 3, false,
                                                    r->blocks_shadow, st))
      return e;
    shadow_resolve_kernel<true><<<grid, 256, 0, st>>>(sl.ps, q_cur, c_cur, sl.vis, dp);
    scan_count_kernel<<<std::min(nblocks, r->sm_count * 2), kScanBlock, 0, st>>>(sl.keep, c_cur, sl.block_sums,
                                                                                  nblocks);
    scan_blocks_kernel<<<1, 1024, 0, st>>>(sl.block_sums, c_cur, c_next);
    scatter_kernel<<<std::min(nblocks, r->sm_count * 2), kScanBlock, 0, st>>>(sl.keep, q_cur, c_cur, sl.block_sums,
                                                                              q_next, nblocks);
    HM_CHECK_LAUNCH("replay bounce");
    std::swap(q_cur, q_next);
    std::swap(c_cur, c_next);
  }
  if (r->mode == MODE_MSNN)
    if (int e = launch_replay_cache_grad(r->P, sl.ps, dp, r->diff_dy + (size_t)f * r->P * 3, st)) return e;
  grad_block_sum_kernel<<<kGradBlocks, 256, 0, st>>>(sl.gacc, r->P, rows, sl.partial);
  grad_parts_sum_kernel<<<1, 384, 0, st>>>(sl.partial, kGradBlocks, rows, r->diff_gframe + (size_t)f * rows);
  HM_CHECK_LAUNCH("replay gradient sums");
  cudaMemcpyAsync(sl.h_err, sl.err, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaEventRecord(sl.done, st);
  sl.in_flight = true;
  return HM_OK;
}

static int diff_backward(Render* r, const float* adjoint, double* host_grad, int n_grad, cudaStream_t user) {
  if (r->diff_frames <= 0) return hm_set_error("hm_render_diff_backward: no differentiable forward to replay"), HM_EINVAL;
  if (r->diff_detached)
    return hm_set_error("hm_render_diff_backward: the last forward was detached (evaluation materials)"), HM_EINVAL;
  if (r->scene->n_groups() != r->diff_groups || r->scene->material_version != r->diff_material_version)
    return hm_set_error("hm_render_diff_backward: the scene's materials changed since the forward"), HM_EINVAL;
  if (r->accum_id != r->diff_frames)
    return hm_set_error("hm_render_diff_backward: frames were rendered after the differentiable forward"), HM_EINVAL;
  const int rows = r->diff_groups * kNd;
  if (n_grad < rows) return hm_set_error("hm_render_diff_backward: %d gradient slots for %d", n_grad, rows), HM_ECAPACITY;
  if (int e = render_sync(r)) return e;
  const cudaStream_t st0 = r->slots[0].st;
  cudaEventRecord(r->ev_submit, user);
  for (auto& sl : r->slots) cudaStreamWaitEvent(sl.st, r->ev_submit, 0);
  if (int e = launch_group_dual(r->scene->dev(), r->diff_dual, r->diff_groups, st0)) return e;
  cudaEventRecord(r->ev_mlp, st0);
  for (auto& sl : r->slots) cudaStreamWaitEvent(sl.st, r->ev_mlp, 0);
  for (int f = 0; f < r->diff_frames; ++f)
    if (int e = replay_frame(r, f, adjoint)) return e;
  if (int e = render_sync(r)) return e;
  grad_parts_sum_kernel<<<1, 384, 0, st0>>>(r->diff_gframe, r->diff_frames, rows, r->diff_gsum);
  HM_CHECK_LAUNCH("replay gradient total");
  if (r->mode == MODE_MSNN) {
    // dL/dW: the cache's backward over every replayed frame's queries at once
    const int64_t n = (int64_t)r->diff_frames * r->P;
    if (int e = hm_mlp_forward(r->mlp, r->diff_in, nullptr, n, st0)) return e;
    if (int e = hm_mlp_backward_output_grad(r->mlp, r->diff_dy, n, st0)) return e;
  }
  cudaError_t e = cudaMemcpyAsync(r->h_gsum, r->diff_gsum, rows * sizeof(double), cudaMemcpyDeviceToHost, st0);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st0);
  if (e != cudaSuccess) return hm_cuda_status(e, "hm_render_diff_backward");
  memcpy(host_grad, r->h_gsum, rows * sizeof(double));
  cudaEventRecord(r->ev_submit, st0);
  cudaStreamWaitEvent((cudaStream_t)user, r->ev_submit, 0);
  return HM_OK;
}

extern "C" int hm_render_diff_forward(hm_render* h, int frames, const hm_hair_params* eval_materials, int n_materials,
                                      void* stream) {
  Render* r = (Render*)h;
  if (!r) return hm_set_error("hm_render_diff_forward: NULL"), HM_EINVAL;
  return diff_forward(r, frames, eval_materials, n_materials, (cudaStream_t)stream);
}

extern "C" int hm_render_diff_backward(hm_render* h, const float* d_adjoint, double* host_grad, int n_grad,
                                       void* stream) {
  Render* r = (Render*)h;
  if (!r || !d_adjoint || !host_grad) return hm_set_error("hm_render_diff_backward: NULL"), HM_EINVAL;
  return diff_backward(r, d_adjoint, host_grad, n_grad, (cudaStream_t)stream);
}

extern "C" int hm_render_reset(hm_render* h) {
  Render* r = (Render*)h;
  if (!r) return HM_EINVAL;
  int st = render_sync(r);
  r->accum_id = 0;
  return st;
}

extern "C" int hm_render_read(hm_render* h, int which, double* host_rgb) {
  Render* r = (Render*)h;
  if (!r || !host_rgb) return hm_set_error("hm_render_read: NULL"), HM_EINVAL;
  if (int st = render_sync(r)) return st;
  const double* src = which == HM_IMAGE_FINAL ? r->acc_final
                      : which == HM_IMAGE_SHORT ? r->acc_pt
                      : which == HM_IMAGE_CACHE ? r->acc_nn : nullptr;
  if (!src) return hm_set_error("hm_render_read: unknown image %d", which), HM_EINVAL;
  if (r->mode != MODE_MSNN && which != HM_IMAGE_FINAL)
    return hm_set_error("hm_render_read: PT and NRC renders have only the final image"), HM_EINVAL;
  const size_t n = (size_t)r->P * 3;
  cudaError_t e = cudaMemcpy(host_rgb, src, n * sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return hm_cuda_status(e, "hm_render_read");
  const double inv = r->accum_id > 0 ? 1.0 / r->accum_id : 0.0;
  for (size_t i = 0; i < n; ++i) host_rgb[i] *= inv;
  return HM_OK;
}

extern "C" int hm_render_get_stats(const hm_render* h, hm_render_stats* out) {
  Render* r = const_cast<Render*>((const Render*)h);
  if (!r || !out) return HM_EINVAL;
  int st = render_sync(r);
  out->frames = r->accum_id;
  out->pixels = r->P;
  out->extension_rays = r->rays_extend;
  out->last_bounces = r->last_bounces;
  out->train_records = r->mode == MODE_MSNN ? r->n_train : (r->mode == MODE_NRC ? r->nrc_records : 0);
  out->every_nth = r->every_nth;
  float loss = 0.f;
  if (r->mlp && r->train && r->accum_id > 0)
    cudaMemcpy(&loss, r->slots[(r->accum_id - 1) % r->depth].d_loss, sizeof(float), cudaMemcpyDeviceToHost);
  out->last_loss = loss;
  return st;
}

extern "C" int hm_render_set_instrumentation(hm_render* h, int timing, int counting) {
  Render* r = (Render*)h;
  if (!r) return HM_EINVAL;
  r->timing = timing != 0;
  r->counting = counting != 0;
  return HM_OK;
}

extern "C" int hm_queue_compact(const int32_t* d_keep, const int32_t* d_queue, int64_t n, int32_t* d_out,
                                int64_t* out_count, void* stream) {
  if (n < 0 || n > (int64_t)1 << 30 || (n > 0 && (!d_keep || !d_queue || !d_out)) || !out_count)
    return hm_set_error("hm_queue_compact: bad arguments"), HM_EINVAL;
  *out_count = 0;
  if (n == 0) return HM_OK;
  const cudaStream_t st = (cudaStream_t)stream;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int nblocks = (int)((n + kScanBlock - 1) / kScanBlock);
  int* buf = nullptr;  // [0] count in, [1] count out, [2..] block sums
  cudaError_t e = cudaMalloc(&buf, (size_t)(nblocks + 3) * sizeof(int));
  if (e != cudaSuccess) return hm_cuda_status(e, "hm_queue_compact");
  const int nn = (int)n;
  cudaMemcpyAsync(buf, &nn, sizeof(int), cudaMemcpyHostToDevice, st);
  // the launches of a bounce round's compaction (render_frame)
  scan_count_kernel<<<std::min(nblocks, sms * 2), kScanBlock, 0, st>>>(d_keep, buf, buf + 2, nblocks);
  scan_blocks_kernel<<<1, 1024, 0, st>>>(buf + 2, buf, buf + 1);
  scatter_kernel<<<std::min(nblocks, sms * 2), kScanBlock, 0, st>>>(d_keep, d_queue, buf, buf + 2, d_out, nblocks);
  e = cudaGetLastError();
  int out = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&out, buf + 1, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(buf);
  if (e != cudaSuccess) return hm_cuda_status(e, "hm_queue_compact");
  *out_count = out;
  return HM_OK;
}

extern "C" int hm_render_set_path_log(hm_render* h, int vertices) {
  if (!h || vertices < 0 || vertices > 4096) return hm_set_error("hm_render_set_path_log: bad arguments"), HM_EINVAL;
  Render* r = (Render*)h;
  if (vertices > 0 && (r->depth != 1 || !r->bscenes.empty()))
    return hm_set_error("hm_render_set_path_log: single-scene renderers with one frame in flight"), HM_EINVAL;
  if (int e = render_sync(r)) return e;
  cudaFree(r->log_ev);
  cudaFree(r->log_vcur);
  r->log_ev = nullptr;
  r->log_vcur = nullptr;
  r->log_slots = 0;
  if (vertices == 0) return HM_OK;
  const int slots = 3 * vertices;
  cudaError_t e = cudaMalloc(&r->log_ev, (size_t)r->P * slots * 3 * sizeof(float4));
  if (e == cudaSuccess) e = cudaMalloc(&r->log_vcur, (size_t)r->P * sizeof(int));
  if (e != cudaSuccess) {
    cudaFree(r->log_ev);
    r->log_ev = nullptr;
    return hm_cuda_status(e, "hm_render_set_path_log");
  }
  r->log_slots = slots;
  return HM_OK;
}

extern "C" int hm_render_read_path_log(hm_render* h, float* host_dst, int64_t n_floats) {
  if (!h || !host_dst) return hm_set_error("hm_render_read_path_log: bad arguments"), HM_EINVAL;
  Render* r = (Render*)h;
  const int64_t need = (int64_t)r->P * r->log_slots * 12;
  if (!r->log_ev || n_floats < need)
    return hm_set_error("hm_render_read_path_log: no log, or %lld floats needed", (long long)need), HM_EINVAL;
  if (int e = render_sync(r)) return e;
  cudaError_t e = cudaMemcpy(host_dst, r->log_ev, need * sizeof(float), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? HM_OK : hm_cuda_status(e, "hm_render_read_path_log");
}

extern "C" int hm_render_get_timings(const hm_render* h, hm_render_timings* out) {
  const Render* r = (const Render*)h;
  if (!r || !out) return HM_EINVAL;
  *out = r->tm;
  return HM_OK;
}

extern "C" hm_mlp* hm_render_cache(hm_render* h) {
  Render* r = (Render*)h;
  return r ? r->mlp : nullptr;
}

// Cache input / target buffers of the last frame (device pointers, valid
// until the next frame): which 0 = frame inputs [P][12], 1 = frame outputs
// [P][3], 2 = training inputs [R][12], 3 = training targets [R][3],
// 4 = G-buffer [P] float4.
extern "C" int hm_render_buffer(hm_render* h, int which, void** dptr, int64_t* count) {
  Render* r = (Render*)h;
  if (!r || !dptr) return HM_EINVAL;
  if (int st = render_sync(r)) return st;
  const FrameBufs& fb = r->slots[r->accum_id > 0 ? (r->accum_id - 1) % r->depth : 0].fb;
  switch (which) {
    case 0: *dptr = fb.nn_frame_in; if (count) *count = (int64_t)r->nn_rows * r->in_ch; break;
    case 1: *dptr = fb.nn_frame_out; if (count) *count = (int64_t)r->nn_rows * 3; break;
    case 2: *dptr = fb.nn_train_in;
      if (count) *count = (int64_t)(r->mode == MODE_NRC ? r->nrc_records : r->n_train) * r->in_ch;
      break;
    case 3: *dptr = fb.nn_train_out;
      if (count) *count = (int64_t)(r->mode == MODE_NRC ? r->nrc_records : r->n_train) * 3;
      break;
    case 4: *dptr = fb.gbuf; if (count) *count = (int64_t)r->P; break;
    case 5: *dptr = r->acc_final; if (count) *count = (int64_t)r->P * 3; break;
    case 6: *dptr = r->acc_pt; if (count) *count = (int64_t)r->P * 3; break;
    case 7: *dptr = r->acc_nn; if (count) *count = (int64_t)r->P * 3; break;
    case 11:
      if (!r->d_samples) return hm_set_error("hm_render_buffer: no scene samples before hm_render_pretrain"), HM_EINVAL;
      *dptr = r->d_samples;
      if (count) *count = (int64_t)r->n_samples;
      break;
    case 8: case 9: case 10: {
      if (r->mode != MODE_NRC) return hm_set_error("hm_render_buffer: NRC buffers of a non-NRC renderer"), HM_EINVAL;
      const NrcBufs& nb = r->slots[r->accum_id > 0 ? (r->accum_id - 1) % r->depth : 0].nrc;
      if (which == 8) { *dptr = nb.gbeta; if (count) *count = (int64_t)r->P; }
      if (which == 9) { *dptr = nb.rec; if (count) *count = (int64_t)r->n_train * kNrcMaxBounces * kNrcRecordF4; }
      if (which == 10) { *dptr = nb.tinfo; if (count) *count = (int64_t)r->n_train; }
      break;
    }
    default: return HM_EINVAL;
  }
  return HM_OK;
}

extern "C" int hm_trace_rays(const hm_scene* h, const float* d_org, const float* d_dir, int64_t n, float tmin,
                             float tmax, int any_hit, float* d_hits, void* stream) {
  Scene* s = const_cast<Scene*>((const Scene*)h);  // the device build is a lazily made cache
  if (!s || n < 0 || (n > 0 && (!d_org || !d_dir || !d_hits))) return hm_set_error("hm_trace_rays: bad args"), HM_EINVAL;
  if (n == 0) return HM_OK;
  if (int st = s->ensure_built()) return st;
  if (n > INT32_MAX) return hm_set_error("hm_trace_rays: at most 2^31-1 rays per call"), HM_ECAPACITY;
  int* err = nullptr;  // [0] error bits, [1] ray-fetch counter
  cudaError_t e = cudaMalloc(&err, 2 * sizeof(int));
  if (e != cudaSuccess) return hm_cuda_status(e, "hm_trace_rays");
  cudaMemsetAsync(err, 0, 2 * sizeof(int), (cudaStream_t)stream);
  BatchRays src{d_org, d_dir, n, tmin, tmax, (float4*)d_hits};
  const Batch nob{nullptr, nullptr, 0};
  int st = any_hit ? launch_persistent<BatchRays, true>(src, s->dev(), nob, tmin, tmax, err + 1, err, nullptr, false,
                                                        persistent_blocks<BatchRays, true>(), (cudaStream_t)stream)
                   : launch_persistent<BatchRays, false>(src, s->dev(), nob, tmin, tmax, err + 1, err, nullptr, false,
                                                         persistent_blocks<BatchRays, false>(), (cudaStream_t)stream);
  if (st != HM_OK) {
    cudaFree(err);
    return st;
  }
  int herr = 0;
  e = cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
  cudaFree(err);
  if (e != cudaSuccess) return hm_cuda_status(e, "hm_trace_rays");
  if (herr) return hm_set_error("traversal gave up on some rays (error bits 0x%x)", herr), HM_ECAPACITY;
  return HM_OK;
}
