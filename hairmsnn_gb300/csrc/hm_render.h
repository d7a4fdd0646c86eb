// Wavefront integrator state shared by the shading (hm_shade.cu) and tracing
// (hm_render.cu) translation units.
#pragma once
#include "hm_scene.h"

namespace hm {

enum PathFlags : uint32_t {
  F_TRAIN = 1u,     // pixel produces a training record this frame
  F_DL = 2u,        // shadow rays of the current vertex are pending
  F_PRIM_HIT = 4u,  // primary ray hit something
  F_PRIM_SURF = 8u, // ... and it was the head surface
  // NRC (nrc.cu:136-310)
  F_NRC_SUFFIX = 16u,    // a training pixel past its cache query (isTrainingSuffix)
  F_NRC_UNBIASED = 32u,  // training pixel traced to the end (every 16th)
  F_NRC_RECALC = 64u,    // a0 of the suffix is taken at the next vertex
  F_NRC_NOSPREAD = 128u, // unbiased suffix past its cache query: no spread test (c = 1e30)
  F_NRC_GSNAP = 256u     // the G-buffer was written when the path took the cache
};

enum RenderMode { MODE_PT = 0, MODE_MSNN = 1, MODE_NRC = 2 };

// NRC buffers of one frame slot.
constexpr int kNrcMaxBounces = 40;  // MAX_BOUNCES (nrc.cuh:13)
constexpr int kNrcRecordF4 = 5;     // per vertex: position / scale, wo, n, direct light, throughput factor
// width of the scene-sample pass's launch grid (numTrainRecordsX,
// render_hair_msnn.h:127): record r is launch index (r % 128, r / 128)
constexpr int kTrainRecordsX = 128;
struct NrcBufs {
  float4* prev;    // [P] previous vertex and the pdf of the direction sampled there
  float4* spread;  // [P] accumulated spread, a0
  float4* gbeta;   // [P] throughput at the cache query (0: no query)
  int* dl_rec;     // [P] train record of the pending direct light (-1: none)
  float4* rec;     // [R][40][5] train buffer (TrainBuffer, nrc.cuh:29-40)
  int4* tinfo;     // [R] bounces, suffix ended at a cache query, unbiased, primary hit
  float c;         // spread threshold multiplier (render_nrc.h:132)
  int all_unbiased;
};

// Structure-of-arrays path state, one slot per pixel (capacity W*H).
struct PathState {
  uint32_t* rng;
  uint32_t* flags;
  int* bounce;
  float4* ray_o;  // extension ray origin (w unused)
  float4* ray_d;  // extension ray direction
  float4* hit;    // t, prim (int bits, -1 miss), u, v
  float4* beta;   // path throughput
  float4* beta_s; // short-path throughput (training pixels)
  float4* col;    // path radiance (miss: emitted radiance of the primary ray)
  float4* col_s;  // short-path radiance (training pixels)
  float4* sh_o0;  // shadow ray 0 origin, w = 1 if valid
  float4* sh_d0;
  float4* sh_o1;  // shadow ray 1
  float4* sh_d1;
  float4* sh_c0;  // contributions if unoccluded
  float4* sh_c1;
  float4* dl_w;   // weight of the visible direct-lighting sum in col
  float4* dl_ws;  // ... in col_s
  float4* beta_d; // detached renders: throughput of the sampling material (Russian roulette)
};

// Per-path ray log (hm_render_set_path_log; ev == nullptr in ordinary
// frames).  Slot 3k + j of a path holds vertex k's extension-ray result
// (j = 0: the ray that found the vertex), its light-sample shadow ray (1) and
// its BSDF-sample shadow ray (2), three float4 each:
//   (result int bits, t, u, RNG state bits), (direction, kind int bits),
//   (origin, 0)
// with result = hit primitive or -1 (extension), 1 unoccluded / 0 occluded
// (shadow); kind -1 marks an empty slot.
struct PathLog {
  float4* ev;  // [P][slots][3]
  int* vcur;   // [P] vertex of the pending shadow rays
  int slots;
};
constexpr int kLogPending = -2;  // a logged shadow ray not resolved yet

HM_D void log_ray(const PathLog& L, int pid, int slot, int kind, int result, float t, float u, uint32_t rng,
                  f3 o, f3 d) {
  if (slot >= L.slots) return;
  float4* e = L.ev + ((size_t)pid * L.slots + slot) * 3;
  e[0] = make_float4(__int_as_float(result), t, u, __uint_as_float(rng));
  e[1] = make_float4(d.x, d.y, d.z, __int_as_float(kind));
  e[2] = make_float4(o.x, o.y, o.z, 0.f);
}

struct FrameParams {
  int mode;        // RenderMode
  int beta;        // BETA - 1 (render_hair_msnn.cu:1170)
  int accum_id;    // frames accumulated so far
  int frame_seed;  // accum_id + 10007 (hair_msnn.cu:194)
  int every_nth;   // one training pixel per every_nth pixels
  int n_train;     // training records per frame
  int in_ch;       // cache input channels (12)
  // scene-sample training pass (TRAIN_DATA_GEN, hair_msnn.cu:222-233): the
  // paths are n_train camera rays towards points sampled on the hair, all
  // training paths; 0 for ordinary frames
  int pretrain;
  const float4* samples;  // points on the hair curves (xyz)
  int n_samples;
  uint32_t sample_key;    // permutation of the samples for this pass
  // differentiable renders: no training pixels (every pixel a short path +
  // cache query), and, for a detached render, the materials (one per strand
  // group) of the hair BSDF values; sampling, pdfs, MIS weights and Russian
  // roulette keep the scene's materials
  int no_train;
  const HairConsts* eval_hc;
  // frames replayed from a CUDA graph read the frame number (accum_id) here
  const int* d_frame;
  PathLog log;
};

// Path replay (Vicini et al. 2021, "Path Replay Backpropagation"): a frame
// of a differentiable render re-traced with the same random numbers, every
// hair vertex adding adjoint-weighted material derivatives of the path's
// radiance; the radiance still to come after a vertex is the path's total
// (kept from its forward frame) minus what the replay has gathered so far.
struct HairConstsD;
struct DiffParams {
  const float4* col_total;       // [P] radiance of each path in the forward frame
  const float* adjoint;          // [P][3] dLoss/dImage
  float adj_scale;               // 1 / frames (the image is their mean)
  float* gacc;                   // [n_groups * 6][P] per-path gradient sums
  float* stash;                  // [13][P] gradient terms waiting for shadow rays; [12]: group
  const HairConstsD* group_dual; // [n_groups] materials with their partials
  int P;
};

// Several scenes in one frame (a batch): the frame's paths, training
// records and accumulators are the scenes' ranges one after another, and
// every path knows its scene.  Single-scene frames pass scenes == nullptr.
struct BatchScene {
  SceneDev s;
  int pix_off, n_pix;                 // paths [pix_off, pix_off + n_pix)
  int train_off, n_train, every_nth;  // training records of this scene
  int beta;                           // BETA - 1
};
struct Batch {
  const BatchScene* scenes;  // device array
  const int* path_scene;     // scene of every path
  int n_paths;
};

// The scene and the per-scene knobs of one path.
struct PathCtx {
  const SceneDev* s;
  int local;       // pixel index inside its scene
  int train_base;  // first training record of its scene
  int every_nth, n_train, beta;
};
template <bool MULTI>
HM_D PathCtx path_ctx(const SceneDev& s, const FrameParams& fp, const Batch& b, int pid) {
  if (!MULTI) return PathCtx{&s, pid, 0, fp.every_nth, fp.n_train, fp.beta};
  const BatchScene& bs = b.scenes[b.path_scene[pid]];
  return PathCtx{&bs.s, pid - bs.pix_off, bs.train_off, bs.every_nth, bs.n_train, bs.beta};
}

struct FrameBufs {
  float* nn_frame_in;   // [P][in_ch]
  float* nn_frame_out;  // [P][3]
  float* nn_train_in;   // [R][in_ch]
  float* nn_train_out;  // [R][3]
  float4* gbuf;         // path colour; w = 1 hit, 2 surface (bit flags as float)
  double* acc_pt;       // [P][3] running sums (FP64)
  double* acc_nn;
  double* acc_final;
  float4* col_out;      // differentiable renders: each path's radiance (NULL otherwise)
};

// Training-pixel choice: the reference shuffles a table of 0..R-1 each frame
// with thrust::shuffle and keeps pixel fbOfs % everyNth == trainIdxs[trOfs] %
// everyNth.  Here the permutation is a keyed Feistel bijection on [0, R)
// (cycle-walking for non-powers of two), deterministic per frame.
HM_HD uint32_t feistel_perm(uint32_t i, uint32_t n, uint32_t key) {
  uint32_t bits = 1;
  while ((1u << bits) < n) ++bits;
  const uint32_t half = (bits + 1) / 2, lo_mask = (1u << half) - 1u;
  uint32_t x = i;
  for (int walk = 0; walk < 64; ++walk) {
    uint32_t l = x >> half, r = x & lo_mask;
    for (int round = 0; round < 4; ++round) {
      uint32_t f = murmur_finalize(r ^ (key + 0x9e3779b9u * (uint32_t)(round + 1))) & lo_mask;
      uint32_t nl = r;
      r = (l ^ f) & lo_mask;
      l = nl;
    }
    x = ((l << half) | r) & ((1u << (2 * half)) - 1u);
    if (x < n) return x;
  }
  return i % n;
}

}  // namespace hm
