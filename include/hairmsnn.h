/* HairMSNN per-path-vertex hot path on GB300 (sm_103a) — C ABI.
 *
 * Plain C: pointers, sizes and status codes only.  Device pointers are CUDA
 * global-memory addresses on the current device; `stream` is a cudaStream_t
 * passed as void* (NULL = the legacy default stream).  Every entry point
 * returns an hm_status; hm_last_error() gives the message of the last failure
 * on the calling thread.  No C++ exception crosses this boundary.
 *
 * Each declaration names the reference interface it replaces
 * (facebookresearch/HairMSNN, paths relative to the repository root).
 */
#ifndef HAIRMSNN_H_
#define HAIRMSNN_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum hm_status {
  HM_OK = 0,
  HM_EINVAL = 1,       /* bad argument (NULL pointer, negative size, bad value) */
  HM_ECUDA = 2,        /* a CUDA runtime call or kernel launch failed */
  HM_ECAPACITY = 3,    /* a fixed-capacity buffer or queue would overflow */
  HM_ETIMEOUT = 4,     /* a bounded device-side wait gave up */
  HM_ENOMEM = 5,       /* device or host allocation failed */
  HM_EPARSE = 6,       /* malformed JSON / config */
  HM_EUNSUPPORTED = 7  /* valid request that this build does not implement */
} hm_status;

const char* hm_status_string(int status);
const char* hm_last_error(void);
/* Library version string and the CUDA arch it was compiled for ("sm_103a"). */
const char* hm_version(void);
/* Synchronous device -> host copy helper for callers without a CUDA runtime
 * binding of their own (no reference counterpart). */
int hm_copy_to_host(void* host_dst, const void* device_src, int64_t bytes);

/* ------------------------------------------------------------------------
 * Hair material.  Replaces the hair block of the scene JSON as parsed by
 * parseScene (scene.cpp:184-231) and the per-hit copy in hairCH
 * (cuda_headers/optix_common.cuh:585-593).  alpha is in RADIANS (the JSON
 * key is in degrees; scene.cpp:207 converts with 3.14159 * deg / 180).
 * ---------------------------------------------------------------------- */
typedef struct hm_hair_params {
  float sigma_a[3];
  float beta_m, beta_n;
  float alpha;
  float gain_r, gain_tt, gain_trt, gain_trrt;
} hm_hair_params;

/* setupHairShading (cuda_headers/disney_hair.cuh:26-41) evaluated on the
 * host: out10 = v[3], s, sin2kAlpha[3], cos2kAlpha[3]. */
int hm_hair_setup(const hm_hair_params* params, float* out10);

/* ------------------------------------------------------------------------
 * Batched hair BSDF.  Replaces the device functions
 *   vec3f disney_hair(Interaction si, float* pdf)          disney_hair.cuh:186
 *   vec3f sample_disney_hair(Interaction& si, vec4f& rand,
 *                            float* pdf)                    disney_hair.cuh:277
 * for a batch of n hair vertices.  All arrays are device pointers in planar
 * layout: a vector array is [3][n] (all x, then all y, then all z).
 *   wo, wi   world-space unit directions (wo points away from the fibre)
 *   tangent  world-space unit fibre tangent (the frame's X axis)
 *   h        dot(Y, n) in [-1, 1] (the reference derives it from the hit)
 *   u        [4][n] uniforms for sampling (the reference's vec4f rand)
 * The shading frame is the reference's: X = tangent, Y = normalize(wo x X),
 * Z = X x Y (optix_common.cuh:571-583).  Outputs: f = f(wo,wi)*cos [3][n]
 * and the 4-lobe mixture pdf [n]; sampling also writes the world-space wi.
 * ---------------------------------------------------------------------- */
typedef struct hm_bsdf_queries {
  const float* wo;
  const float* wi; /* eval only; may be NULL for sampling */
  const float* tangent;
  const float* h;
  const float* u; /* sampling only; may be NULL for eval */
} hm_bsdf_queries;

int hm_bsdf_eval(const hm_bsdf_queries* q, float* f, float* pdf, int64_t n,
                 const hm_hair_params* params, void* stream);
int hm_bsdf_sample(const hm_bsdf_queries* q, float* wi_out, float* f, float* pdf, int64_t n,
                   const hm_hair_params* params, void* stream);
/* disney_hair (disney_hair.cuh:186) with its derivatives with respect to the
 * material, for appearance fitting (no reference counterpart: the
 * reference does not differentiate).  Parameters in this order: sigma_a r,
 * g, b, beta_m, beta_n, alpha (radians).  f [3][n] and pdf [n] as
 * hm_bsdf_eval; df [6][3][n] = d f[c] / d param[j] at df[(j*3 + c)*n + i];
 * dpdf [6][n] (may be NULL).  Forward-mode (dual-number) evaluation. */
int hm_bsdf_eval_grad(const hm_bsdf_queries* q, float* f, float* pdf, float* df, float* dpdf, int64_t n,
                      const hm_hair_params* params, void* stream);

/* Synthetic BSDF workload generator (no reference counterpart: the
 * benchmark's input).  Per query one murmur-seeded LCG stream (the
 * reference's random.cuh:58-65 with pixel index = query index): wo, wi,
 * tangent uniform on the sphere, h uniform in [-1,1), u uniform.  wi and u
 * may be NULL. */
int hm_bsdf_gen_queries(uint32_t seed, int64_t n, float* wo, float* wi, float* tangent, float* h,
                        float* u, void* stream);

/* ------------------------------------------------------------------------
 * Radiance-cache network.  Replaces TINY_MLP (cuda_headers/neural_network.cuh
 * :33-50, cuda/neural_network.cu:17-64) and the tiny-cuda-nn Trainer calls
 * of the frame driver (render_hair_msnn.cu:683-691).
 *   config_json  tiny-cuda-nn style JSON TEXT with "loss", "optimizer",
 *                "encoding", "network" (the reference passes a file path to
 *                TINY_MLP; read the file and pass its contents)
 *   in_ch/out_ch input / output channels (the reference uses 12 / 3,
 *                headers/render_hair_msnn.h:145)
 *   precision    HM_PREC_*; seed: parameter initialisation stream.
 *                FP16 / BF16 / FP8_E4M3 run inference and training on the
 *                tensor cores (operands rounded to that type, FP32
 *                accumulation; E4M3 with per-layer weight scales and
 *                per-query activation scales, its training backward on
 *                FP16 operands); FP16 and E4M3 training use a static loss
 *                scale of 128, divided out before the optimizer and by
 *                hm_mlp_get_gradients.  Parameters and optimizer state
 *                stay FP32.
 * Device buffers are row-major per query: in [n][in_ch], out [n][out_ch]
 * (tiny-cuda-nn's column-major GPUMatrix(ptr, ch, n)).  Any n >= 0 is
 * accepted (the reference needs n % 128 == 0, scene.cpp:300-306).  The
 * handle owns parameters, optimizer state and workspace; one handle per
 * stream at a time.
 * ---------------------------------------------------------------------- */
typedef enum hm_precision {
  HM_PREC_FP32 = 0,
  HM_PREC_FP16 = 1,
  HM_PREC_BF16 = 2,
  HM_PREC_FP8_E4M3 = 3
} hm_precision;

typedef struct hm_mlp hm_mlp;

typedef struct hm_mlp_desc {
  int in_ch, out_ch;
  int encoded_width;        /* encoding output before padding */
  int padded_input_width;   /* network input width (multiple of 16) */
  int width;                /* n_neurons */
  int n_hidden_layers;
  int padded_output_width;  /* 16 */
  int64_t n_params;         /* network + encoding parameters */
  int64_t n_network_params; /* weight matrices (first in the parameter vector) */
  int precision;
  int step;                 /* optimizer steps taken */
  float learning_rate;      /* current (decayed) base learning rate */
} hm_mlp_desc;

/* TINY_MLP::TINY_MLP(configPath, inputCh, outputCh), neural_network.cu:34-56 */
hm_mlp* hm_mlp_create(const char* config_json, int in_ch, int out_ch, int precision, uint32_t seed,
                      int* status);
void hm_mlp_destroy(hm_mlp* mlp);
int hm_mlp_info(const hm_mlp* mlp, hm_mlp_desc* out);
/* Parses a config without touching the device (sizes or HM_EPARSE). */
int hm_mlp_describe_config(const char* config_json, int in_ch, int out_ch, hm_mlp_desc* out);
/* TINY_MLP::inference(in, out, size), neural_network.cu:58-64 */
int hm_mlp_inference(hm_mlp* mlp, const float* d_in, float* d_out, int64_t n, void* stream);
/* No counterpart in the reference.  hm_mlp_inference without any device
 * allocation, for callers that must not allocate once running: the encoded
 * inputs go to one static 4 MiB device scratch per device (n * padded input
 * width <= 2^20 floats, else HM_ECAPACITY; FP16/BF16/E4M3 handles encode
 * inside the tensor-core kernel and use no scratch).  Calls on one device must not
 * overlap (they share the scratch); make the first call on each device before
 * any stream capture (it resolves the scratch address).  The address is kept
 * for the life of the process: resetting a device (cudaDeviceReset, or any
 * other end of its primary context) while the library is loaded is not
 * supported by this entry point. */
int hm_mlp_inference_noalloc(hm_mlp* mlp, const float* d_in, float* d_out, int64_t n, void* stream);
/* The bounded device-side wait, run out on purpose (no reference
 * counterpart; failure-detection tests).  Every wait of the tensor-core
 * kernels on an mbarrier gives up after a fixed number of tries, records
 * the fact in a host-visible flag and lets the kernel return, so that a
 * lost completion shows as HM_ETIMEOUT instead of a hung GPU.  This call
 * launches one block that waits `tries` times (1 .. 2^20) on a barrier
 * nothing completes: it returns HM_ETIMEOUT when the wait expired and the
 * kernel returned, and the context stays usable. */
int hm_debug_wait_expiry(int tries, void* stream);
/* Form of the later FP16 / BF16 tensor-core inferences (no reference
 * counterpart; tests and timing).  Three forms give the same bits: the
 * warp-specialised kernel (encoder warps and layer warps overlapped in one
 * CTA per SM, no workspace; width 32 or 64, where the weights, two or six
 * layer-0 operand stages and two hidden operands fit in shared memory), the
 * encode kernel followed by the layer kernel (a workspace of encoded
 * operands), and the layer kernel encoding its own tiles.  0 (the default):
 * the warp-specialised kernel where it fits, except that an inference with
 * a workspace on a network whose encoding holds a hash grid takes the
 * encode kernel + layer kernel (faster for latency-bound table gathers).
 * 1: never the warp-specialised kernel.  2: only it
 * (HM_EUNSUPPORTED where it does not fit, and for E4M3).  Process-wide; not
 * synchronised with inferences in flight on other threads. */
int hm_debug_tc_path(int path);
/* Trainer::training_step + Trainer::loss (render_hair_msnn.cu:690-691),
 * split into its three phases and fused: forward keeps the activations
 * (d_out may be NULL; d_in must stay valid until backward), backward takes
 * the targets [n][out_ch] and writes the loss to the device scalar d_loss
 * (may be NULL), optimizer_step applies ExponentialDecay(Adam). */
int hm_mlp_forward(hm_mlp* mlp, const float* d_in, float* d_out, int64_t n, void* stream);
int hm_mlp_backward(hm_mlp* mlp, const float* d_target, int64_t n, float* d_loss, void* stream);
/* The backward of the last forward with a given dL/d(output) [n][out_ch]
 * instead of a loss (tcnn's Network::backward with dL_doutput; used to
 * carry image gradients into the cache weights).  Gradients as for
 * hm_mlp_backward; the loss is not computed. */
int hm_mlp_backward_output_grad(hm_mlp* mlp, const float* d_dloss_doutput, int64_t n, void* stream);
int hm_mlp_optimizer_step(hm_mlp* mlp, float loss_scale, void* stream);
int hm_mlp_training_step(hm_mlp* mlp, const float* d_in, const float* d_target, int64_t n,
                         float* d_loss, void* stream);
/* Loss of the last backward, copied to the host (synchronises). */
int hm_mlp_last_loss(hm_mlp* mlp, float* host_loss);
/* TINY_MLP::reset, neural_network.cu:17-21 (all parameters to zero). */
int hm_mlp_reset(hm_mlp* mlp);
/* Host copies of the FP32 master parameters / last gradients (n_params floats). */
int hm_mlp_get_params(const hm_mlp* mlp, float* host_out);
int hm_mlp_set_params(hm_mlp* mlp, const float* host_in);
int hm_mlp_get_gradients(const hm_mlp* mlp, float* host_out);
/* TINY_MLP::loadWeights, neural_network.cu:23-32.  hm_mlp_load reads either
 * a tiny-cuda-nn trainer snapshot as JSON text ({"n_params", "params_type"
 * "float" or "__half", "params_binary": {"bytes": [...]}}: what
 * TINY_MLP::loadWeights deserialises; optimizer state is not read) or the
 * library's own binary snapshot (which keeps the step and learning rate);
 * hm_mlp_save writes the JSON form when `path` ends in ".json", else the
 * binary one. */
int hm_mlp_save(const hm_mlp* mlp, const char* path);
int hm_mlp_load(hm_mlp* mlp, const char* path);

/* ------------------------------------------------------------------------
 * Scene.  Replaces parseScene (scene.cpp:119-339), the OWL geometry and
 * texture set-up of RenderWindow_HairMSNN::initialize (render_hair_msnn.cu
 * :98-412) and the OptiX acceleration-structure builds (owlGroupBuildAccel,
 * :316-384, 412): the scene owns device copies of the hair curves (cubic
 * B-spline segments), the head mesh, the environment sampling tables
 * (generateEnvSamplingTables, scene.cpp:349-425) and an LBVH over all
 * primitives.  json_text uses the reference's keys (camera, hair, integrator,
 * lights, tcnn, surface) with the same defaults and the same image-size
 * limits; the missing assets are replaced by generators:
 *   hair.procedural    {type straight|curly, strands, control_points, length,
 *                       radius, root_min_z, helix_radius, helix_pitch, seed}
 *   surface.procedural {type ellipsoid, triangles, radii[3], diffuse[3], alpha}
 *   lights.sky         {turbidity, sun[3], width, height, scale, rotation}
 *                      (Preetham et al. 1999 sky baked to a lat-long map)
 * As parseScene: a hair block without "type" keeps the default material
 * (alpha 0.03 rad), and the bounds behind the scene scale of a HAIR file
 * start at the origin (extractHairData's).  Unlike it, a missing integrator
 * key takes its default, and a scene without any light is refused.
 * base_dir resolves relative file names (tcnn.config).  Returns NULL and a
 * status (HM_EPARSE for bad JSON or a malformed .hair/.obj file, HM_EINVAL for a
 * missing file, HM_EUNSUPPORTED for .exr environment maps).
 * ---------------------------------------------------------------------- */
typedef struct hm_scene hm_scene;

typedef struct hm_scene_desc {
  int n_strands, n_control_points, n_segments;
  int n_vertices, n_triangles, n_bvh_nodes;
  int width, height, spp, path_v1, path_v2;
  int env_width, env_height, n_dir_lights;
  int mis, env_pdf, has_env;
  int shading_catrom; /* 1: curves shaded as Catmull-Rom (reference closest-hit quirk) */
  float scene_scale;
  float bounds_min[3], bounds_max[3];
  int n_bvh_wide_nodes; /* 8-wide nodes traversed by the kernels (0 before the build) */
  int n_groups;         /* strand groups with their own material (0: one material) */
  int segment_splits;   /* BVH leaves per hair segment (integrator.segment_splits: 1, 2 (default), 4);
                           HM_SCENE_BVH_LEAVES ids: segment k's part j is k + j * n_segments,
                           triangle i is n_segments * segment_splits + i */
} hm_scene_desc;

enum hm_scene_array {
  HM_SCENE_CONTROL_POINTS = 0, /* float4 (x, y, z, radius) */
  HM_SCENE_SEGMENTS = 1,       /* int32 first control point of each segment */
  HM_SCENE_VERTICES = 2,       /* float3 */
  HM_SCENE_NORMALS = 3,        /* float3 */
  HM_SCENE_TRIANGLES = 4,      /* int3 */
  HM_SCENE_ENV = 5,            /* float4 lat-long radiance, z up */
  HM_SCENE_ENV_CPDF = 6,       /* [H][W+1] */
  HM_SCENE_ENV_CCDF = 7,
  HM_SCENE_ENV_MPDF = 8,       /* [H+1] */
  HM_SCENE_ENV_MCDF = 9,
  HM_SCENE_DIR_LIGHTS = 10,    /* 6 floats each: normalised from, emit */
  HM_SCENE_BVH_NODES = 11,     /* 64 bytes each: child AABBs + child indices */
  HM_SCENE_BVH_LEAVES = 12,    /* int32 primitive of each leaf slot */
  HM_SCENE_CAMERA = 13,        /* pos, dir_00, dir_du, dir_dv (12 floats) */
  HM_SCENE_MATERIALS = 14,     /* 16 floats: hair params, diffuse, alpha, env scale/rotation */
  HM_SCENE_BVH_WIDE_NODES = 15, /* 224 bytes each: lo.x[8] hi.x[8] lo.y[8] hi.y[8] lo.z[8] hi.z[8]
                                   child[8] (>= 0 wide node, < 0 leaf ~slot); empty slots hold
                                   code -1 and the box [+inf, +inf] */
  HM_SCENE_STRAND_GROUPS = 16,   /* int32 group of each strand (empty: one material) */
  HM_SCENE_GROUP_MATERIALS = 17, /* hm_hair_params of each group */
  HM_SCENE_SEGMENT_GROUPS = 18   /* int32 group of each segment (empty: one material) */
};

/* Host-only: parses and generates (no device work). */
hm_scene* hm_scene_create(const char* json_text, const char* base_dir, int* status);
/* Uploads the scene and builds its LBVH on the current device (also done on
 * first use by hm_render_create / hm_trace_rays). */
int hm_scene_build(hm_scene* scene);
void hm_scene_destroy(hm_scene* scene);
int hm_scene_info(const hm_scene* scene, hm_scene_desc* out);
/* Host copy of one scene array (bytes: hm_scene_export_size). */
int64_t hm_scene_export_size(const hm_scene* scene, int which);
int hm_scene_export(const hm_scene* scene, int which, void* host_out, int64_t capacity_bytes);
/* Strand groups (no reference counterpart: the reference has one hair
 * material per scene, copied into every hit by hairCH, optix_common.cuh
 * :585-593).  Every strand gets a group in [0, n_groups), n_groups <= 64,
 * and every group its own material; a new grouping starts with every group
 * at the scene's material.  The scene JSON can give the same with
 * hair.groups = {count, assign: "azimuth" | "index", materials: [...]}.
 * hm_scene_set_group_materials replaces the groups' materials (n_groups = 1
 * on an ungrouped scene replaces the scene's material); it waits for the
 * device, so frames in flight finish with the old materials. */
int hm_scene_set_strand_groups(hm_scene* scene, const int32_t* strand_group, int n_strands, int n_groups);
int hm_scene_set_group_materials(hm_scene* scene, const hm_hair_params* materials, int n_groups);

/* Closest-hit (any_hit = 0) or any-hit traversal of n rays: d_org, d_dir
 * [n][3]; d_hits [n][4] = (t, primitive id as int bits (-1 miss), u, v):
 * u is the curve parameter for hair segments (primitives 0..n_segments-1),
 * (u, v) the barycentrics of vertices 1 and 2 for triangles.  Replaces
 * owl::traceRay with its closest-hit / any-hit programs. */
int hm_trace_rays(const hm_scene* scene, const float* d_org, const float* d_dir, int64_t n, float tmin,
                  float tmax, int any_hit, float* d_hits, void* stream);

/* ------------------------------------------------------------------------
 * Renderer.  Replaces RenderWindow_HairMSNN::render (render_hair_msnn.cu
 * :699-771) with the device programs of cuda/hair_msnn.cu (rayGenCam,
 * msnnPathTrace, msnnTrainingPath) and, in HM_MODE_PT, the plain path tracer
 * of render_path_tracing.cu / cuda/path_tracing.cu.  One hm_render_frame is
 * one sample per pixel: wavefront paths -> (MSNN) cache training step on
 * the frame's records -> cache inference -> compose; images accumulate in
 * FP64.  `beta` is the BETA command-line knob (render_hair_msnn.cu:1154,
 * internal beta = BETA - 1).
 * ---------------------------------------------------------------------- */
typedef struct hm_render hm_render;

/* HM_MODE_NRC: the reference's comparison renderer, neural radiance caching
 * (RenderWindowNRC, render_nrc.cu:640-701, cuda/nrc.cu): each path stops
 * where its spread passes c * a0 and takes the cache there; one pixel in
 * every everyNth traces a training suffix and gives one record per vertex
 * (train_records default 65536 = 1638 pixels x 40 vertices); the cache takes
 * 9 inputs (position, wo, n).  Single scenes; the final image only. */
enum hm_render_mode { HM_MODE_PT = 0, HM_MODE_MSNN = 1, HM_MODE_NRC = 2 };
enum hm_image { HM_IMAGE_FINAL = 0, HM_IMAGE_SHORT = 1, HM_IMAGE_CACHE = 2 };

typedef struct hm_render_options {
  int mode;                      /* hm_render_mode */
  int beta;                      /* BETA >= 0 (internal beta = BETA - 1) */
  int train_records;             /* per frame; 0 = 16384 (render_hair_msnn.h:127-129), NRC 65536 */
  int train;                     /* online cache training on/off (tcnn.init_train) */
  int cache_precision;           /* HM_PREC_* */
  uint32_t seed;                 /* cache initialisation */
  const char* cache_config_json; /* NULL: the scene's tcnn.config, else the built-in one */
  int frames_in_flight;          /* frames pipelined on their own streams (1..8); 0: up to 8,
                                    fewer when their path state would pass ~2 GB */
  float nrc_c;                   /* NRC spread threshold multiplier c (0: 0.01, render_nrc.h:132) */
} hm_render_options;

typedef struct hm_render_stats {
  int frames, pixels;
  int64_t extension_rays;
  int last_bounces;
  int train_records, every_nth;
  float last_loss;
} hm_render_stats;

hm_render* hm_render_create(hm_scene* scene, const hm_render_options* options, int* status);
void hm_render_destroy(hm_render* render);
/* Enqueues one frame and returns without waiting: up to frames_in_flight
 * frames overlap (the path tracing of frame k+1 never reads the cache, so it
 * runs while frame k's long training paths finish); the cache step and the
 * FP64 accumulation stay in frame order, so images are bit-identical to
 * serial frames.  The frame is ordered after work already enqueued on
 * `stream`; use hm_render_wait to order later work after it.
 * A frame's traversal errors are returned by a later call (when its slot is
 * reused, or by hm_render_read / _get_stats / _reset, which synchronise).
 * With instrumentation on, frames run one at a time. */
int hm_render_frame(hm_render* render, void* stream);
/* Many scenes rendered as one (no reference counterpart; the batched-render
 * configuration): every frame takes one sample per pixel of every scene, the
 * paths of all scenes share the same kernel launches (each path knows its
 * scene and walks that scene's tree), and one cache network is trained on
 * and queried for all of them.  betas: per-scene BETA (NULL: options->beta).
 * Images are stored scene after scene: read them with hm_render_read
 * ([total pixels][3]) and slice with hm_render_batch_scene, which gives a
 * scene's first pixel and size (single-scene renderers: scene 0). */
hm_render* hm_render_create_batch(hm_scene* const* scenes, const int* betas, int n_scenes,
                                  const hm_render_options* options, int* status);
int hm_render_batch_scene(const hm_render* render, int scene, int* pixel_offset, int* width, int* height);
/* Scene-sample training of the cache before rendering: the reference's
 * initial training (render_hair_msnn.cu:641-650: genTrainingData + train for
 * one second of wall time, TRAIN_DATA_GEN pass hair_msnn.cu:222-233) as an
 * explicit number of passes.  Each pass traces train_records training paths
 * aimed from the camera at points sampled on the hair (about 10^6, placed
 * by segment length as fetchSceneSamples, render_hair_msnn.cu:34-97) and
 * takes one training step.  Record r of the k-th pass (k counted over the
 * renderer's life from 0) aims at sample perm_k(r), a keyed permutation of
 * the samples standing in for the reference's shuffled sceneIndices, and
 * seeds its RNG as the reference's launch index (r % 128, r / 128) over the
 * frame's width with frame number k.  With a path log on and train_records
 * <= pixels, the log holds the last pass's paths (record r at path r).
 * HairMSNN renderers only; waits for frames in flight and returns when the
 * passes have finished. */
int hm_render_pretrain(hm_render* render, int passes, void* stream);
/* Launch-shape autotuner (no reference counterpart): times `frames`
 * pipelined frames per candidate and keeps the fastest persistent-traversal
 * grids (resident blocks per SM) and shading grid.  The shapes change no
 * result; the tuning frames do not train the cache and are dropped from the
 * image (the renderer is reset), so a tuned renderer renders bit for bit
 * what an untuned one does.  `out` (may be NULL) receives the choice.
 * With frames in flight, 16 or more frames per candidate: fewer include too
 * much of the pipeline's fill and drain (6 frames picked shapes 4% slower
 * at 512x512). */
typedef struct hm_render_tuning {
  int extend_blocks_per_sm, shadow_blocks_per_sm, shade_blocks_per_sm;
  float ms_per_frame; /* best time per frame seen while tuning */
} hm_render_tuning;
int hm_render_autotune(hm_render* render, int frames, void* stream, hm_render_tuning* out);
/* Launch mode (no reference counterpart).  on (the default): each frame's
 * path tracing (camera and every bounce round: extend, shade, shadow,
 * resolve, compact) is one CUDA graph per frame slot, captured on first use
 * and replayed every frame with the frame number read from device memory;
 * recaptured when launch shapes or materials change.  off: the same kernels
 * launched one by one.  Images are bit-identical either way; instrumented
 * frames always launch one by one. */
int hm_render_set_graphs(hm_render* render, int on);
/* Frames the renderer keeps in flight (the resolved frames_in_flight). */
int hm_render_frames_in_flight(const hm_render* render);
/* Makes `stream` wait for every frame in flight (no host synchronisation). */
int hm_render_wait(hm_render* render, void* stream);
/* Asynchronous read-back on `stream` of the FP64 running sums (divide by the
 * number of frames) of all frames enqueued so far, [H][W][3]; host_dst should
 * be pinned.  The sums are first copied to a device snapshot (allocated on
 * the first call, P x 3 doubles) and the host copy is made from it: the next
 * frame's accumulation waits only for the device copy. */
int hm_render_read_async(hm_render* render, int which, double* host_dst, void* stream);
/* Restart accumulation (the reference's cameraChanged resets accumId). */
int hm_render_reset(hm_render* render);
/* Average of the accumulated frames, FP64 [H][W][3], row 0 = bottom. */
int hm_render_read(hm_render* render, int which, double* host_rgb);
int hm_render_get_stats(const hm_render* render, hm_render_stats* out);
/* Per-frame instrumentation (the reference's renderTime / trainTime /
 * inferTime, render_hair_msnn.cu:649-770, measured with CUDA events on the
 * render stream).  timing: event pairs around every stage of each frame;
 * counting: traversal work counters (slower kernels; for an untimed pass). */
typedef struct hm_render_timings {
  float total_ms, camera_ms, extend_ms, shade_ms, shadow_ms, compact_ms, finalize_ms;
  float train_ms, infer_ms, compose_ms;
  int bounces, kernel_launches;
  int64_t extension_rays, shadow_rays;
  int64_t extend_nodes, extend_prims, shadow_nodes, shadow_prims;
  /* per bounce (first 48): paths traced, extension and shadow traversal ms */
  int paths_by_bounce[48];
  float extend_ms_by_bounce[48], shadow_ms_by_bounce[48];
} hm_render_timings;
int hm_render_set_instrumentation(hm_render* render, int timing, int counting);
int hm_render_get_timings(const hm_render* render, hm_render_timings* out);
/* The wavefront's queue compaction (no reference counterpart: the OptiX
 * megakernel has no queues): out = the entries queue[i] with keep[i] != 0,
 * in order (a stable partition), *out_count their number.  The same three
 * kernels (block counts, block-offset scan, scatter) that compact the path
 * queue between bounce rounds of a frame.  Device arrays of n int32; waits
 * for the stream. */
int hm_queue_compact(const int32_t* d_keep, const int32_t* d_queue, int64_t n, int32_t* d_out, int64_t* out_count,
                     void* stream);
/* Per-path ray log (no reference counterpart; parity tests).  With
 * vertices > 0 every later frame records, for each path, the rays it traced
 * at its first `vertices` vertices; hm_render_read_path_log copies the last
 * frame's log, [P][3 * vertices][12] floats: slot 3k + j is vertex k's
 * extension ray (j = 0, the ray that found the vertex), light-sample shadow
 * ray (1) and BSDF-sample shadow ray (2) as
 *   result (int bits: hit primitive or -1; shadow: 1 unoccluded, 0 occluded),
 *   t, u, RNG state when the ray was traced (extension rays; uint bits),
 *   direction[3], kind (int bits: 0, 1, 2; -1 empty slot), origin[3], 0.
 * Single-scene renderers (PT, HairMSNN, NRC) created with frames_in_flight = 1.
 * vertices = 0 turns the log off. */
int hm_render_set_path_log(hm_render* render, int vertices);
int hm_render_read_path_log(hm_render* render, float* host_dst, int64_t n_floats);
/* The render's cache network (owned by the render; NULL in PT mode). */
hm_mlp* hm_render_cache(hm_render* render);
/* Device buffers of the last frame: 0 cache inputs [P][12], 1 cache outputs
 * [P][3], 2 training inputs [R][12], 3 training targets [R][3], 4 G-buffer;
 * and the FP64 running sums [P][3] of the frames accumulated so far (divide
 * by the frame count): 5 final image, 6 short paths, 7 cache.  NRC renders
 * (9 input channels; rows [P, P + T) of 0/1 are the T training pixels'
 * suffix queries): 8 throughput at each pixel's cache query (float4 [P]),
 * 9 train buffer (float4 [T][40][5]: position / scale, wo, n, direct light,
 * throughput factor), 10 per training pixel (int4: bounces, suffix ended at
 * a query, unbiased, primary hit).  11: the points of the scene-sample
 * training pass (float4 [N], xyz; after hm_render_pretrain). */
int hm_render_buffer(hm_render* render, int which, void** dptr, int64_t* count);

/* ------------------------------------------------------------------------
 * Differentiable rendering by path replay (no reference counterpart; the
 * differentiable appearance-fit configuration).  Single-scene renderers.
 *
 * hm_render_diff_forward restarts accumulation and enqueues `frames` frames
 * (one sample per pixel each) with the cache frozen: no training pixels and
 * no training step, so in HairMSNN mode every hair pixel is its short path
 * plus the cache at the primary hit.  The image is then
 * hm_render_read(HM_IMAGE_FINAL), the mean of the frames.  Each path's
 * radiance is kept (16 bytes per path and frame) for the replay.
 *   eval_materials (may be NULL): a detached render for finite differences:
 *   the hair BSDF values come from these materials (one per strand group),
 *   while directions, pdfs, MIS weights and Russian roulette keep the
 *   scene's; such a forward cannot be replayed.
 *
 * hm_render_diff_backward replays the paths of the last forward with the
 * same random numbers and returns dL/d(material) for d_adjoint = dL/dImage
 * ([H][W][3] FP32 on the device, the layout of hm_render_read):
 * host_grad[g * 6 + k] (FP64), k = sigma_a r, g, b, beta_m, beta_n, alpha
 * (radians), for every strand group g (one group on an ungrouped scene);
 * n_grad >= 6 * groups.  The sampling is detached (the sampled directions,
 * pdfs and MIS weights are held fixed; Path Replay Backpropagation, Vicini
 * et al. 2021): the result is the exact derivative of the detached render
 * and an unbiased estimate of the derivative of the expected image.  In
 * HairMSNN mode the cache network's parameter gradients
 * (hm_mlp_get_gradients on hm_render_cache) receive dL/d(weights).
 * Synchronises. */
int hm_render_diff_forward(hm_render* render, int frames, const hm_hair_params* eval_materials, int n_materials,
                           void* stream);
int hm_render_diff_backward(hm_render* render, const float* d_adjoint, double* host_grad, int n_grad, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* HAIRMSNN_H_ */
