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
 *   precision    HM_PREC_*; seed: parameter initialisation stream
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
/* Trainer::training_step + Trainer::loss (render_hair_msnn.cu:690-691),
 * split into its three phases and fused: forward keeps the activations
 * (d_out may be NULL; d_in must stay valid until backward), backward takes
 * the targets [n][out_ch] and writes the loss to the device scalar d_loss
 * (may be NULL), optimizer_step applies ExponentialDecay(Adam). */
int hm_mlp_forward(hm_mlp* mlp, const float* d_in, float* d_out, int64_t n, void* stream);
int hm_mlp_backward(hm_mlp* mlp, const float* d_target, int64_t n, float* d_loss, void* stream);
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
/* TINY_MLP::loadWeights, neural_network.cu:23-32 (own binary snapshot format). */
int hm_mlp_save(const hm_mlp* mlp, const char* path);
int hm_mlp_load(hm_mlp* mlp, const char* path);

#ifdef __cplusplus
}
#endif

#endif /* HAIRMSNN_H_ */
