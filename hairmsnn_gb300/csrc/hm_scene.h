// Scene: hair curves, head mesh, lights, camera and integrator settings.
// Host-side description (std::vector) plus the device copies the kernels use.
#pragma once
#include <string>
#include <vector>

#include "hm_common.cuh"
#include "hm_hair_bsdf.cuh"

namespace hm {

constexpr int kWide = 8;                  // children per node of the traversed BVH
constexpr int kWideF4 = 7 * kWide / 4;    // float4 per wide node (6 bounds + 1 code per child)
constexpr int kWideNodeBytes = 16 * kWideF4;

HM_D f3 ldf3(const float3* p) {
  const float* q = reinterpret_cast<const float*>(p);
  return mk(__ldg(q), __ldg(q + 1), __ldg(q + 2));
}
HM_D int3 ldi3(const int3* p) {
  const int* q = reinterpret_cast<const int*>(p);
  return make_int3(__ldg(q), __ldg(q + 1), __ldg(q + 2));
}

constexpr int kMaxStrandGroups = 64;  // materials per scene (group ids are bytes)

// Device view of the scene, passed to every render kernel by value.
struct SceneDev {
  // hair: cubic B-spline segments over control points (x, y, z, radius)
  const float4* cp;
  const int* seg;  // first control point of each segment
  int n_seg;
  // BVH leaves per segment: segment k's part j (its u range [j, j+1) / split)
  // is leaf primitive k + j * n_seg; triangles follow at n_hprim
  int seg_split;
  int n_hprim;  // n_seg * seg_split
  int shading_catrom;  // 1: shade with the Catmull-Rom interpretation (reference CH quirk)
  // head mesh
  const float3* vtx;
  const float3* nrm;
  const int3* tri;
  int n_tri;
  f3 diffuse;
  float alpha;  // already clamp(alpha, .01, 1)^2 as triangleMeshCH does
  // BVH over [segments | triangles]: node i has two children (child AABBs inline)
  const float4* nodes;  // 4 float4 per node
  int n_nodes;
  const int* prim_of_leaf;  // leaf slot -> primitive id
  // the same tree collapsed to kWide-wide nodes (what the traversal walks):
  // kWideF4 float4 per node, lo.x[8] hi.x[8] lo.y[8] hi.y[8] lo.z[8] hi.z[8]
  // child[8] (>= 0 wide node, < 0 leaf ~slot; empty slots: code -1 and the
  // box [+inf, +inf], which every ray misses)
  const float4* wnodes;
  int n_wnodes;
  // environment (lat-long, z up) and its sampling tables
  int has_env, env_pdf_sampling;
  const float4* env;
  int env_w, env_h;
  const float* cpdf;  // [H][W+1]
  const float* ccdf;
  const float* mpdf;  // [H+1]
  const float* mcdf;
  float env_scale, env_rot_phi;
  // directional lights
  int n_dlights;
  const float* dlights;  // [n][6]: from (normalised), emit
  int n_total_lights;
  // camera (cameraChanged, render_hair_msnn.cu:1093-1118)
  f3 cam_pos, cam_d00, cam_du, cam_dv;
  // material, integrator
  HairConsts hair;
  hm_hair_params hair_raw;  // the parameters `hair` was made from
  // strand groups: segment -> group, per-group material (n_groups == 0:
  // every segment uses `hair`)
  const uint8_t* seg_group;
  const HairConsts* group_hc;
  const hm_hair_params* group_raw;
  int n_groups;
  int mis;
  int width, height;
  int path_v1, path_v2;
  float scene_scale;
};

struct Scene {
  // ---- host data
  std::vector<float4> cp;
  std::vector<int> seg;
  int n_strands = 0;
  std::vector<int> strand_seg;  // first segment of every strand (n_strands + 1 entries)
  // strand groups (empty: one material, `hair`)
  std::vector<int> strand_group;
  std::vector<hm_hair_params> group_mats;
  std::vector<int> seg_group_host;  // group of every segment (derived)
  int material_version = 0;          // bumped by every change of groups or materials
  std::vector<float3> vtx, nrm;
  std::vector<int3> tri;
  f3 diffuse{0.5f, 0.5f, 0.5f};
  float alpha_raw = 1.f;
  std::vector<float4> env;
  int env_w = 0, env_h = 0;
  std::vector<float> cpdf, ccdf, mpdf, mcdf;
  float env_scale = 1.f, env_rot_phi = 0.f;
  bool has_env = false, env_pdf = true;
  std::vector<float> dlights;  // 6 per light
  hm_hair_params hair{};
  f3 cam_from{0, 0, 5}, cam_at{0, 0, 0}, cam_up{0, 1, 0};
  float cos_fovy = 0.66f;
  int width = 512, height = 512, spp = 16, path_v1 = 1, path_v2 = 40;
  bool mis = true;
  int shading_catrom = 0;
  int seg_split = 2;  // BVH leaves per hair segment (1, 2 or 4)
  f3 bmin{1e30f, 1e30f, 1e30f}, bmax{-1e30f, -1e30f, -1e30f};
  float scene_scale = 1.f;
  std::string cache_config;  // tcnn JSON text (scene "tcnn.config")
  std::string cache_weights;  // path of a weight snapshot (scene "tcnn.init_weights"), "" for none
  bool cache_train = true;
  std::string image_output, stats_output;

  // ---- device copies
  float4* d_cp = nullptr;
  int* d_seg = nullptr;
  float3* d_vtx = nullptr;
  float3* d_nrm = nullptr;
  int3* d_tri = nullptr;
  float4* d_env = nullptr;
  float *d_cpdf = nullptr, *d_ccdf = nullptr, *d_mpdf = nullptr, *d_mcdf = nullptr;
  float* d_dlights = nullptr;
  float4* d_nodes = nullptr;
  int* d_prim_of_leaf = nullptr;
  int n_nodes = 0;
  float4* d_wnodes = nullptr;
  int n_wnodes = 0;
  uint8_t* d_seg_group = nullptr;
  HairConsts* d_group_hc = nullptr;
  hm_hair_params* d_group_raw = nullptr;
  bool built = false;

  ~Scene();
  int ensure_built();
  int upload();
  int build_bvh(cudaStream_t st);
  SceneDev dev() const;
  int n_prims() const { return (int)seg.size() * seg_split + (int)tri.size(); }
  int n_groups() const { return group_mats.empty() ? 1 : (int)group_mats.size(); }
  int set_strand_groups(const int* groups, int n, int n_groups);
  int set_group_materials(const hm_hair_params* m, int n);
  int upload_groups();
};

int scene_from_json(const char* text, const char* base_dir, Scene* s);
void env_sampling_tables(const float4* env, int w, int h, std::vector<float>& cpdf, std::vector<float>& ccdf,
                         std::vector<float>& mpdf, std::vector<float>& mcdf);

}  // namespace hm
