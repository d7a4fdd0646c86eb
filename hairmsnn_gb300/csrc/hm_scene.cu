// Scene construction: the reference's scene JSON (parseScene, scene.cpp:119-339)
// plus procedural generators standing in for the absent .hair / .obj / .exr
// assets, the environment sampling tables (generateEnvSamplingTables,
// scene.cpp:349-425) and the pinhole camera (cameraChanged,
// render_hair_msnn.cu:1093-1118).  Host C++; device copies in Scene::upload.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <fstream>
#include <sstream>

#include "hm_exr.h"
#include "hm_json.h"
#include "hm_scene.h"

namespace hm {

static f3 f3_of(const Json& a, f3 d) {
  if (!a.is_array() || a.size() < 3) return d;
  return mk((float)a[0].as_number(), (float)a[1].as_number(), (float)a[2].as_number());
}

static bool read_file(const std::string& path, std::string* out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::stringstream ss;
  ss << f.rdbuf();
  *out = ss.str();
  return true;
}

static std::string join_path(const std::string& base, const std::string& p) {
  if (p.empty() || p[0] == '/' || base.empty()) return p;
  return base + "/" + p;
}

// ------------------------------------------------------------ procedural hair
// Deterministic per seed: roots uniformly on the upper cap of the head
// ellipsoid, strands leave along the surface normal, bend towards -z (gravity)
// and are kept outside the head; `curly` adds a helix around the local
// direction.  Control points are cubic B-spline points (x, y, z, radius).
struct HairGen {
  std::string type = "straight";
  int strands = 10000, cps = 64;
  float length = 2.f, radius = 4e-4f;
  float root_min_z = 0.25f;
  float helix_radius = 0.05f, helix_pitch = 0.1f;  // curly only (scene units)
  uint32_t seed = 1;
};

static void gen_hair(const HairGen& g, f3 head_r, Scene* s) {
  uint32_t st = rng_seed((int)g.seed, 0x4a1u);
  const float step = g.length / (float)(g.cps - 1);
  s->n_strands = g.strands;
  s->cp.reserve((size_t)g.strands * g.cps);
  s->seg.reserve((size_t)g.strands * (g.cps - 3));
  auto inside = [&](f3 p, float margin) {
    f3 q = mk(p.x / (head_r.x + margin), p.y / (head_r.y + margin), p.z / (head_r.z + margin));
    return dot(q, q) < 1.f;
  };
  for (int k = 0; k < g.strands; ++k) {
    // uniform direction on the cap z >= root_min_z of the unit sphere
    float u1 = lcg_next(st), u2 = lcg_next(st);
    float z = g.root_min_z + (1.f - g.root_min_z) * u1;
    float r = sqrtf(fmaxf(0.f, 1.f - z * z));
    float phi = 2.f * kPi * u2;
    f3 n = mk(r * cosf(phi), r * sinf(phi), z);
    f3 p = mk(n.x * head_r.x, n.y * head_r.y, n.z * head_r.z);
    f3 gn = normalize(mk(n.x / head_r.x, n.y / head_r.y, n.z / head_r.z));  // surface normal
    f3 dir = gn;
    float jitter = 0.15f * (lcg_next(st) - 0.5f);
    float hphase = 2.f * kPi * lcg_next(st);
    int first = (int)s->cp.size();
    s->strand_seg.push_back((int)s->seg.size());
    for (int i = 0; i < g.cps; ++i) {
      f3 q = p;
      if (g.type == "curly") {
        // helix around the strand's running direction
        f3 a = normalize(cross(dir, fabsf(dir.z) < 0.9f ? mk(0, 0, 1) : mk(1, 0, 0)));
        f3 b = cross(dir, a);
        float ang = hphase + 2.f * kPi * (float)i * step / g.helix_pitch;
        float hr = g.helix_radius * fminf(1.f, (float)i / 4.f);
        q = p + a * (hr * cosf(ang)) + b * (hr * sinf(ang));
      }
      s->cp.push_back(make_float4(q.x, q.y, q.z, g.radius));
      // advance: bend towards gravity, stay outside the head
      dir = normalize(dir + mk(jitter * dir.y, -jitter * dir.x, -0.12f));
      f3 np = p + dir * step;
      if (inside(np, 0.02f)) {
        f3 out = normalize(mk(np.x / head_r.x, np.y / head_r.y, np.z / head_r.z));
        np = mk(out.x * (head_r.x + 0.021f), out.y * (head_r.y + 0.021f), out.z * (head_r.z + 0.021f));
        dir = normalize(np - p);
      }
      p = np;
    }
    for (int i = 0; i + 3 < g.cps; ++i) s->seg.push_back(first + i);
  }
  s->strand_seg.push_back((int)s->seg.size());
}

// ------------------------------------------------------------ .hair files
// Cem Yuksel's HAIR format (its published description): a 128-byte header
// ("HAIR", strand count, point count, a bit field of the arrays present,
// default segments / thickness / transparency / colour, 88 bytes of text),
// then the arrays present, in order: segments (uint16 per strand), points
// (3 floats per point), thickness (float per point), transparency (float per
// point), colours (3 floats per point).  Strands become cubic B-splines as in
// Scene::extractHairData (scene.cpp:10-73): a phantom point p0 + (p0 - p1)
// before each strand and pN + (pN - pN-1) after it, one segment starting at
// the phantom and at every point but the last two, radius 0.2 x thickness.
// The bounds (and so the scene scale) are those of the file's own points.
static int load_hair_file(const std::string& path, Scene* s, f3* raw_lo, f3* raw_hi) {
  std::string data;
  if (!read_file(path, &data)) return hm_set_error("scene: cannot read hair file %s", path.c_str()), HM_EINVAL;
  if (data.size() < 128 || data.compare(0, 4, "HAIR") != 0)
    return hm_set_error("scene: %s is not a HAIR file", path.c_str()), HM_EPARSE;
  auto u32 = [&](size_t off) {
    uint32_t v;
    memcpy(&v, data.data() + off, 4);
    return v;
  };
  auto f32 = [&](size_t off) {
    float v;
    memcpy(&v, data.data() + off, 4);
    return v;
  };
  const uint32_t n_strands = u32(4), n_points = u32(8), flags = u32(12), d_segments = u32(16);
  const float d_thickness = f32(20);
  size_t off = 128;
  const size_t seg_bytes = (flags & 1) ? (size_t)n_strands * 2 : 0;
  const size_t pts_bytes = (flags & 2) ? (size_t)n_points * 12 : 0;
  const size_t thk_bytes = (flags & 4) ? (size_t)n_points * 4 : 0;
  if (!(flags & 2)) return hm_set_error("scene: %s has no points array", path.c_str()), HM_EPARSE;
  if (data.size() < off + seg_bytes + pts_bytes + thk_bytes)
    return hm_set_error("scene: %s is truncated", path.c_str()), HM_EPARSE;
  const uint8_t* base = reinterpret_cast<const uint8_t*>(data.data());
  const uint8_t* segs = (flags & 1) ? base + off : nullptr;
  off += seg_bytes;
  const uint8_t* pts = base + off;
  off += pts_bytes;
  const uint8_t* thk = (flags & 4) ? base + off : nullptr;
  auto point = [&](int64_t i) {
    i = std::min<int64_t>(std::max<int64_t>(i, 0), (int64_t)n_points - 1);
    float v[3];
    memcpy(v, pts + 12 * i, 12);
    return mk(v[0], v[1], v[2]);
  };
  auto width = [&](int64_t i) {
    if (!thk) return d_thickness;
    float v;
    memcpy(&v, thk + 4 * i, 4);
    return v;
  };
  // extractHairData's bounds start from HairModel's defaults, (0, 0, 0)
  // (model.h): the origin is always inside them, and with it in the scene
  // scale (hairModel.scale, render_hair_msnn.cu:357)
  f3 lo = mk(0.f, 0.f, 0.f), hi = mk(0.f, 0.f, 0.f);
  uint32_t strand = 0;
  int left = -1;
  s->cp.clear();
  s->seg.clear();
  s->strand_seg.clear();
  for (int64_t i = 0; i < (int64_t)n_points; ++i) {
    const f3 p = point(i);
    const float w = width(i);
    lo = mk(fminf(lo.x, p.x), fminf(lo.y, p.y), fminf(lo.z, p.z));
    hi = mk(fmaxf(hi.x, p.x), fmaxf(hi.y, p.y), fmaxf(hi.z, p.z));
    bool first = false;
    if (left == -1) {
      if (strand == n_strands) break;
      uint16_t ns = (uint16_t)d_segments;
      if (segs) memcpy(&ns, segs + 2 * strand, 2);
      left = ns;
      ++strand;
      first = true;
    }
    if (first) {
      s->strand_seg.push_back((int)s->seg.size());
      const f3 q = p + (p - point(i + 1));
      s->cp.push_back(make_float4(q.x, q.y, q.z, 0.2f * w));
      s->seg.push_back((int)s->cp.size() - 1);
    }
    s->cp.push_back(make_float4(p.x, p.y, p.z, 0.2f * w));
    if (left > 1) {
      s->seg.push_back((int)s->cp.size() - 1);
    } else if (left == 0) {
      const f3 q = p + (p - point(i - 1));
      s->cp.push_back(make_float4(q.x, q.y, q.z, 0.2f * w));
    }
    --left;
  }
  // a strand cut short by the point count leaves segments without their
  // last control points: drop them
  while (!s->seg.empty() && s->seg.back() + 3 >= (int)s->cp.size()) s->seg.pop_back();
  s->n_strands = (int)strand;
  s->strand_seg.push_back((int)s->seg.size());
  for (int& o : s->strand_seg) o = std::min(o, (int)s->seg.size());
  if (s->seg.empty()) return hm_set_error("scene: %s has no complete segment", path.c_str()), HM_EPARSE;
  *raw_lo = lo;
  *raw_hi = hi;
  return HM_OK;
}

// ------------------------------------------------------------ .obj files
// Wavefront OBJ: "v", "vn" and "f" records (1-based or negative indices,
// v, v/vt, v//vn, v/vt/vn), polygons split into fans.  As loadOBJ
// (model.cpp:233-345) does, every triangle gets its own three vertices and
// the file's normals; a face without normals gets its geometric normal.
static int load_obj_file(const std::string& path, Scene* s) {
  std::string data;
  if (!read_file(path, &data)) return hm_set_error("scene: cannot read OBJ file %s", path.c_str()), HM_EINVAL;
  std::vector<f3> v, vn;
  s->vtx.clear();
  s->nrm.clear();
  s->tri.clear();
  size_t pos = 0;
  while (pos < data.size()) {
    size_t end = data.find('\n', pos);
    if (end == std::string::npos) end = data.size();
    std::string line = data.substr(pos, end - pos);
    pos = end + 1;
    if (line.size() < 2) continue;
    if (line[0] == 'v' && (line[1] == ' ' || line[1] == '\t')) {
      float x = 0, y = 0, z = 0;
      if (sscanf(line.c_str() + 2, "%f %f %f", &x, &y, &z) == 3) v.push_back(mk(x, y, z));
    } else if (line[0] == 'v' && line[1] == 'n') {
      float x = 0, y = 0, z = 0;
      if (sscanf(line.c_str() + 3, "%f %f %f", &x, &y, &z) == 3) vn.push_back(mk(x, y, z));
    } else if (line[0] == 'f' && (line[1] == ' ' || line[1] == '\t')) {
      std::vector<int> fv, fn;
      const char* c = line.c_str() + 2;
      while (*c) {
        while (*c == ' ' || *c == '\t' || *c == '\r') ++c;
        if (!*c) break;
        int a = 0, b = 0, n = 0;
        int got = 0;
        char* e = nullptr;
        a = (int)strtol(c, &e, 10);
        got = e != c;
        c = e;
        if (*c == '/') {
          ++c;
          if (*c != '/') {
            b = (int)strtol(c, &e, 10);
            c = e;
          }
          if (*c == '/') {
            ++c;
            n = (int)strtol(c, &e, 10);
            c = e;
          }
        }
        (void)b;
        while (*c && *c != ' ' && *c != '\t') ++c;
        if (!got) break;
        const int vi = a > 0 ? a - 1 : (int)v.size() + a;
        const int ni = n > 0 ? n - 1 : (n < 0 ? (int)vn.size() + n : -1);
        if (vi < 0 || vi >= (int)v.size()) return hm_set_error("scene: %s: vertex index out of range", path.c_str()), HM_EPARSE;
        fv.push_back(vi);
        fn.push_back(ni >= 0 && ni < (int)vn.size() ? ni : -1);
      }
      for (size_t k = 1; k + 1 < fv.size(); ++k) {
        const int ids[3] = {fv[0], fv[k], fv[k + 1]};
        const int nid[3] = {fn[0], fn[k], fn[k + 1]};
        const f3 gn = normalize(cross(v[ids[1]] - v[ids[0]], v[ids[2]] - v[ids[0]]));
        const int b0 = (int)s->vtx.size();
        for (int q = 0; q < 3; ++q) {
          s->vtx.push_back(make_float3(v[ids[q]].x, v[ids[q]].y, v[ids[q]].z));
          const f3 nn = nid[q] >= 0 ? vn[nid[q]] : gn;
          s->nrm.push_back(make_float3(nn.x, nn.y, nn.z));
        }
        s->tri.push_back(make_int3(b0, b0 + 1, b0 + 2));
      }
    }
  }
  if (s->tri.empty()) return hm_set_error("scene: %s has no faces", path.c_str()), HM_EPARSE;
  return HM_OK;
}

// ------------------------------------------------------------ head ellipsoid
static void gen_ellipsoid(int triangles, f3 radii, Scene* s) {
  int nu = std::max(3, (int)lrintf(sqrtf((float)triangles / 2.f)));
  int nv = std::max(2, (int)lrintf((float)triangles / (2.f * (float)nu)) + 1);
  auto push = [&](float th, float ph) {
    f3 d = mk(sinf(th) * cosf(ph), sinf(th) * sinf(ph), cosf(th));
    f3 p = mk(d.x * radii.x, d.y * radii.y, d.z * radii.z);
    f3 n = normalize(mk(d.x / radii.x, d.y / radii.y, d.z / radii.z));
    s->vtx.push_back(make_float3(p.x, p.y, p.z));
    s->nrm.push_back(make_float3(n.x, n.y, n.z));
  };
  push(0.f, 0.f);  // north pole = 0
  for (int v = 1; v < nv; ++v)
    for (int u = 0; u < nu; ++u) push(kPi * (float)v / (float)nv, 2.f * kPi * (float)u / (float)nu);
  push(kPi, 0.f);  // south pole
  const int south = (int)s->vtx.size() - 1;
  auto ring = [&](int v, int u) { return 1 + (v - 1) * nu + (u % nu); };
  for (int u = 0; u < nu; ++u) s->tri.push_back(make_int3(0, ring(1, u), ring(1, u + 1)));
  for (int v = 1; v + 1 < nv; ++v)
    for (int u = 0; u < nu; ++u) {
      s->tri.push_back(make_int3(ring(v, u), ring(v + 1, u), ring(v + 1, u + 1)));
      s->tri.push_back(make_int3(ring(v, u), ring(v + 1, u + 1), ring(v, u + 1)));
    }
  for (int u = 0; u < nu; ++u) s->tri.push_back(make_int3(ring(nv - 1, u), south, ring(nv - 1, u + 1)));
}

// ------------------------------------------------------------ Preetham sky
// Preetham, Shirley, Smits, "A Practical Analytic Model for Daylight"
// (SIGGRAPH 1999): Perez distribution with turbidity-dependent coefficients
// for Y, x, y; zenith values from the paper's fits; xyY -> XYZ -> linear
// sRGB.  Normalised so the zenith luminance is 1 before `scale`.  Below the
// horizon a dim grey ground (0.3 x the horizon luminance).
static void bake_sky(float T, f3 sun, int W, int H, float scale, std::vector<float4>* env) {
  sun = normalize(sun);
  const double ths = acos(std::min(1.0, std::max(-1.0, (double)sun.z)));
  auto perez = [](const double c[5], double th, double gm) {
    double ct = std::max(cos(th), 1e-3);
    return (1.0 + c[0] * exp(c[1] / ct)) * (1.0 + c[2] * exp(c[3] * gm) + c[4] * cos(gm) * cos(gm));
  };
  const double cY[5] = {0.1787 * T - 1.4630, -0.3554 * T + 0.4275, -0.0227 * T + 5.3251, 0.1206 * T - 2.5771,
                        -0.0670 * T + 0.3703};
  const double cx[5] = {-0.0193 * T - 0.2592, -0.0665 * T + 0.0008, -0.0004 * T + 0.2125, -0.0641 * T - 0.8989,
                        -0.0033 * T + 0.0452};
  const double cy[5] = {-0.0167 * T - 0.2608, -0.0950 * T + 0.0092, -0.0079 * T + 0.2102, -0.0441 * T - 1.6537,
                        -0.0109 * T + 0.0529};
  const double chi = (4.0 / 9.0 - T / 120.0) * (M_PI - 2.0 * ths);
  const double Yz = (4.0453 * T - 4.9710) * tan(chi) - 0.2155 * T + 2.4192;
  const double t2 = ths * ths, t3 = t2 * ths, TT = (double)T * T;
  const double xz = TT * (0.00166 * t3 - 0.00375 * t2 + 0.00209 * ths) +
                    T * (-0.02903 * t3 + 0.06377 * t2 - 0.03202 * ths + 0.00394) +
                    (0.11693 * t3 - 0.21196 * t2 + 0.06052 * ths + 0.25886);
  const double yz = TT * (0.00275 * t3 - 0.00610 * t2 + 0.00317 * ths) +
                    T * (-0.04214 * t3 + 0.08970 * t2 - 0.04153 * ths + 0.00516) +
                    (0.15346 * t3 - 0.26756 * t2 + 0.06670 * ths + 0.26688);
  auto sky = [&](double th, double gm, double out[3]) {
    double Y = Yz * perez(cY, th, gm) / perez(cY, 0.0, ths);
    double x = xz * perez(cx, th, gm) / perez(cx, 0.0, ths);
    double y = yz * perez(cy, th, gm) / perez(cy, 0.0, ths);
    double X = x / y * Y, Z = (1.0 - x - y) / y * Y;
    out[0] = 3.2406 * X - 1.5372 * Y - 0.4986 * Z;
    out[1] = -0.9689 * X + 1.8758 * Y + 0.0415 * Z;
    out[2] = 0.0557 * X - 0.2040 * Y + 1.0570 * Z;
    for (int c = 0; c < 3; ++c) out[c] = std::max(0.0, out[c] / Yz);
  };
  env->assign((size_t)W * H, make_float4(0, 0, 0, 1));
  for (int y = 0; y < H; ++y) {
    double th = M_PI * (y + 0.5) / H;
    for (int x = 0; x < W; ++x) {
      double ph = 2.0 * M_PI * (x + 0.5) / W;
      double d[3] = {sin(th) * cos(ph), sin(th) * sin(ph), cos(th)};
      double c[3];
      if (th <= M_PI / 2) {
        double cg = d[0] * sun.x + d[1] * sun.y + d[2] * sun.z;
        sky(th, acos(std::min(1.0, std::max(-1.0, cg))), c);
      } else {
        double h[3];
        sky(M_PI / 2 - 1e-3, M_PI / 2, h);
        double g = 0.3 * (0.2126 * h[0] + 0.7152 * h[1] + 0.0722 * h[2]);
        c[0] = g * 1.0; c[1] = g * 0.9; c[2] = g * 0.8;
      }
      (*env)[(size_t)y * W + x] = make_float4((float)(c[0] * scale), (float)(c[1] * scale), (float)(c[2] * scale), 1.f);
    }
  }
}

// generateEnvSamplingTables (scene.cpp:349-425): row-conditional and
// marginal tables of the map's mean radiance weighted by sin(theta), in the
// same single-precision operation order (the tables must be bit-identical).
// Row y of the conditional tables holds W + 1 entries: the running sum
// (cdf, normalised by the row's total) and the weights (pdf, whose last
// entry is the row's total); the marginal tables do the same over the rows'
// totals.
void env_sampling_tables(const float4* env, int width, int height, std::vector<float>& row_pdf,
                         std::vector<float>& row_cdf, std::vector<float>& marg_pdf, std::vector<float>& marg_cdf) {
  const int stride = width + 1;
  row_pdf.assign((size_t)stride * height, 0.f);
  row_cdf.assign((size_t)stride * height, 0.f);
  auto mean_rgb = [](float4 c) { return (c.x + c.y + c.z) * (1.0f / 3.0f); };
  for (int y = 0; y < height; y++) {
    float* w = row_pdf.data() + (size_t)y * stride;
    float* acc = row_cdf.data() + (size_t)y * stride;
    const float sin_t = sinf(3.14159f * (y + 0.5f) / height);
    w[0] = mean_rgb(env[y * width]) * sin_t;
    acc[0] = 0.0f;
    for (int x = 1; x < width; x++) {
      w[x] = mean_rgb(env[y * width + x]) * sin_t;
      acc[x] = acc[x - 1] + w[x - 1] / width;
    }
    const float row_total = acc[width - 1] + w[width - 1] / width;
    w[width] = row_total;
    if (row_total > 0.0f) {
      const float scale = 1.0f / row_total;
      for (int x = 1; x < width; x++) acc[x] *= scale;
    }
    acc[width] = 1.0f;
  }
  marg_pdf.assign(height + 1, 0.f);
  marg_cdf.assign(height + 1, 0.f);
  marg_pdf[0] = row_pdf[width];
  marg_cdf[0] = 0.0f;
  for (int r = 1; r < height; r++) {
    marg_pdf[r] = row_pdf[(size_t)r * stride + width];
    marg_cdf[r] = marg_cdf[r - 1] + marg_pdf[r - 1] / height;
  }
  const float total = marg_cdf[height - 1] + marg_pdf[height - 1] / height;
  marg_pdf[height] = total;
  if (total > 0.0f)
    for (int r = 1; r < height; r++) marg_cdf[r] /= total;
  marg_cdf[height] = 1.0f;
}

static void grow(f3& lo, f3& hi, f3 p) {
  lo = mk(fminf(lo.x, p.x), fminf(lo.y, p.y), fminf(lo.z, p.z));
  hi = mk(fmaxf(hi.x, p.x), fmaxf(hi.y, p.y), fmaxf(hi.z, p.z));
}

int scene_from_json(const char* text, const char* base_dir, Scene* s) {
  Json j;
  try {
    j = json_parse(text);
  } catch (const std::exception& e) {
    hm_set_error("scene: %s", e.what());
    return HM_EPARSE;
  }
  const std::string base = base_dir ? base_dir : "";
  f3 hair_lo = mk(0, 0, 0), hair_hi = mk(0, 0, 0);
  bool hair_from_file = false;
  try {
    // ---- surface (head)
    const Json& surf = j["surface"];
    bool has_surface = false, has_hair = false;
    f3 head_r = mk(0.85f, 0.95f, 1.0f);
    if (surf.has("procedural")) {
      const Json& p = surf["procedural"];
      if (p.string_or("type", "ellipsoid") != "ellipsoid") throw JsonError("scene: unknown surface procedural type");
      head_r = f3_of(p["radii"], head_r);
      gen_ellipsoid((int)p.number_or("triangles", 20000), head_r, s);
      s->diffuse = f3_of(p["diffuse"], mk(0.35f, 0.25f, 0.2f));
      s->alpha_raw = (float)p.number_or("alpha", 1.0);
      has_surface = true;
    } else if (surf.has("geometry")) {
      if (int st = load_obj_file(join_path(base, surf["geometry"].as_string()), s)) return st;
      s->diffuse = f3_of(surf["diffuse"], mk(0.35f, 0.25f, 0.2f));
      s->alpha_raw = (float)surf.number_or("alpha", 1.0);
      has_surface = true;
    }
    // ---- hair geometry
    const Json& hair = j["hair"];
    if (hair.has("procedural")) {
      const Json& p = hair["procedural"];
      HairGen g;
      g.type = p.string_or("type", "straight");
      if (g.type != "straight" && g.type != "curly") throw JsonError("scene: hair.procedural.type");
      g.strands = (int)p.number_or("strands", 10000);
      g.cps = (int)p.number_or("control_points", 64);
      g.length = (float)p.number_or("length", 2.0);
      g.radius = (float)p.number_or("radius", 4e-4);
      g.root_min_z = (float)p.number_or("root_min_z", 0.25);
      g.helix_radius = (float)p.number_or("helix_radius", 0.05);
      g.helix_pitch = (float)p.number_or("helix_pitch", 0.1);
      g.seed = (uint32_t)p.number_or("seed", 1);
      if (g.strands < 1 || g.cps < 4 || !(g.length > 0) || !(g.radius > 0)) throw JsonError("scene: bad hair.procedural");
      gen_hair(g, head_r, s);
      has_hair = true;
    } else if (hair.has("geometry")) {
      if (int st = load_hair_file(join_path(base, hair["geometry"].as_string()), s, &hair_lo, &hair_hi)) return st;
      hair_from_file = true;
      has_hair = true;
    }
    if (!has_surface && !has_hair) throw JsonError("scene: either hair or surface must be defined");
    // ---- camera (required)
    const Json& cam = j["camera"];
    if (!cam.is_object() || !cam.has("from") || !cam.has("to") || !cam.has("up") || !cam.has("cos_fovy"))
      throw JsonError("scene: camera must be defined");
    s->cam_from = f3_of(cam["from"], s->cam_from);
    s->cam_at = f3_of(cam["to"], s->cam_at);
    s->cam_up = f3_of(cam["up"], s->cam_up);
    s->cos_fovy = (float)cam["cos_fovy"].as_number();
    // ---- hair BSDF (defaults of scene.cpp:186-231)
    s->hair.sigma_a[0] = 0.06f; s->hair.sigma_a[1] = 0.1f; s->hair.sigma_a[2] = 0.2f;
    s->hair.beta_m = 0.3f;
    s->hair.beta_n = 0.3f;
    s->hair.alpha = 0.03f;  // the Scene default (radians), kept when there is no hair.type
    s->hair.gain_r = s->hair.gain_tt = s->hair.gain_trt = s->hair.gain_trrt = 1.f;
    // parseScene reads the material only after hair.type (its first
    // statement, scene.cpp:188): without it every field keeps the default
    if (hair.has("type") && hair["type"].is_number()) {
      if (hair["sigma_a"].is_array()) {
        f3 sa = f3_of(hair["sigma_a"], mk(0.06f, 0.1f, 0.2f));
        s->hair.sigma_a[0] = sa.x; s->hair.sigma_a[1] = sa.y; s->hair.sigma_a[2] = sa.z;
      }
      s->hair.beta_m = (float)hair.number_or("beta_m", 0.3);
      s->hair.beta_n = (float)hair.number_or("beta_n", 0.3);
      s->hair.alpha = hair.has("alpha") ? 3.14159f * (float)hair["alpha"].as_number() / 180.f : 0.f;
      s->hair.gain_r = (float)hair.number_or("Gain R", 1.0);
      s->hair.gain_tt = (float)hair.number_or("Gain TT", 1.0);
      s->hair.gain_trt = (float)hair.number_or("Gain TRT", 1.0);
      s->hair.gain_trrt = (float)hair.number_or("Gain TRRT", 1.0);
    }
    // ---- strand groups (no reference counterpart): per-group materials
    if (hair.has("groups")) {
      const Json& gj = hair["groups"];
      const int count = (int)gj.number_or("count", 1);
      if (count < 1 || count > kMaxStrandGroups) throw JsonError("scene: hair.groups.count out of range");
      const std::string how = gj.string_or("assign", "azimuth");
      if (how != "azimuth" && how != "index") throw JsonError("scene: hair.groups.assign must be azimuth or index");
      std::vector<int> grp(s->n_strands, 0);
      if (how == "index") {
        for (int k = 0; k < s->n_strands; ++k) grp[k] = k % count;
      } else {
        // azimuth of each strand's root (its second control point) around the
        // mean root, split into `count` equal wedges
        std::vector<f3> root(s->n_strands);
        double cx = 0.0, cy = 0.0;
        for (int k = 0; k < s->n_strands; ++k) {
          const int a = s->strand_seg[k];
          const int cpi = a < (int)s->seg.size() ? s->seg[a] + 1 : 0;
          const float4 c = s->cp.empty() ? make_float4(0, 0, 0, 0) : s->cp[std::min(cpi, (int)s->cp.size() - 1)];
          root[k] = mk(c.x, c.y, c.z);
          cx += c.x;
          cy += c.y;
        }
        cx /= std::max(1, s->n_strands);
        cy /= std::max(1, s->n_strands);
        for (int k = 0; k < s->n_strands; ++k) {
          const double ang = std::atan2((double)root[k].y - cy, (double)root[k].x - cx) + 3.141592653589793;
          grp[k] = std::min(count - 1, (int)(ang / (2.0 * 3.141592653589793) * count));
        }
      }
      std::vector<hm_hair_params> mats(count, s->hair);
      const Json& mj = gj["materials"];
      if (mj.is_array()) {
        if ((int)mj.size() > count) throw JsonError("scene: more hair.groups.materials than groups");
        for (size_t g = 0; g < mj.size(); ++g) {
          const Json& m = mj[g];
          hm_hair_params& p = mats[g];
          if (m["sigma_a"].is_array()) {
            f3 sa = f3_of(m["sigma_a"], mk(p.sigma_a[0], p.sigma_a[1], p.sigma_a[2]));
            p.sigma_a[0] = sa.x; p.sigma_a[1] = sa.y; p.sigma_a[2] = sa.z;
          }
          p.beta_m = (float)m.number_or("beta_m", p.beta_m);
          p.beta_n = (float)m.number_or("beta_n", p.beta_n);
          if (m.has("alpha")) p.alpha = 3.14159f * (float)m["alpha"].as_number() / 180.f;
          p.gain_r = (float)m.number_or("Gain R", p.gain_r);
          p.gain_tt = (float)m.number_or("Gain TT", p.gain_tt);
          p.gain_trt = (float)m.number_or("Gain TRT", p.gain_trt);
          p.gain_trrt = (float)m.number_or("Gain TRRT", p.gain_trrt);
        }
      }
      s->strand_group = grp;
      s->group_mats = mats;
    }
    // ---- lights
    const Json& lights = j["lights"];
    if (lights.has("sky")) {
      const Json& sk = lights["sky"];
      s->env_w = (int)sk.number_or("width", 512);
      s->env_h = (int)sk.number_or("height", 256);
      if (s->env_w < 2 || s->env_h < 2 || s->env_w > 8192 || s->env_h > 8192) throw JsonError("scene: bad sky size");
      bake_sky((float)sk.number_or("turbidity", 3.0), f3_of(sk["sun"], mk(3, 3, 3)), s->env_w, s->env_h,
               (float)sk.number_or("radiance_scale", 1.0), &s->env);
      s->has_env = true;
      s->env_scale = (float)sk.number_or("scale", 1.0);
      s->env_rot_phi = (float)sk.number_or("rotation", 0.0);
    } else if (lights.has("environment")) {
      // parseScene (scene.cpp:234-253): {"exr": path, "scale": s, "rotation": r}
      const Json& ev = lights["environment"];
      const std::string path = join_path(base, ev["exr"].as_string());
      std::string data, err;
      if (!read_file(path, &data)) {
        hm_set_error("scene: cannot read environment map %s", path.c_str());
        return HM_EINVAL;
      }
      if (int st = exr_load_rgba(data, &s->env, &s->env_w, &s->env_h, &err)) {
        hm_set_error("scene: %s: %s", path.c_str(), err.c_str());
        return st;
      }
      s->has_env = true;
      s->env_scale = (float)ev["scale"].as_number();
      s->env_rot_phi = (float)ev.number_or("rotation", 0.0);
    }
    if (lights["directional"].is_array()) {
      for (size_t i = 0; i < lights["directional"].size(); ++i) {
        const Json& d = lights["directional"][i];
        f3 from = normalize(f3_of(d["from"], mk(0, 0, 1)));
        f3 emit = f3_of(d["emit"], mk(1, 1, 1));
        s->dlights.insert(s->dlights.end(), {from.x, from.y, from.z, emit.x, emit.y, emit.z});
      }
    }
    if (!s->has_env && s->dlights.empty()) throw JsonError("scene: either directional or environment light must be defined");
    // ---- integrator (scene.cpp:286-311)
    const Json& in = j["integrator"];
    if (!in.is_object()) throw JsonError("scene: integrator must be defined");
    s->spp = (int)in.number_or("spp", 1);
    s->path_v1 = (int)in.number_or("path_v1", 1);
    s->path_v2 = (int)in.number_or("path_v2", 40);
    s->width = (int)in.number_or("width", 512);
    s->height = (int)in.number_or("height", 512);
    s->mis = in.bool_or("MIS", true);
    s->env_pdf = in.bool_or("ENV_PDF", true);
    s->image_output = in.string_or("image_output", "");
    s->stats_output = in.string_or("stats_output", "");
    s->shading_catrom = in.bool_or("shade_catmull_rom", false) ? 1 : 0;
    // BVH leaves per segment (no reference counterpart: OptiX builds its own
    // curve hierarchy); 2 halves the curve tests per ray (measured 5.2 -> 3.5
    // per extension ray, 10% faster frames) for twice the leaves
    s->seg_split = (int)in.number_or("segment_splits", 2);
    if (s->seg_split != 1 && s->seg_split != 2 && s->seg_split != 4)
      throw JsonError("scene: integrator.segment_splits must be 1, 2 or 4");
    if (s->width <= 0 || s->height <= 0 || (int64_t)s->width * s->height > 2048 * 2048 ||
        ((int64_t)s->width * s->height) % 128 != 0)
      throw JsonError("scene: image size must be at most 2K x 2K and a multiple of 128 pixels");
    if (s->path_v2 < 1 || s->path_v2 > 1024) throw JsonError("scene: path_v2 out of range");
    // ---- cache network (scene.cpp:316-335)
    const Json& tc = j["tcnn"];
    if (tc.is_object()) {
      std::string cfg = tc.string_or("config", "");
      if (!cfg.empty() && !read_file(join_path(base, cfg), &s->cache_config))
        throw JsonError("scene: cannot read tcnn.config " + cfg);
      s->cache_train = tc.bool_or("init_train", false);
      const std::string w = tc.string_or("init_weights", "");  // scene.cpp:330-331
      if (!w.empty()) s->cache_weights = join_path(base, w);
    }
  } catch (const std::exception& e) {
    hm_set_error("%s", e.what());
    return HM_EPARSE;
  }
  // ---- bounds and scale (render_hair_msnn.cu:318-357)
  f3 lo = mk(1e30f, 1e30f, 1e30f), hi = mk(-1e30f, -1e30f, -1e30f);
  for (auto& v : s->vtx) grow(lo, hi, mk(v.x, v.y, v.z));
  float surf_scale = s->vtx.empty() ? 0.f : length(hi - lo);
  f3 hlo = mk(1e30f, 1e30f, 1e30f), hhi = mk(-1e30f, -1e30f, -1e30f);
  if (hair_from_file) {  // extractHairData's bounds: the file's points, not the phantoms
    hlo = hair_lo;
    hhi = hair_hi;
  } else {
    for (auto& c : s->cp) grow(hlo, hhi, mk(c.x, c.y, c.z));
  }
  float hair_scale = s->cp.empty() ? 0.f : length(hhi - hlo);
  if (!s->cp.empty()) {
    grow(lo, hi, hlo);
    grow(lo, hi, hhi);
  }
  s->bmin = lo;
  s->bmax = hi;
  s->scene_scale = fmaxf(hair_scale, surf_scale);
  if (s->has_env) env_sampling_tables(s->env.data(), s->env_w, s->env_h, s->cpdf, s->ccdf, s->mpdf, s->mcdf);
  return HM_OK;
}

template <class T>
static cudaError_t up(T** d, const std::vector<T>& h) {
  if (h.empty()) return cudaSuccess;
  cudaError_t e = cudaMalloc(d, h.size() * sizeof(T));
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
}

int Scene::upload() {
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = up(&d_cp, cp);
  if (e == cudaSuccess) e = up(&d_seg, seg);
  if (e == cudaSuccess) e = up(&d_vtx, vtx);
  if (e == cudaSuccess) e = up(&d_nrm, nrm);
  if (e == cudaSuccess) e = up(&d_tri, tri);
  if (e == cudaSuccess) e = up(&d_env, env);
  if (e == cudaSuccess) e = up(&d_cpdf, cpdf);
  if (e == cudaSuccess) e = up(&d_ccdf, ccdf);
  if (e == cudaSuccess) e = up(&d_mpdf, mpdf);
  if (e == cudaSuccess) e = up(&d_mcdf, mcdf);
  if (e == cudaSuccess) e = up(&d_dlights, dlights);
  return e == cudaSuccess ? HM_OK : hm_cuda_status(e, "scene upload");
}

Scene::~Scene() {
  cudaFree(d_cp); cudaFree(d_seg); cudaFree(d_vtx); cudaFree(d_nrm); cudaFree(d_tri);
  cudaFree(d_env); cudaFree(d_cpdf); cudaFree(d_ccdf); cudaFree(d_mpdf); cudaFree(d_mcdf);
  cudaFree(d_dlights); cudaFree(d_nodes); cudaFree(d_prim_of_leaf); cudaFree(d_wnodes);
  cudaFree(d_seg_group); cudaFree(d_group_hc); cudaFree(d_group_raw);
}

// Strand groups: every segment takes its strand's group.
int Scene::set_strand_groups(const int* groups, int n, int ng) {
  if (n != n_strands) return hm_set_error("strand groups: %d entries for %d strands", n, n_strands), HM_EINVAL;
  if (ng < 1 || ng > kMaxStrandGroups) return hm_set_error("strand groups: 1..%d groups", kMaxStrandGroups), HM_EINVAL;
  for (int k = 0; k < n; ++k)
    if (groups[k] < 0 || groups[k] >= ng) return hm_set_error("strand groups: group %d of strand %d", groups[k], k), HM_EINVAL;
  strand_group.assign(groups, groups + n);
  if ((int)group_mats.size() != ng) group_mats.assign(ng, hair);
  ++material_version;
  return built ? upload_groups() : HM_OK;
}

int Scene::set_group_materials(const hm_hair_params* m, int n) {
  if (group_mats.empty()) {
    if (n != 1) return hm_set_error("group materials: the scene has one material"), HM_EINVAL;
    hair = m[0];
    ++material_version;
    return HM_OK;
  }
  if (n != (int)group_mats.size())
    return hm_set_error("group materials: %d given for %d groups", n, (int)group_mats.size()), HM_EINVAL;
  group_mats.assign(m, m + n);
  ++material_version;
  return built ? upload_groups() : HM_OK;
}

// Device tables of the groups.  Frames in flight may read them: wait first.
int Scene::upload_groups() {
  if (group_mats.empty()) return HM_OK;
  cudaError_t e = cudaDeviceSynchronize();
  const int ng = (int)group_mats.size();
  if (e == cudaSuccess && !d_seg_group) e = cudaMalloc(&d_seg_group, std::max<size_t>(1, seg.size()));
  if (e == cudaSuccess && !d_group_hc) e = cudaMalloc(&d_group_hc, kMaxStrandGroups * sizeof(HairConsts));
  if (e == cudaSuccess && !d_group_raw) e = cudaMalloc(&d_group_raw, kMaxStrandGroups * sizeof(hm_hair_params));
  if (e != cudaSuccess) return hm_cuda_status(e, "strand group tables");
  seg_group_host.assign(seg.size(), 0);
  if (!strand_group.empty())
    for (int k = 0; k < n_strands; ++k)
      for (int i = strand_seg[k]; i < strand_seg[k + 1]; ++i) seg_group_host[i] = strand_group[k];
  std::vector<uint8_t> sg(seg_group_host.begin(), seg_group_host.end());
  std::vector<HairConsts> hc(ng);
  for (int g = 0; g < ng; ++g) hc[g] = hair_consts_from_params(group_mats[g]);
  if (!sg.empty()) e = cudaMemcpy(d_seg_group, sg.data(), sg.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d_group_hc, hc.data(), ng * sizeof(HairConsts), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(d_group_raw, group_mats.data(), ng * sizeof(hm_hair_params), cudaMemcpyHostToDevice);
  return e == cudaSuccess ? HM_OK : hm_cuda_status(e, "strand group upload");
}

SceneDev Scene::dev() const {
  SceneDev d{};
  d.cp = d_cp;
  d.seg = d_seg;
  d.n_seg = (int)seg.size();
  d.seg_split = seg_split;
  d.n_hprim = d.n_seg * seg_split;
  d.shading_catrom = shading_catrom;
  d.vtx = d_vtx;
  d.nrm = d_nrm;
  d.tri = d_tri;
  d.n_tri = (int)tri.size();
  d.diffuse = diffuse;
  float a = fminf(fmaxf(alpha_raw, 0.01f), 1.f);  // triangleMeshCH, optix_common.cuh:551-552
  d.alpha = a * a;
  d.nodes = d_nodes;
  d.n_nodes = n_nodes;
  d.prim_of_leaf = d_prim_of_leaf;
  d.wnodes = d_wnodes;
  d.n_wnodes = n_wnodes;
  d.has_env = has_env;
  d.env_pdf_sampling = env_pdf;
  d.env = d_env;
  d.env_w = env_w;
  d.env_h = env_h;
  d.cpdf = d_cpdf;
  d.ccdf = d_ccdf;
  d.mpdf = d_mpdf;
  d.mcdf = d_mcdf;
  d.env_scale = env_scale;
  d.env_rot_phi = env_rot_phi;
  d.n_dlights = (int)(dlights.size() / 6);
  d.dlights = d_dlights;
  d.n_total_lights = d.n_dlights + (has_env ? 1 : 0);
  // cameraChanged (render_hair_msnn.cu:1093-1118)
  f3 d00 = normalize(cam_at - cam_from);
  float aspect = (float)width / (float)height;
  f3 ddu = cos_fovy * aspect * normalize(cross(d00, cam_up));
  f3 ddv = cos_fovy * normalize(cross(ddu, d00));
  d00 = d00 - 0.5f * ddu;
  d00 = d00 - 0.5f * ddv;
  d.cam_pos = cam_from;
  d.cam_d00 = d00;
  d.cam_du = ddu;
  d.cam_dv = ddv;
  d.hair = hair_consts_from_params(hair);
  d.hair_raw = hair;
  if (!group_mats.empty() && d_seg_group) {
    d.seg_group = d_seg_group;
    d.group_hc = d_group_hc;
    d.group_raw = d_group_raw;
    d.n_groups = (int)group_mats.size();
  }
  d.mis = mis;
  d.width = width;
  d.height = height;
  d.path_v1 = path_v1;
  d.path_v2 = path_v2;
  d.scene_scale = scene_scale;
  return d;
}

}  // namespace hm

using namespace hm;

namespace hm {
int Scene::ensure_built() {
  if (built) return HM_OK;
  int st = upload();
  if (st == HM_OK) st = upload_groups();
  if (st == HM_OK) st = build_bvh(0);
  if (st == HM_OK) {
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) st = hm_cuda_status(e, "scene build");
  }
  if (st == HM_OK) built = true;
  return st;
}
}  // namespace hm

// Parses and generates on the host only; device copies and the LBVH are made
// by hm_scene_build (or on first use by a render / trace call).
extern "C" hm_scene* hm_scene_create(const char* json_text, const char* base_dir, int* status) {
  int dummy;
  if (!status) status = &dummy;
  Scene* s = new Scene();
  int st = scene_from_json(json_text, base_dir, s);
  *status = st;
  if (st != HM_OK) {
    delete s;
    return nullptr;
  }
  return (hm_scene*)s;
}

extern "C" int hm_scene_build(hm_scene* h) {
  Scene* s = (Scene*)h;
  if (!s) return hm_set_error("hm_scene_build: NULL"), HM_EINVAL;
  return s->ensure_built();
}

extern "C" void hm_scene_destroy(hm_scene* h) { delete (Scene*)h; }

extern "C" int hm_scene_info(const hm_scene* h, hm_scene_desc* out) {
  const Scene* s = (const Scene*)h;
  if (!s || !out) return hm_set_error("hm_scene_info: NULL"), HM_EINVAL;
  memset(out, 0, sizeof(*out));
  out->n_strands = s->n_strands;
  out->n_control_points = (int)s->cp.size();
  out->n_segments = (int)s->seg.size();
  out->n_vertices = (int)s->vtx.size();
  out->n_triangles = (int)s->tri.size();
  out->n_bvh_nodes = s->n_nodes;
  out->n_bvh_wide_nodes = s->n_wnodes;
  out->n_groups = s->group_mats.empty() ? 0 : (int)s->group_mats.size();
  out->segment_splits = s->seg_split;
  out->width = s->width;
  out->height = s->height;
  out->spp = s->spp;
  out->path_v1 = s->path_v1;
  out->path_v2 = s->path_v2;
  out->env_width = s->env_w;
  out->env_height = s->env_h;
  out->n_dir_lights = (int)(s->dlights.size() / 6);
  out->mis = s->mis;
  out->env_pdf = s->env_pdf;
  out->has_env = s->has_env;
  out->shading_catrom = s->shading_catrom;
  out->scene_scale = s->scene_scale;
  out->bounds_min[0] = s->bmin.x; out->bounds_min[1] = s->bmin.y; out->bounds_min[2] = s->bmin.z;
  out->bounds_max[0] = s->bmax.x; out->bounds_max[1] = s->bmax.y; out->bounds_max[2] = s->bmax.z;
  return HM_OK;
}

template <class T>
static int export_vec(const std::vector<T>& v, void* out, int64_t cap) {
  int64_t bytes = (int64_t)(v.size() * sizeof(T));
  if (!out) return (int)HM_OK;
  if (cap < bytes) return hm_set_error("hm_scene_export: buffer too small (%lld < %lld)", (long long)cap, (long long)bytes), HM_ECAPACITY;
  if (bytes) memcpy(out, v.data(), bytes);
  return HM_OK;
}

extern "C" int64_t hm_scene_export_size(const hm_scene* h, int which) {
  const Scene* s = (const Scene*)h;
  if (!s) return -1;
  switch (which) {
    case HM_SCENE_CONTROL_POINTS: return (int64_t)s->cp.size() * 16;
    case HM_SCENE_SEGMENTS: return (int64_t)s->seg.size() * 4;
    case HM_SCENE_VERTICES: return (int64_t)s->vtx.size() * 12;
    case HM_SCENE_NORMALS: return (int64_t)s->nrm.size() * 12;
    case HM_SCENE_TRIANGLES: return (int64_t)s->tri.size() * 12;
    case HM_SCENE_ENV: return (int64_t)s->env.size() * 16;
    case HM_SCENE_ENV_CPDF: return (int64_t)s->cpdf.size() * 4;
    case HM_SCENE_ENV_CCDF: return (int64_t)s->ccdf.size() * 4;
    case HM_SCENE_ENV_MPDF: return (int64_t)s->mpdf.size() * 4;
    case HM_SCENE_ENV_MCDF: return (int64_t)s->mcdf.size() * 4;
    case HM_SCENE_DIR_LIGHTS: return (int64_t)s->dlights.size() * 4;
    case HM_SCENE_BVH_NODES: return (int64_t)s->n_nodes * 64;
    case HM_SCENE_BVH_LEAVES: return (int64_t)s->n_prims() * 4;
    case HM_SCENE_BVH_WIDE_NODES: return (int64_t)s->n_wnodes * kWideNodeBytes;
    case HM_SCENE_CAMERA: return 12 * 4;
    case HM_SCENE_MATERIALS: return 16 * 4;
    case HM_SCENE_STRAND_GROUPS: return (int64_t)s->strand_group.size() * 4;
    case HM_SCENE_GROUP_MATERIALS: return (int64_t)s->group_mats.size() * (int64_t)sizeof(hm_hair_params);
    case HM_SCENE_SEGMENT_GROUPS: return s->group_mats.empty() ? 0 : (int64_t)s->seg.size() * 4;
    default: return -1;
  }
}

extern "C" int hm_scene_export(const hm_scene* h, int which, void* out, int64_t cap) {
  const Scene* s = (const Scene*)h;
  if (!s || !out) return hm_set_error("hm_scene_export: NULL"), HM_EINVAL;
  switch (which) {
    case HM_SCENE_CONTROL_POINTS: return export_vec(s->cp, out, cap);
    case HM_SCENE_SEGMENTS: return export_vec(s->seg, out, cap);
    case HM_SCENE_VERTICES: return export_vec(s->vtx, out, cap);
    case HM_SCENE_NORMALS: return export_vec(s->nrm, out, cap);
    case HM_SCENE_TRIANGLES: return export_vec(s->tri, out, cap);
    case HM_SCENE_ENV: return export_vec(s->env, out, cap);
    case HM_SCENE_ENV_CPDF: return export_vec(s->cpdf, out, cap);
    case HM_SCENE_ENV_CCDF: return export_vec(s->ccdf, out, cap);
    case HM_SCENE_ENV_MPDF: return export_vec(s->mpdf, out, cap);
    case HM_SCENE_ENV_MCDF: return export_vec(s->mcdf, out, cap);
    case HM_SCENE_DIR_LIGHTS: return export_vec(s->dlights, out, cap);
    case HM_SCENE_STRAND_GROUPS: return export_vec(s->strand_group, out, cap);
    case HM_SCENE_GROUP_MATERIALS: return export_vec(s->group_mats, out, cap);
    case HM_SCENE_SEGMENT_GROUPS: {
      if (s->group_mats.empty()) return HM_OK;
      std::vector<int> sg(s->seg.size(), 0);
      if (!s->strand_group.empty())
        for (int k = 0; k < s->n_strands; ++k)
          for (int i = s->strand_seg[k]; i < s->strand_seg[k + 1]; ++i) sg[i] = s->strand_group[k];
      return export_vec(sg, out, cap);
    }
    case HM_SCENE_BVH_NODES:
    case HM_SCENE_BVH_LEAVES:
    case HM_SCENE_BVH_WIDE_NODES: {
      if (!s->built) return hm_set_error("hm_scene_export: call hm_scene_build first"), HM_EINVAL;
      int64_t bytes = which == HM_SCENE_BVH_NODES ? (int64_t)s->n_nodes * 64
                      : which == HM_SCENE_BVH_LEAVES ? (int64_t)s->n_prims() * 4 : (int64_t)s->n_wnodes * kWideNodeBytes;
      if (cap < bytes) return hm_set_error("hm_scene_export: buffer too small"), HM_ECAPACITY;
      const void* src = which == HM_SCENE_BVH_NODES ? (const void*)s->d_nodes
                        : which == HM_SCENE_BVH_LEAVES ? (const void*)s->d_prim_of_leaf : (const void*)s->d_wnodes;
      if (!bytes) return HM_OK;
      cudaError_t e = cudaMemcpy(out, src, bytes, cudaMemcpyDeviceToHost);
      return e == cudaSuccess ? HM_OK : hm_cuda_status(e, "hm_scene_export bvh");
    }
    case HM_SCENE_CAMERA: {
      if (cap < 48) return HM_ECAPACITY;
      SceneDev d = s->dev();
      float c[12] = {d.cam_pos.x, d.cam_pos.y, d.cam_pos.z, d.cam_d00.x, d.cam_d00.y, d.cam_d00.z,
                     d.cam_du.x, d.cam_du.y, d.cam_du.z, d.cam_dv.x, d.cam_dv.y, d.cam_dv.z};
      memcpy(out, c, sizeof(c));
      return HM_OK;
    }
    case HM_SCENE_MATERIALS: {
      if (cap < 64) return HM_ECAPACITY;
      float m[16] = {s->hair.sigma_a[0], s->hair.sigma_a[1], s->hair.sigma_a[2], s->hair.beta_m, s->hair.beta_n,
                     s->hair.alpha, s->hair.gain_r, s->hair.gain_tt, s->hair.gain_trt, s->hair.gain_trrt,
                     s->diffuse.x, s->diffuse.y, s->diffuse.z, s->alpha_raw, s->env_scale, s->env_rot_phi};
      memcpy(out, m, sizeof(m));
      return HM_OK;
    }
    default:
      return hm_set_error("hm_scene_export: unknown array %d", which), HM_EINVAL;
  }
}

extern "C" int hm_scene_set_strand_groups(hm_scene* h, const int32_t* groups, int n_strands, int n_groups) {
  Scene* s = (Scene*)h;
  if (!s || (!groups && n_strands)) return hm_set_error("hm_scene_set_strand_groups: NULL"), HM_EINVAL;
  return s->set_strand_groups(groups, n_strands, n_groups);
}

extern "C" int hm_scene_set_group_materials(hm_scene* h, const hm_hair_params* materials, int n_groups) {
  Scene* s = (Scene*)h;
  if (!s || !materials) return hm_set_error("hm_scene_set_group_materials: NULL"), HM_EINVAL;
  return s->set_group_materials(materials, n_groups);
}
