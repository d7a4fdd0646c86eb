// ORACLE geometry + integrator (test infrastructure only).
//
// * LBVH: the same algorithm as the device build (AABBs, 30-bit Morton codes
//   of box centres in the scene box, unique 64-bit keys code<<32|id, Karras
//   2012 radix tree, child boxes stored in the parent) on the host; the node
//   array must match the device's bit for bit.
// * Traversal and intersection: the same closest-hit / any-hit traversal and
//   the same ray-space cubic and Moller-Trumbore intersectors, FP32 without
//   multiply-add contraction (the device build contracts: hits are compared
//   with a tolerance).
// * Integrator: written in the reference's own per-pixel loop structure -
//   rayGenCam, msnnPathTrace, msnnTrainingPath, pathTrace, directLighting,
//   sampleLights, sampleBSDF, msnnNextPathVertex, hairCH, triangleMeshCH, miss
//   (cuda/hair_msnn.cu:17-312, cuda/path_tracing.cu:19-66,
//   cuda_headers/optix_common.cuh:10-616) - so it independently checks the
//   wavefront restructuring of the device path.  The training-pixel choice
//   uses the library's keyed Feistel permutation (the reference's
//   thrust::shuffle is not reproducible).
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <thread>
#include <memory>
#include <vector>

#include "hm_oracle_math.h"

using namespace hmo;

namespace {

struct Box {
  float lo[3], hi[3];
};

struct OScene {
  std::vector<float> cp;  // [n_cp][4]
  std::vector<int> seg;
  std::vector<float> vtx, nrm;  // [n][3]
  std::vector<int> tri;         // [n][3]
  std::vector<float> env;       // [H][W][4]
  int env_w = 0, env_h = 0;
  std::vector<float> cpdf, ccdf, mpdf, mcdf;
  std::vector<float> dl;  // [n][6]
  V3 cam_pos, cam_d00, cam_du, cam_dv;
  float hp[10];
  HairShading hs;
  // strand groups: group of every segment and the groups' materials (empty:
  // every segment uses hs)
  std::vector<int> seg_group;
  std::vector<HairShading> ghs;
  V3 diffuse;
  float alpha;  // clamp(alpha,.01,1)^2
  float env_scale = 1.f, env_rot = 0.f;
  int width = 0, height = 0, path_v1 = 1, path_v2 = 40, mis = 1, env_pdf = 1, has_env = 0, catrom = 0;
  int seg_split = 1;  // BVH leaves per segment: part j of segment k is leaf primitive k + j * n_seg
  float scene_scale = 1.f;
  // BVH
  std::vector<float> nodes;  // [n_int][16]
  std::vector<int> leaf_prim;
  int n_seg() const { return (int)seg.size(); }
  int n_hprim() const { return (int)seg.size() * seg_split; }
  int n_prims() const { return n_hprim() + (int)tri.size() / 3; }
  int n_dl() const { return (int)dl.size() / 6; }
};

// ------------------------------------------------------------ BVH build
// One de Casteljau halving (left or right half) of a cubic Bezier.
void bezier_half(float w[4][4], int right) {
  for (int k = 0; k < 4; ++k) {
    const float m01 = (w[0][k] + w[1][k]) * 0.5f, m12 = (w[1][k] + w[2][k]) * 0.5f;
    const float m23 = (w[2][k] + w[3][k]) * 0.5f;
    const float m012 = (m01 + m12) * 0.5f, m123 = (m12 + m23) * 0.5f, m = (m012 + m123) * 0.5f;
    if (right) {
      w[0][k] = m; w[1][k] = m123; w[2][k] = m23;
    } else {
      w[1][k] = m01; w[2][k] = m012; w[3][k] = m;
    }
  }
}

Box prim_box(const OScene& s, int p) {
  Box b;
  if (p < s.n_hprim()) {
    // hull of the Bezier control points of the segment's part, grown by
    // their largest radius (same operation order as the device build)
    const int part = p / s.n_seg();
    const float* c = &s.cp[4 * s.seg[p - part * s.n_seg()]];
    float w[4][4];
    for (int k = 0; k < 4; ++k) {
      const float q0 = c[k], q1 = c[4 + k], q2 = c[8 + k], q3 = c[12 + k];
      w[0][k] = ((q0 + 4.f * q1) + q2) * (1.f / 6.f);
      w[1][k] = (2.f * q1 + q2) * (1.f / 3.f);
      w[2][k] = (q1 + 2.f * q2) * (1.f / 3.f);
      w[3][k] = ((q1 + 4.f * q2) + q3) * (1.f / 6.f);
    }
    for (int bit = s.seg_split >> 1; bit > 0; bit >>= 1) bezier_half(w, part & bit);
    const float r = fmaxf(fmaxf(w[0][3], w[1][3]), fmaxf(w[2][3], w[3][3]));
    for (int k = 0; k < 3; ++k) {
      b.lo[k] = fminf(fminf(w[0][k], w[1][k]), fminf(w[2][k], w[3][k])) - r;
      b.hi[k] = fmaxf(fmaxf(w[0][k], w[1][k]), fmaxf(w[2][k], w[3][k])) + r;
    }
  } else {
    const int* t = &s.tri[3 * (p - s.n_hprim())];
    const float *a = &s.vtx[3 * t[0]], *bb = &s.vtx[3 * t[1]], *c = &s.vtx[3 * t[2]];
    for (int k = 0; k < 3; ++k) {
      b.lo[k] = fminf(fminf(a[k], bb[k]), c[k]);
      b.hi[k] = fmaxf(fmaxf(a[k], bb[k]), c[k]);
    }
  }
  return b;
}

uint32_t expand_bits10(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

int delta(const std::vector<uint64_t>& k, int i, int j) {
  if (j < 0 || j >= (int)k.size()) return -1;
  return __builtin_clzll(k[i] ^ k[j]);
}

void build_bvh(OScene& s) {
  const int n = s.n_prims();
  const int n_int = std::max(1, n - 1);
  s.nodes.assign((size_t)n_int * 16, 0.f);
  s.leaf_prim.assign(n, 0);
  std::vector<Box> boxes(n);
  float slo[3] = {INFINITY, INFINITY, INFINITY}, shi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int p = 0; p < n; ++p) {
    boxes[p] = prim_box(s, p);
    for (int k = 0; k < 3; ++k) {
      slo[k] = fminf(slo[k], boxes[p].lo[k]);
      shi[k] = fmaxf(shi[k], boxes[p].hi[k]);
    }
  }
  auto write_slot = [&](int node, int slot, const Box& b) {
    float* f = &s.nodes[16 * node + 6 * slot];
    for (int k = 0; k < 3; ++k) {
      f[k] = b.lo[k];
      f[3 + k] = b.hi[k];
    }
  };
  auto set_children = [&](int node, int c0, int c1) {
    memcpy(&s.nodes[16 * node + 12], &c0, 4);
    memcpy(&s.nodes[16 * node + 13], &c1, 4);
  };
  if (n == 1) {
    write_slot(0, 0, boxes[0]);
    Box e;
    for (int k = 0; k < 3; ++k) {
      e.lo[k] = INFINITY;
      e.hi[k] = -INFINITY;
    }
    write_slot(0, 1, e);
    set_children(0, ~0, ~0);
    s.leaf_prim[0] = 0;
    return;
  }
  std::vector<uint64_t> keys(n);
  for (int p = 0; p < n; ++p) {
    uint32_t q[3];
    for (int k = 0; k < 3; ++k) {
      float c = (boxes[p].lo[k] + boxes[p].hi[k]) * 0.5f;
      float ext = shi[k] - slo[k];
      float qq = ext > 0.f ? (c - slo[k]) / ext : 0.f;
      float v = fminf(fmaxf(qq * 1024.f, 0.f), 1023.f);
      q[k] = (uint32_t)v;
    }
    uint32_t code = (expand_bits10(q[0]) << 2) | (expand_bits10(q[1]) << 1) | expand_bits10(q[2]);
    keys[p] = ((uint64_t)code << 32) | (uint32_t)p;
  }
  std::sort(keys.begin(), keys.end());
  std::vector<int> c0(n_int), c1(n_int);
  for (int i = 0; i < n - 1; ++i) {
    int d = (delta(keys, i, i + 1) - delta(keys, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta(keys, i, i - d);
    int lmax = 2;
    while (delta(keys, i, i + lmax * d) > dmin) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
      if (delta(keys, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = delta(keys, i, j);
    int sp = 0;
    for (int div = 2;; div *= 2) {
      int t = (l + div - 1) / div;
      if (delta(keys, i, i + (sp + t) * d) > dnode) sp += t;
      if (t <= 1) break;
    }
    int gamma = i + sp * d + std::min(d, 0);
    int lo = std::min(i, j), hi = std::max(i, j);
    c0[i] = lo == gamma ? ~gamma : gamma;
    c1[i] = hi == gamma + 1 ? ~(gamma + 1) : gamma + 1;
  }
  for (int leaf = 0; leaf < n; ++leaf) s.leaf_prim[leaf] = (int)(keys[leaf] & 0xffffffffu);
  // post-order refit (iterative)
  std::vector<Box> nb(n_int);
  std::vector<int> stack;
  std::vector<char> state(n_int, 0);
  stack.push_back(0);
  auto child_box = [&](int c) { return c < 0 ? boxes[s.leaf_prim[~c]] : nb[c]; };
  while (!stack.empty()) {
    int v = stack.back();
    if (!state[v]) {
      state[v] = 1;
      if (c1[v] >= 0) stack.push_back(c1[v]);
      if (c0[v] >= 0) stack.push_back(c0[v]);
      continue;
    }
    stack.pop_back();
    Box a = child_box(c0[v]), b = child_box(c1[v]);
    write_slot(v, 0, a);
    write_slot(v, 1, b);
    set_children(v, c0[v], c1[v]);
    for (int k = 0; k < 3; ++k) {
      nb[v].lo[k] = fminf(a.lo[k], b.lo[k]);
      nb[v].hi[k] = fmaxf(a.hi[k], b.hi[k]);
    }
  }
}

// ------------------------------------------------------------ traversal
struct OHit {
  float t;
  int prim;
  float u, v;
};

bool tri_hit(const OScene& s, int ti, V3 o, V3 d, float tmin, float tmax, float* t_out, float* u_out, float* v_out) {
  const int* tv = &s.tri[3 * ti];
  V3 v0(s.vtx[3 * tv[0]], s.vtx[3 * tv[0] + 1], s.vtx[3 * tv[0] + 2]);
  V3 v1(s.vtx[3 * tv[1]], s.vtx[3 * tv[1] + 1], s.vtx[3 * tv[1] + 2]);
  V3 v2(s.vtx[3 * tv[2]], s.vtx[3 * tv[2] + 1], s.vtx[3 * tv[2] + 2]);
  V3 e1 = v1 - v0, e2 = v2 - v0;
  V3 pv = cross(d, e2);
  float det = dot(e1, pv);
  if (fabsf(det) < 1e-20f) return false;
  float inv = 1.f / det;
  V3 tv0 = o - v0;
  float u = dot(tv0, pv) * inv;
  if (u < 0.f || u > 1.f) return false;
  V3 qv = cross(tv0, e1);
  float v = dot(d, qv) * inv;
  if (v < 0.f || u + v > 1.f) return false;
  float t = dot(e2, qv) * inv;
  if (!(t > tmin && t < tmax)) return false;
  *t_out = t;
  *u_out = u;
  *v_out = v;
  return true;
}

struct P4 {
  float x, y, z, r;
};

bool curve_hit(const OScene& s, int si, int part, V3 o, V3 d, float tmin, float tmax, float* t_out, float* u_out) {
  const float* q = &s.cp[4 * s.seg[si]];
  float w[4][4];
  for (int c = 0; c < 4; ++c) {
    w[0][c] = (q[c] + 4.f * q[4 + c] + q[8 + c]) * (1.f / 6.f);
    w[1][c] = (2.f * q[4 + c] + q[8 + c]) * (1.f / 3.f);
    w[2][c] = (q[4 + c] + 2.f * q[8 + c]) * (1.f / 3.f);
    w[3][c] = (q[4 + c] + 4.f * q[8 + c] + q[12 + c]) * (1.f / 6.f);
  }
  const float sign = copysignf(1.f, d.z);
  const float k = -1.f / (sign + d.z);
  const float m = d.x * d.y * k;
  V3 ax(1.f + sign * d.x * d.x * k, sign * m, -sign * d.x);
  V3 ay(m, sign + d.y * d.y * k, -d.y);
  P4 b[4];
  for (int i = 0; i < 4; ++i) {
    V3 p = V3(w[i][0], w[i][1], w[i][2]) - o;
    b[i] = P4{dot(p, ax), dot(p, ay), dot(p, d), w[i][3]};
  }
  for (int bit = s.seg_split >> 1; bit > 0; bit >>= 1) {  // down to the part (de Casteljau halvings)
    auto mid = [](P4 a, P4 c) { return P4{(a.x + c.x) * 0.5f, (a.y + c.y) * 0.5f, (a.z + c.z) * 0.5f, (a.r + c.r) * 0.5f}; };
    P4 m01 = mid(b[0], b[1]), m12 = mid(b[1], b[2]), m23 = mid(b[2], b[3]);
    P4 m012 = mid(m01, m12), m123 = mid(m12, m23), m = mid(m012, m123);
    if (part & bit) {
      b[0] = m; b[1] = m123; b[2] = m23;
    } else {
      b[1] = m01; b[2] = m012; b[3] = m;
    }
  }
  float rmax = fmaxf(fmaxf(b[0].r, b[1].r), fmaxf(b[2].r, b[3].r));
  auto mn = [&](float P4::*f) { return fminf(fminf(b[0].*f, b[1].*f), fminf(b[2].*f, b[3].*f)); };
  auto mx = [&](float P4::*f) { return fmaxf(fmaxf(b[0].*f, b[1].*f), fmaxf(b[2].*f, b[3].*f)); };
  if (mn(&P4::x) - rmax > 0.f || mx(&P4::x) + rmax < 0.f || mn(&P4::y) - rmax > 0.f || mx(&P4::y) + rmax < 0.f ||
      mx(&P4::z) + rmax < tmin || mn(&P4::z) - rmax > tmax)
    return false;
  float l0 = fmaxf(fmaxf(fabsf(b[0].x - 2.f * b[1].x + b[2].x), fabsf(b[0].y - 2.f * b[1].y + b[2].y)),
                   fmaxf(fabsf(b[1].x - 2.f * b[2].x + b[3].x), fabsf(b[1].y - 2.f * b[2].y + b[3].y)));
  float eps = fmaxf(rmax * 0.1f, 1e-12f);
  float fr = 1.41421356f * 6.f * l0 / (8.f * eps);
  int depth = fr > 1.f ? (int)lrintf(0.5f * log2f(fr)) : 0;
  depth = std::min(std::max(depth, 0), 5);
  int np = 1 << depth;
  float inv_np = 1.f / (float)np;
  bool found = false;
  float best_t = tmax, best_u = 0.f;
  P4 a = b[0];
  for (int kk = 0; kk < np; ++kk) {
    float tt = (float)(kk + 1) * inv_np, s1 = 1.f - tt;
    float c0 = s1 * s1 * s1, c1 = 3.f * s1 * s1 * tt, c2 = 3.f * s1 * tt * tt, c3 = tt * tt * tt;
    P4 e{c0 * b[0].x + c1 * b[1].x + c2 * b[2].x + c3 * b[3].x, c0 * b[0].y + c1 * b[1].y + c2 * b[2].y + c3 * b[3].y,
         c0 * b[0].z + c1 * b[1].z + c2 * b[2].z + c3 * b[3].z, c0 * b[0].r + c1 * b[1].r + c2 * b[2].r + c3 * b[3].r};
    float sx = e.x - a.x, sy = e.y - a.y;
    float len2 = sx * sx + sy * sy;
    if (len2 > 0.f) {
      float ww = -(a.x * sx + a.y * sy) / len2;
      if (ww >= 0.f && ww < 1.f) {
        P4 pc{a.x + (e.x - a.x) * ww, a.y + (e.y - a.y) * ww, a.z + (e.z - a.z) * ww, a.r + (e.r - a.r) * ww};
        float d2 = pc.x * pc.x + pc.y * pc.y, rr = pc.r * pc.r;
        if (d2 < rr) {
          float t = pc.z - sqrtf(rr - d2);
          if (t > tmin && t < best_t) {
            best_t = t;
            best_u = ((float)kk + ww) * inv_np;
            found = true;
          }
        }
      }
    }
    a = e;
  }
  if (found) {
    *t_out = best_t;
    *u_out = ((float)part + best_u) * (1.f / (float)s.seg_split);
  }
  return found;
}

OHit trace(const OScene& s, V3 o, V3 d, float tmin, float tmax, bool any) {
  OHit h{tmax, -1, 0.f, 0.f};
  auto inv1 = [](float x) { return fabsf(x) > 1e-20f ? 1.f / x : copysignf(1e20f, x); };
  V3 inv(inv1(d.x), inv1(d.y), inv1(d.z));
  int stack[64];
  int sp = 0, node = 0;
  auto test = [&](const float* f, float* t0, float* t1) {
    for (int c = 0; c < 2; ++c) {
      const float* b = f + 6 * c;
      float tx0 = (b[0] - o.x) * inv.x, tx1 = (b[3] - o.x) * inv.x;
      float ty0 = (b[1] - o.y) * inv.y, ty1 = (b[4] - o.y) * inv.y;
      float tz0 = (b[2] - o.z) * inv.z, tz1 = (b[5] - o.z) * inv.z;
      float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), tmin));
      float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), h.t));
      (c == 0 ? *t0 : *t1) = tn <= tf ? tn : INFINITY;
    }
  };
  // a leaf primitive; *id = the segment, or n_seg + the triangle
  auto prim_hit = [&](int prim, float* t, float* u, float* v, int* id) {
    if (prim < s.n_hprim()) {
      *v = 0.f;
      const int part = prim / s.n_seg();
      *id = prim - part * s.n_seg();
      return curve_hit(s, *id, part, o, d, tmin, h.t, t, u);
    }
    *id = s.n_seg() + (prim - s.n_hprim());
    return tri_hit(s, prim - s.n_hprim(), o, d, tmin, h.t, t, u, v);
  };
  for (int guard = 0; guard < (1 << 22); ++guard) {
    const float* f = &s.nodes[16 * node];
    float t0, t1;
    test(f, &t0, &t1);
    int c0, c1;
    memcpy(&c0, f + 12, 4);
    memcpy(&c1, f + 13, 4);
    if (c0 < 0 && t0 < INFINITY) {
      float t, u, v;
      int id;
      if (prim_hit(s.leaf_prim[~c0], &t, &u, &v, &id)) {
        h = OHit{t, id, u, v};
        if (any) return h;
      }
      t0 = INFINITY;
      if (t1 > h.t) t1 = INFINITY;
    }
    if (c1 < 0 && t1 < INFINITY) {
      float t, u, v;
      int id;
      if (prim_hit(s.leaf_prim[~c1], &t, &u, &v, &id)) {
        h = OHit{t, id, u, v};
        if (any) return h;
      }
      t1 = INFINITY;
      if (t0 > h.t) t0 = INFINITY;
    }
    bool g0 = t0 < INFINITY, g1 = t1 < INFINITY;
    if (g0 && g1) {
      int nr = t0 <= t1 ? c0 : c1, fr = t0 <= t1 ? c1 : c0;
      if (sp >= 64) return h;
      stack[sp++] = fr;
      node = nr;
    } else if (g0) {
      node = c0;
    } else if (g1) {
      node = c1;
    } else {
      if (sp == 0) return h;
      node = stack[--sp];
    }
  }
  return h;
}

// ------------------------------------------------------------ integrator (reference structure)
struct SI {
  bool hit = false, surface = true;
  V3 Le, p, wo, wi, wo_local, wi_local, n, t;
  V3 to_local[3], to_world[3];
  float radius = 0.f;
  int group = 0;  // strand group of a hair hit
};

const HairShading& hair_of(const OScene& s, const SI& si) { return s.ghs.empty() ? s.hs : s.ghs[si.group]; }

float tex_nearest(const std::vector<float>& t, int w, int h, float u, float v) {
  int x = std::min(std::max((int)floorf(u * (float)w), 0), w - 1);
  int y = std::min(std::max((int)floorf(v * (float)h), 0), h - 1);
  return t[(size_t)y * w + x];
}
V3 tex_linear(const OScene& s, float u, float v) {
  float xb = u * (float)s.env_w - 0.5f, yb = v * (float)s.env_h - 0.5f;
  float fx = floorf(xb), fy = floorf(yb);
  float ax = xb - fx, ay = yb - fy;
  int x0 = (int)fx, y0 = (int)fy;
  auto fetch = [&](int x, int y) {
    x = std::min(std::max(x, 0), s.env_w - 1);
    y = std::min(std::max(y, 0), s.env_h - 1);
    const float* c = &s.env[4 * ((size_t)y * s.env_w + x)];
    return V3(c[0], c[1], c[2]);
  };
  V3 a = fetch(x0, y0), b = fetch(x0 + 1, y0), c = fetch(x0, y0 + 1), d = fetch(x0 + 1, y0 + 1);
  return (1.f - ay) * ((1.f - ax) * a + ax * b) + ay * ((1.f - ax) * c + ax * d);
}

V3 env_radiance(const OScene& s, V3 dir) {  // getEnvironmentRadiance
  if (!s.has_env) return V3(0.f);
  float theta = spherical_theta(dir);
  float phi = spherical_phi(dir) + s.env_rot;
  if (phi > kTwoPi) phi = phi - kTwoPi;
  float x = phi / (2.f * kPi);
  float y = theta / kPi;
  return s.env_scale * tex_linear(s, x, y);
}

float env_pdf(const OScene& s, V3 wi) {  // getEnvironmentPdf
  if (!s.env_pdf) return 1.f / (4.f * kPi);
  float width = (float)s.env_w, height = (float)s.env_h;
  float theta = spherical_theta(wi);
  float phi = spherical_phi(wi) + s.env_rot;
  if (phi > kTwoPi) phi = phi - kTwoPi;
  float u = phi / (2.f * kPi), v = theta / kPi;
  int iu = std::min(std::max((int)(u * s.env_w), 0), s.env_w - 1);
  int iv = std::min(std::max((int)(v * s.env_h), 0), s.env_h - 1);
  int cw = s.env_w + 1;
  float cdf_last_u = tex_nearest(s.cpdf, cw, s.env_h, 1.f, iv / height);
  float cdf_last_v = tex_nearest(s.mpdf, s.env_h + 1, 1, 1.f, 0.f);
  float sin_theta = osinf(theta);
  float denom = (2.f * kPi * kPi * sin_theta) * cdf_last_u * cdf_last_v;
  float cdf_u = tex_nearest(s.cpdf, cw, s.env_h, iu / width, iv / height);
  float cdf_v = tex_nearest(s.mpdf, s.env_h + 1, 1, iv / height, 0.f);
  return denom != 0.f ? (cdf_u * cdf_v) / denom : 0.f;
}

V3 sample_env(const OScene& s, SI& si, uint32_t& rng, float* pdf) {  // sampleEnvironmentLight
  V3 rval(0.f);
  if (s.env_pdf) {
    auto lower_bound = [&](float u, const std::vector<float>& cdf, int tw, int th, float y, float size) {
      int first = 0, count = (int)size;
      while (count > 0) {
        int step = count >> 1, middle = first + step;
        if (tex_nearest(cdf, tw, th, middle / size, y) < u) {
          first = middle + 1;
          count -= step + 1;
        } else {
          count = step;
        }
      }
      return std::max(0, first - 1);
    };
    float ux = lcg_randomf(rng);  // vec2f(lcg, lcg): first draw is .x
    float uy = lcg_randomf(rng);
    float width = (float)s.env_w, height = (float)s.env_h;
    int cw = s.env_w + 1, mh = s.env_h + 1;
    int iv = lower_bound(uy, s.mcdf, mh, 1, 0.f, height);
    float cdf_v = tex_nearest(s.mcdf, mh, 1, iv / height, 0.f);
    float cdf_next_v = tex_nearest(s.mcdf, mh, 1, (iv + 1) / height, 0.f);
    float dv = (cdf_next_v - uy) / (cdf_next_v - cdf_v);
    float v = (iv + dv) / height;
    int iu = lower_bound(ux, s.ccdf, cw, s.env_h, iv / height, width);
    float cdf_u = tex_nearest(s.ccdf, cw, s.env_h, iu / width, iv / height);
    float cdf_next_u = tex_nearest(s.ccdf, cw, s.env_h, (iu + 1) / width, iv / height);
    float du = (cdf_next_u - ux) / (cdf_next_u - cdf_u);
    float u = (iu + du) / width;
    rval = s.env_scale * tex_linear(s, u, v);
    float cdf_last_u = tex_nearest(s.cpdf, cw, s.env_h, 1.f, iv / height);
    float cdf_last_v = tex_nearest(s.mpdf, mh, 1, 1.f, 0.f);
    float pu = tex_nearest(s.cpdf, cw, s.env_h, iu / width, iv / height);
    float pv = tex_nearest(s.mpdf, mh, 1, iv / height, 0.f);
    float theta = kPi * v;
    float sin_theta = osinf(theta);
    float denom = (2.f * kPi * kPi * sin_theta) * cdf_last_u * cdf_last_v;
    *pdf = denom != 0.f ? (pu * pv) / denom : 0.f;
    float phi = 2.f * kPi * u - s.env_rot;
    if (phi < 0) phi = kTwoPi + phi;
    si.wi = V3(sin_theta * ocosf(phi), sin_theta * osinf(phi), ocosf(theta));
    si.wi_local = normalize(apply_mat(si.to_local, si.wi));
  } else {
    float a = lcg_randomf(rng);
    float b = lcg_randomf(rng);
    si.wi = uniform_sample_sphere(a, b);
    si.wi_local = normalize(apply_mat(si.to_local, si.wi));
    *pdf = 1.f / (4.f * kPi);
    rval = env_radiance(s, si.wi);
  }
  return rval;
}

// ------------------------------------------------------------ per-path event log
// Every ray a path traces, in the order it traces them: the record the tests
// compare with the reference's own integrator (every owl::traceRay call) and
// with the device's per-path log.  kEvFloats floats per event:
//   [0] kind (int bits: 0 radiance, 1 light-sample shadow, 2 BSDF-sample shadow)
//   [1] result (int bits: radiance = hit primitive, -1 miss; shadow = 1 unoccluded)
//   [2] t of the hit (radiance), [3] u of the hit
//   [4..6] origin, [7..9] direction, [10] RNG state when the ray was traced
//   (radiance rays only; uint bits), [11] 0
constexpr int kEvFloats = 12;
struct EvLog {
  float* ev = nullptr;
  int cap = 0, n = 0;
};
thread_local EvLog* tl_log = nullptr;

void log_event(int kind, int result, float t, float u, V3 o, V3 d, uint32_t rng) {
  EvLog* L = tl_log;
  if (!L) return;
  if (L->n < L->cap) {
    float* e = L->ev + (size_t)L->n * kEvFloats;
    memcpy(e + 0, &kind, 4);
    memcpy(e + 1, &result, 4);
    e[2] = t;
    e[3] = u;
    e[4] = o.x; e[5] = o.y; e[6] = o.z;
    e[7] = d.x; e[8] = d.y; e[9] = d.z;
    memcpy(e + 10, &rng, 4);
    e[11] = 0.f;
  }
  ++L->n;
}

// owl::traceRay(RADIANCE): closest hit -> hairCH / triangleMeshCH, else miss.
// rng: the path's RNG state when the ray is traced (logged only).
void trace_radiance(const OScene& s, V3 o, V3 d, SI& si, uint32_t rng = 0) {
  OHit h = trace(s, o, d, 0.f, 1e30f, false);
  log_event(0, h.prim < 0 ? -1 : h.prim, h.prim < 0 ? 0.f : h.t, h.prim < 0 ? 0.f : h.u, o, d, rng);
  if (h.prim < 0) {  // miss (optix_common.cuh:604-616)
    si.hit = false;
    si.Le = V3(0.f);
    if (s.has_env) si.Le = env_radiance(s, si.wi);
    return;
  }
  if (h.prim < s.n_seg()) {  // hairCH
    si.group = s.seg_group.empty() ? 0 : s.seg_group[h.prim];
    const float* q = &s.cp[4 * s.seg[h.prim]];
    V4 cps[4];
    for (int i = 0; i < 4; ++i) cps[i] = V4(q[4 * i], q[4 * i + 1], q[4 * i + 2], q[4 * i + 3]);
    Cubic ip = s.catrom ? Cubic::from_catrom(cps) : Cubic::from_bspline(cps);
    float u = h.u;
    V3 p = o + h.t * d;
    si.radius = ip.position4(u).w;
    V3 n = surface_normal(ip, u, &p);
    si.n = normalize(n);
    si.t = curve_tangent(ip, u);
    si.p = p;
    V3 X = si.t, Y = normalize(cross(si.wo, X)), Z = normalize(cross(X, Y));
    si.to_local[0] = X;
    si.to_local[1] = Y;
    si.to_local[2] = Z;
    si.to_world[0] = V3(X.x, Y.x, Z.x);
    si.to_world[1] = V3(X.y, Y.y, Z.y);
    si.to_world[2] = V3(X.z, Y.z, Z.z);
    si.wo_local = normalize(apply_mat(si.to_local, si.wo));
    si.hit = true;
    si.surface = false;
  } else {  // triangleMeshCH
    const int* t = &s.tri[3 * (h.prim - s.n_seg())];
    float bu = h.u, bv = h.v;
    auto interp = [&](const std::vector<float>& a) {
      V3 A(a[3 * t[0]], a[3 * t[0] + 1], a[3 * t[0] + 2]);
      V3 B(a[3 * t[1]], a[3 * t[1] + 1], a[3 * t[1] + 2]);
      V3 C(a[3 * t[2]], a[3 * t[2] + 1], a[3 * t[2] + 2]);
      return (1.f - bu - bv) * A + bu * B + bv * C;
    };
    si.p = interp(s.vtx);
    si.n = normalize(interp(s.nrm));
    orthonormal_basis(si.n, si.to_local, si.to_world);
    si.t = si.to_local[0];
    si.wo_local = normalize(apply_mat(si.to_local, si.wo));
    si.radius = 0.f;
    si.hit = true;
    si.surface = true;
  }
}

// owl::traceRay(SHADOW); kind 1 = light sample, 2 = BSDF sample (logged only).
bool visible(const OScene& s, V3 o, V3 d, int kind) {
  const bool v = trace(s, o, d, 0.f, 1e30f, true).prim < 0;
  log_event(kind, v ? 1 : 0, 0.f, 0.f, o, d, 0u);
  return v;
}

V3 hair_f(const OScene& s, const SI& si, float* pdf) {
  return disney_hair(si.wo_local, si.wi_local, dot(si.to_local[1], si.n), hair_of(s, si), pdf);
}

V3 sample_lights(const OScene& s, SI& si, uint32_t& rng, bool& is_delta) {  // sampleLights
  is_delta = false;
  V3 emit(0.f), final_color(0.f);
  float light_pdf = 1.f, bsdf_pdf = 1.f;
  float rand = lcg_randomf(rng);
  int nt = s.n_dl() + (s.has_env ? 1 : 0);
  int sel = (int)floorf(rand * nt);
  if (sel >= s.n_dl()) {
    light_pdf = light_pdf * 1.f / nt;
    float env_p = 1.f;
    emit = sample_env(s, si, rng, &env_p);
    light_pdf = light_pdf * env_p;
  } else {
    light_pdf = light_pdf * 1.f / nt;
    const float* L = &s.dl[6 * sel];
    emit = V3(L[3], L[4], L[5]);
    si.wi = normalize(V3(L[0], L[1], L[2]));
    si.wi_local = normalize(apply_mat(si.to_local, si.wi));
    is_delta = true;
  }
  bool lower = dot(si.wi, si.n) < 0.f;
  V3 nd = si.n;
  if (si.surface && lower) return final_color;
  if (!si.surface && lower) {
    nd = -si.n;
    si.p = si.p + 2.f * si.radius * nd;
  }
  if (visible(s, si.p + 1e-3f * nd, si.wi, 1)) {
    V3 bsdf(0.f);
    if (!si.surface) {
      bsdf = hair_f(s, si, &bsdf_pdf);
    } else {
      bsdf = frostbite_ggx(si.wo_local, si.wi_local, s.diffuse, s.alpha);
      bsdf_pdf = pdf_ggx(s.alpha, si.wo_local, normalize(si.wo_local + si.wi_local));
    }
    if (s.mis && !is_delta)
      final_color = bsdf * emit * power_heuristic(light_pdf, bsdf_pdf) / light_pdf;
    else
      final_color = bsdf * emit / light_pdf;
  }
  return final_color;
}

V3 sample_bsdf(const OScene& s, SI& si, uint32_t& rng) {  // sampleBSDF
  float r0 = lcg_randomf(rng);
  float r1 = lcg_randomf(rng);
  V3 emit(0.f), bsdf(0.f), final_color(0.f);
  float light_pdf = 1.f, bsdf_pdf = 1.f;
  if (!si.surface) {
    float r[4] = {r0, r1, 0.f, 0.f};
    r[2] = lcg_randomf(rng);
    r[3] = lcg_randomf(rng);
    V3 wil;
    bsdf = sample_disney_hair(si.wo_local, dot(si.to_local[1], si.n), r, hair_of(s, si), &wil, &bsdf_pdf, nullptr);
    si.wi_local = wil;
    si.wi = normalize(apply_mat(si.to_world, si.wi_local));
  } else {
    si.wi_local = sample_ggx(r0, r1, s.alpha, si.wo_local, &bsdf_pdf);
    si.wi = normalize(apply_mat(si.to_world, si.wi_local));
    bsdf = frostbite_ggx(si.wo_local, si.wi_local, s.diffuse, s.alpha);
  }
  bool lower = dot(si.wi, si.n) < 0.f;
  V3 nd = si.n;
  if (si.surface && lower) return final_color;
  if (!si.surface && lower) {
    nd = -si.n;
    si.p = si.p + 2.f * si.radius * nd;
  }
  if (visible(s, si.p + 1e-3f * nd, si.wi, 2)) {
    int nt = s.n_dl() + (s.has_env ? 1 : 0);
    emit = env_radiance(s, si.wi);
    light_pdf = env_pdf(s, si.wi) * 1.f / nt;
    if (s.mis)
      final_color = bsdf * emit * power_heuristic(bsdf_pdf, light_pdf) / bsdf_pdf;
    else
      final_color = bsdf * emit / bsdf_pdf;
  }
  return final_color;
}

V3 direct_lighting(const OScene& s, SI si, uint32_t& rng) {  // directLighting
  V3 final_color(0.f);
  if (s.mis) {
    bool is_delta = false;
    V3 l = sample_lights(s, si, rng, is_delta);
    V3 b(0.f);
    if (!is_delta) b = sample_bsdf(s, si, rng);
    final_color = final_color + (l + b);
  } else {
    bool is_delta = false;
    final_color = final_color + sample_lights(s, si, rng, is_delta);
  }
  if (isnan(final_color.x) || isnan(final_color.y) || isnan(final_color.z)) final_color = V3(0.f);
  return final_color;
}

V3 next_vertex(const OScene& s, SI& si, uint32_t& rng, float* pdf_out = nullptr) {  // msnnNextPathVertex / nextPathVertex
  float r0 = lcg_randomf(rng);
  float r1 = lcg_randomf(rng);
  float next_pdf = 1.f;
  V3 next_bsdf(0.f);
  if (!si.surface) {
    float r[4] = {r0, r1, 0.f, 0.f};
    r[2] = lcg_randomf(rng);
    r[3] = lcg_randomf(rng);
    V3 wil;
    next_bsdf = sample_disney_hair(si.wo_local, dot(si.to_local[1], si.n), r, hair_of(s, si), &wil, &next_pdf, nullptr);
    si.wi_local = wil;
    si.wi = normalize(apply_mat(si.to_world, si.wi_local));
  } else {
    si.wi_local = sample_ggx(r0, r1, s.alpha, si.wo_local, &next_pdf);
    si.wi = normalize(apply_mat(si.to_world, si.wi_local));
    next_bsdf = frostbite_ggx(si.wo_local, si.wi_local, s.diffuse, s.alpha);
  }
  si.hit = false;
  si.wo = -si.wi;
  bool lower = dot(si.wi, si.n) < 0.f;
  V3 nd = si.n;
  if (lower && !si.surface) {
    nd = -si.n;
    si.p = si.p + 2.f * si.radius * nd;
  }
  V3 mul = next_pdf == 0.f ? next_bsdf : next_bsdf / next_pdf;
  if (isnan(mul.x) || isnan(mul.y) || isnan(mul.z)) mul = V3(1.f);
  if (pdf_out) *pdf_out = next_pdf;  // nextPathVertexNRC returns it (nrc.cu:17-66)
  trace_radiance(s, si.p + 1e-3f * nd, -si.wo, si, rng);
  return mul;
}

// nrcTracePaths (cuda/nrc.cu:136-310) in the reference's loop, with
// nrcSpread (utils.cuh:86-90).  Outputs of one pixel: the G-buffer
// (radiance, beta), its cache query row, and for a training pixel the train
// buffer (TrainBuffer, nrc.cuh:29-40) and the suffix's query row.
constexpr int kNrcMaxBounces = 40;
struct NrcOut {
  V3 rad, beta;
  float query[9];
  float suffix_query[9];
  float rec[kNrcMaxBounces][15];  // vert, wo, n, vertRadiance, vertBeta
  int bounces = 0, thit = 0;
};

float nrc_spread(V3 x1, V3 x2, float abscos, float pdf) {
  float l = length(x2 - x1);
  return sqrtf(l * l / pdf / abscos);
}

void nrc_query_row(const OScene& s, const SI& si, float* row) {
  V3 p = si.p / s.scene_scale;
  float r[9] = {p.x, p.y, p.z, si.wo.x, si.wo.y, si.wo.z, si.n.x, si.n.y, si.n.z};
  memcpy(row, r, sizeof(r));
}

void nrc_trace_paths(const OScene& s, SI si, uint32_t& rng, bool training, bool unbiased, float c, NrcOut& o) {
  bool suffix = false, recalc = false;
  float l0 = length(si.p - s.cam_pos);
  float a0 = l0 * l0 / (4.f * 3.1415926f) / fabsf(si.wo_local.z);
  V3 prev_point(0.f);
  float spread = 0.f;
  V3 final_color(0.f), beta(1.f);
  for (int bounce = 0; bounce < kNrcMaxBounces; bounce++) {
    V3 direct = direct_lighting(s, si, rng);
    final_color = final_color + beta * direct;
    V3 prev_wo = si.wo, prev_n = si.n;
    prev_point = si.p;
    float prev_pdf = 1.f;
    V3 this_beta = next_vertex(s, si, rng, &prev_pdf);
    beta = beta * this_beta;
    if (training) {
      if (recalc) {
        float l = length(si.p - prev_point);
        a0 = l * l / (4.f * 3.1415926f) / fabsf(si.wo_local.z);
        recalc = false;
      }
      V3 q = prev_point / s.scene_scale;
      float r[15] = {q.x, q.y, q.z, prev_wo.x, prev_wo.y, prev_wo.z, prev_n.x, prev_n.y, prev_n.z,
                     direct.x, direct.y, direct.z, this_beta.x, this_beta.y, this_beta.z};
      memcpy(o.rec[bounce], r, sizeof(r));
    }
    spread = spread + nrc_spread(si.p, prev_point, fabsf(si.wo_local.z), prev_pdf);
    bool cond = spread * spread > c * a0;
    if (!si.hit || bounce == kNrcMaxBounces - 1) {
      if (!suffix) {
        o.rad = final_color;
        o.beta = V3(0.f);
      }
      o.bounces = bounce;
      o.thit = 0;
      break;
    } else if (cond && !suffix) {
      o.rad = final_color;
      o.beta = beta;
      nrc_query_row(s, si, o.query);
      if (training) {
        suffix = true;
        recalc = true;
        spread = 0.f;
      } else {
        break;
      }
    } else if (cond && suffix) {
      nrc_query_row(s, si, o.suffix_query);
      o.bounces = bounce;
      o.thit = 1;
      if (!unbiased) break;
      c = 1e30f;
    }
  }
}

V3 msnn_path_trace(const OScene& s, SI si, uint32_t& rng, int v2_stop, int beta_int) {
  V3 beta(1.f);
  V3 final_color = direct_lighting(s, si, rng);
  for (int b = 1; b <= v2_stop; b++) {
    V3 mul = next_vertex(s, si, rng);
    beta = beta * mul;
    if (!si.hit) break;
    final_color = final_color + 1.f * beta * direct_lighting(s, si, rng);
    float q = fmaxf(0.05f, 1.f - luminance(beta));
    float eps = lcg_randomf(rng);
    if (eps < q || b > beta_int) break;
    beta = beta / (1.f - q);
  }
  return final_color;
}

V3 msnn_training_path(const OScene& s, SI si, uint32_t& rng, V3* short_color, int beta_int) {
  V3 beta(1.f), beta_s(1.f);
  V3 final_color = direct_lighting(s, si, rng);
  *short_color = final_color;
  for (int b = 1; b < s.path_v2; b++) {
    V3 mul = next_vertex(s, si, rng);
    beta = beta * mul;
    beta_s = beta_s * mul;
    if (!si.hit) break;
    V3 dl = direct_lighting(s, si, rng);
    final_color = final_color + beta * dl;
    *short_color = *short_color + 1.f * beta_s * dl;
    float q = fmaxf(0.05f, 1.f - luminance(beta));
    float qs = fmaxf(0.05f, 1.f - luminance(beta_s));
    float eps = lcg_randomf(rng);
    if (eps < qs || b > beta_int) beta_s = V3(0.f);
    if (eps < q) break;
    beta = beta / (1.f - q);
    if (beta_s.x != 0.f || beta_s.y != 0.f || beta_s.z != 0.f) beta_s = beta_s / (1.f - qs);
  }
  return final_color;
}

V3 path_trace(const OScene& s, SI si, uint32_t& rng, int v1, int v2) {
  if (v2 < v1) return V3(0.f);
  V3 beta(1.f), final_color(0.f);
  if (v1 == 0) final_color = direct_lighting(s, si, rng);
  for (int b = 1; b <= v2; b++) {
    V3 mul = next_vertex(s, si, rng);
    beta = beta * mul;
    if (!si.hit) break;
    if (b >= v1) final_color = final_color + beta * direct_lighting(s, si, rng);
    float q = fmaxf(0.05f, 1.f - luminance(beta));
    float eps = lcg_randomf(rng);
    if (eps < q) break;
    beta = beta / (1.f - q);
  }
  return final_color;
}

uint32_t feistel_perm(uint32_t i, uint32_t n, uint32_t key) {
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

}  // namespace

extern "C" {

void* hmo_scene_new(const float* cp, int n_cp, const int* seg, int n_seg, const float* vtx, const float* nrm, int n_vtx,
                    const int* tri, int n_tri, const float* env, int env_w, int env_h, const float* cpdf,
                    const float* ccdf, const float* mpdf, const float* mcdf, const float* dl, int n_dl,
                    const float* camera12, const float* mat16, const int* settings9, float scene_scale) {
  OScene* s = new OScene();
  s->cp.assign(cp, cp + 4 * (size_t)n_cp);
  s->seg.assign(seg, seg + n_seg);
  s->vtx.assign(vtx, vtx + 3 * (size_t)n_vtx);
  s->nrm.assign(nrm, nrm + 3 * (size_t)n_vtx);
  s->tri.assign(tri, tri + 3 * (size_t)n_tri);
  s->env_w = env_w;
  s->env_h = env_h;
  if (env_w > 0) {
    s->env.assign(env, env + 4 * (size_t)env_w * env_h);
    s->cpdf.assign(cpdf, cpdf + (size_t)(env_w + 1) * env_h);
    s->ccdf.assign(ccdf, ccdf + (size_t)(env_w + 1) * env_h);
    s->mpdf.assign(mpdf, mpdf + env_h + 1);
    s->mcdf.assign(mcdf, mcdf + env_h + 1);
  }
  s->dl.assign(dl, dl + 6 * (size_t)n_dl);
  s->cam_pos = V3(camera12[0], camera12[1], camera12[2]);
  s->cam_d00 = V3(camera12[3], camera12[4], camera12[5]);
  s->cam_du = V3(camera12[6], camera12[7], camera12[8]);
  s->cam_dv = V3(camera12[9], camera12[10], camera12[11]);
  for (int i = 0; i < 10; ++i) s->hp[i] = mat16[i];
  s->hs = setup_hair_shading(s->hp);
  s->diffuse = V3(mat16[10], mat16[11], mat16[12]);
  float a = fminf(fmaxf(mat16[13], 0.01f), 1.f);
  s->alpha = a * a;
  s->env_scale = mat16[14];
  s->env_rot = mat16[15];
  s->width = settings9[0];
  s->height = settings9[1];
  s->path_v1 = settings9[2];
  s->path_v2 = settings9[3];
  s->mis = settings9[4];
  s->env_pdf = settings9[5];
  s->has_env = settings9[6];
  s->catrom = settings9[7];
  s->seg_split = settings9[8];
  s->scene_scale = scene_scale;
  build_bvh(*s);
  return s;
}

void hmo_scene_free(void* h) { delete (OScene*)h; }

// One frame of the NRC G_BUFFER pass (rayGenCam, nrc.cu:312-356) for pixels
// [p0, p0 + np): gbuf [np][7] = radiance, beta, hit; query / suffix_query
// [np][9]; records [np][40][15]; tinfo [np][4] = bounces, suffix ended at a
// query, unbiased, training pixel.
//
// hmo_render_nrc_ev: the same plus each path's ray log and event count (as
// hmo_render_pixels_ev; events / n_events may be NULL).
void hmo_render_nrc_ev(void* h, int accum_id, int every_nth, int n_train, float c, int p0, int np, float* gbuf,
                       float* query, float* suffix_query, float* records, int* tinfo, float* events, int* n_events,
                       int max_events, int threads) {
  OScene* s = (OScene*)h;
  auto work = [&](int b, int e) {
    EvLog log;
    for (int pid = b; pid < e; ++pid) {
      if (events) {
        log.ev = events + (size_t)(pid - p0) * max_events * kEvFloats;
        log.cap = max_events;
        log.n = 0;
        tl_log = &log;
      }
      ulp_seed_path((uint32_t)pid);
      const int x = pid % s->width, y = pid / s->width;
      uint32_t rng = get_rng(accum_id + 10007, (uint32_t)x, (uint32_t)y, (uint32_t)s->width, (uint32_t)s->height);
      bool training = false;
      const int tr = pid / every_nth;
      if (tr < n_train) {
        uint32_t pick = feistel_perm((uint32_t)tr, (uint32_t)n_train, (uint32_t)accum_id) % every_nth;
        training = (uint32_t)(pid % every_nth) == pick;
      }
      const bool unbiased = training && tr % 16 == 0;
      float ox = lcg_randomf(rng);
      float oy = lcg_randomf(rng);
      float su = ((float)x + ox) / (float)s->width, sv = ((float)y + oy) / (float)s->height;
      V3 dir = normalize(s->cam_d00 + su * s->cam_du + sv * s->cam_dv);
      SI si;
      si.hit = false;
      si.wo = -1.f * dir;
      si.wi = dir;
      trace_radiance(*s, s->cam_pos, dir, si, rng);
      std::unique_ptr<NrcOut> o(new NrcOut());
      memset(o->query, 0, sizeof(o->query));
      memset(o->suffix_query, 0, sizeof(o->suffix_query));
      memset(o->rec, 0, sizeof(o->rec));
      bool hit = si.hit && !(si.surface && si.wo_local.z < 0.f);
      if (!hit) {
        o->rad = si.hit ? V3(0.f) : si.Le;
        o->beta = V3(0.f);
      } else {
        nrc_trace_paths(*s, si, rng, training, unbiased, c, *o);
      }
      const int i = pid - p0;
      float g[7] = {o->rad.x, o->rad.y, o->rad.z, o->beta.x, o->beta.y, o->beta.z, hit ? 1.f : 0.f};
      memcpy(gbuf + 7 * (size_t)i, g, sizeof(g));
      memcpy(query + 9 * (size_t)i, o->query, sizeof(o->query));
      memcpy(suffix_query + 9 * (size_t)i, o->suffix_query, sizeof(o->suffix_query));
      memcpy(records + (size_t)i * kNrcMaxBounces * 15, o->rec, sizeof(o->rec));
      int t[4] = {o->bounces, o->thit, unbiased ? 1 : 0, training ? 1 : 0};
      memcpy(tinfo + 4 * (size_t)i, t, sizeof(t));
      if (n_events) n_events[i] = log.n;
    }
    tl_log = nullptr;
  };
  if (threads <= 1) {
    work(p0, p0 + np);
    return;
  }
  std::vector<std::thread> pool;
  int chunk = (np + threads - 1) / threads;
  for (int k = 0; k < threads; ++k) {
    int b = p0 + k * chunk, e = std::min(p0 + np, b + chunk);
    if (b < e) pool.emplace_back(work, b, e);
  }
  for (auto& t : pool) t.join();
}

void hmo_render_nrc(void* h, int accum_id, int every_nth, int n_train, float c, int p0, int np, float* gbuf,
                    float* query, float* suffix_query, float* records, int* tinfo, int threads) {
  hmo_render_nrc_ev(h, accum_id, every_nth, n_train, c, p0, np, gbuf, query, suffix_query, records, tinfo, nullptr,
                    nullptr, 0, threads);
}

// Strand groups: group of every segment, each group's 10 material floats.
void hmo_scene_set_groups(void* h, const int* seg_group, int n_seg, const float* mats10, int n_groups) {
  OScene* s = (OScene*)h;
  s->seg_group.assign(seg_group, seg_group + n_seg);
  s->ghs.clear();
  for (int g = 0; g < n_groups; ++g) s->ghs.push_back(setup_hair_shading(mats10 + 10 * g));
}

int hmo_bvh_sizes(void* h, int* n_nodes, int* n_leaves) {
  OScene* s = (OScene*)h;
  *n_nodes = (int)s->nodes.size() / 16;
  *n_leaves = (int)s->leaf_prim.size();
  return 0;
}

void hmo_bvh_export(void* h, float* nodes, int* leaves) {
  OScene* s = (OScene*)h;
  memcpy(nodes, s->nodes.data(), s->nodes.size() * sizeof(float));
  memcpy(leaves, s->leaf_prim.data(), s->leaf_prim.size() * sizeof(int));
}

void hmo_trace_rays(void* h, const float* org, const float* dir, int n, float tmin, float tmax, int any, float* hits) {
  OScene* s = (OScene*)h;
  for (int i = 0; i < n; ++i) {
    OHit r = trace(*s, V3(org[3 * i], org[3 * i + 1], org[3 * i + 2]), V3(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]),
                   tmin, tmax, any != 0);
    hits[4 * i] = r.t;
    memcpy(&hits[4 * i + 1], &r.prim, 4);
    hits[4 * i + 2] = r.u;
    hits[4 * i + 3] = r.v;
  }
}

// One frame of rayGenCam for pixels [p0, p0 + np).  mode 0 = plain PT
// (color = the NaN-scrubbed pathTrace result), 1 = HairMSNN G-buffer pass
// (color = the G-buffer's shortPathColor, nn_in = the cache input row,
// train_out = the training target of a training pixel, flags bit0 hit,
// bit1 surface, bit2 training pixel).
//
// hmo_render_pixels_ev: the same, plus each path's event log (events
// [np][max_events][kEvFloats], see log_event; n_events [np] = events the
// path traced, possibly more than max_events) and its RNG state when the
// path ended (rng_end [np]).  events / n_events / rng_end may be NULL.
void hmo_render_pixels_ev(void* h, int mode, int beta_knob, int accum_id, int every_nth, int n_train, int p0, int np,
                          float* color, float* nn_in, float* train_out, int* flags, float* events, int* n_events,
                          uint32_t* rng_end, int max_events, int threads) {
  OScene* s = (OScene*)h;
  auto work = [&](int b, int e) {
    EvLog log;
    for (int pid = b; pid < e; ++pid) {
      if (events) {
        log.ev = events + (size_t)(pid - p0) * max_events * kEvFloats;
        log.cap = max_events;
        log.n = 0;
        tl_log = &log;
      }
      const int x = pid % s->width, y = pid / s->width;
      ulp_seed_path((uint32_t)pid);
      uint32_t rng = get_rng(accum_id + 10007, (uint32_t)x, (uint32_t)y, (uint32_t)s->width, (uint32_t)s->height);
      bool training = false;
      if (mode == 1) {
        int tr = pid / every_nth;
        if (tr < n_train) {
          uint32_t pick = feistel_perm((uint32_t)tr, (uint32_t)n_train, (uint32_t)accum_id) % every_nth;
          training = (uint32_t)(pid % every_nth) == pick;
        }
      }
      float ox = lcg_randomf(rng);
      float oy = lcg_randomf(rng);
      float su = ((float)x + ox) / (float)s->width, sv = ((float)y + oy) / (float)s->height;
      V3 dir = normalize(s->cam_d00 + su * s->cam_du + sv * s->cam_dv);
      SI si;
      si.hit = false;
      si.wo = -1.f * dir;
      si.wi = dir;
      trace_radiance(*s, s->cam_pos, dir, si, rng);
      V3 c(0.f), sc(0.f);
      const int i = pid - p0;
      if (mode == 0) {
        c = !si.hit ? si.Le : path_trace(*s, si, rng, s->path_v1 - 1, s->path_v2 - 1);
        if (isnan(c.x) || isnan(c.y) || isnan(c.z)) c = V3(0.f);
      } else {
        if (training) {
          if (si.hit) c = msnn_training_path(*s, si, rng, &sc, beta_knob - 1);
          if (isnan(c.x) || isnan(c.y) || isnan(c.z)) c = V3(0.f);
          if (isinf(c.x) || isinf(c.y) || isinf(c.z)) c = V3(1e5f);
          if (isnan(sc.x) || isnan(sc.y) || isnan(sc.z)) sc = V3(0.01f);
          if (isinf(sc.x) || isinf(sc.y) || isinf(sc.z)) sc = V3(1e5f);
          train_out[3 * i] = c.x - sc.x;
          train_out[3 * i + 1] = c.y - sc.y;
          train_out[3 * i + 2] = c.z - sc.z;
          if (!si.hit) c = si.Le;
        } else {
          c = !si.hit ? si.Le : msnn_path_trace(*s, si, rng, s->path_v2 - 1, beta_knob - 1);
        }
        V3 p = si.hit ? si.p / s->scene_scale : V3(0.f);
        V3 t = si.hit ? si.t : V3(0.f);
        float row[12] = {p.x, p.y, p.z, si.wo.x, si.wo.y, si.wo.z, t.x, t.y, t.z, 0.f, 0.f, 0.f};
        memcpy(nn_in + 12 * i, row, sizeof(row));
      }
      color[3 * i] = c.x;
      color[3 * i + 1] = c.y;
      color[3 * i + 2] = c.z;
      flags[i] = (si.hit ? 1 : 0) | (si.hit && si.surface ? 2 : 0) | (training ? 4 : 0);
      if (n_events) n_events[i] = log.n;
      if (rng_end) rng_end[i] = rng;
    }
    tl_log = nullptr;
  };
  if (threads <= 1) {
    work(p0, p0 + np);
    return;
  }
  std::vector<std::thread> pool;
  int chunk = (np + threads - 1) / threads;
  for (int k = 0; k < threads; ++k) {
    int b = p0 + k * chunk, e = std::min(p0 + np, b + chunk);
    if (b < e) pool.emplace_back(work, b, e);
  }
  for (auto& t : pool) t.join();
}

// One TRAIN_DATA_GEN launch of rayGenCam (hair_msnn.cu:187-275) for
// training records [p0, p0 + np) of a rec_x-wide launch grid: record r =
// x + rec_x * y aims from the camera at points[r] (the reference's
// sampledPoints[sceneIndices[trOfs]], gathered by the caller), seeds its RNG
// with launch index (x, y) over the frame's width (get_rng with the frame
// buffer's size, hair_msnn.cu:193-194) and runs msnnTrainingPath.
// train_in [np][12] / train_out [np][3]: nnTrainInput / nnTrainOutput at
// trOfs; flags bit0 hit, bit1 surface; events / n_events / rng_end as in
// hmo_render_pixels_ev (may be NULL).
void hmo_render_traingen_ev(void* h, int beta_knob, int accum_id, int rec_x, const float* points, int p0, int np,
                            float* train_in, float* train_out, int* flags, float* events, int* n_events,
                            uint32_t* rng_end, int max_events, int threads) {
  OScene* s = (OScene*)h;
  auto work = [&](int b, int e) {
    EvLog log;
    for (int r = b; r < e; ++r) {
      const int i = r - p0;
      if (events) {
        log.ev = events + (size_t)i * max_events * kEvFloats;
        log.cap = max_events;
        log.n = 0;
        tl_log = &log;
      }
      ulp_seed_path((uint32_t)r);
      const int x = r % rec_x, y = r / rec_x;
      uint32_t rng = get_rng(accum_id + 10007, (uint32_t)x, (uint32_t)y, (uint32_t)s->width, (uint32_t)s->height);
      const V3 sp(points[3 * (size_t)i], points[3 * (size_t)i + 1], points[3 * (size_t)i + 2]);
      const V3 dir = normalize(sp - s->cam_pos);
      SI si;
      si.hit = false;
      si.wo = -1.f * dir;
      si.wi = dir;
      trace_radiance(*s, s->cam_pos, dir, si, rng);
      V3 c(0.f), sc(0.f);
      if (si.hit) c = msnn_training_path(*s, si, rng, &sc, beta_knob - 1);
      if (isnan(c.x) || isnan(c.y) || isnan(c.z)) c = V3(0.f);
      if (isinf(c.x) || isinf(c.y) || isinf(c.z)) c = V3(1e5f);
      if (isnan(sc.x) || isnan(sc.y) || isnan(sc.z)) sc = V3(0.01f);
      if (isinf(sc.x) || isinf(sc.y) || isinf(sc.z)) sc = V3(1e5f);
      train_out[3 * (size_t)i] = c.x - sc.x;
      train_out[3 * (size_t)i + 1] = c.y - sc.y;
      train_out[3 * (size_t)i + 2] = c.z - sc.z;
      V3 p = si.hit ? si.p / s->scene_scale : V3(0.f);
      V3 t = si.hit ? si.t : V3(0.f);
      float row[12] = {p.x, p.y, p.z, si.wo.x, si.wo.y, si.wo.z, t.x, t.y, t.z, 0.f, 0.f, 0.f};
      memcpy(train_in + 12 * (size_t)i, row, sizeof(row));
      flags[i] = (si.hit ? 1 : 0) | (si.hit && si.surface ? 2 : 0);
      if (n_events) n_events[i] = log.n;
      if (rng_end) rng_end[i] = rng;
    }
    tl_log = nullptr;
  };
  if (threads <= 1) {
    work(p0, p0 + np);
    return;
  }
  std::vector<std::thread> pool;
  int chunk = (np + threads - 1) / threads;
  for (int k = 0; k < threads; ++k) {
    int b = p0 + k * chunk, e = std::min(p0 + np, b + chunk);
    if (b < e) pool.emplace_back(work, b, e);
  }
  for (auto& t : pool) t.join();
}

// The training-pixel permutation (the reference's shuffled trainIdxs table).
uint32_t hmo_feistel_perm(uint32_t i, uint32_t n, uint32_t key) { return feistel_perm(i, n, key); }

void hmo_render_pixels(void* h, int mode, int beta_knob, int accum_id, int every_nth, int n_train, int p0, int np,
                       float* color, float* nn_in, float* train_out, int* flags, int threads) {
  hmo_render_pixels_ev(h, mode, beta_knob, accum_id, every_nth, n_train, p0, np, color, nn_in, train_out, flags,
                       nullptr, nullptr, nullptr, 0, threads);
}

}  // extern "C"
