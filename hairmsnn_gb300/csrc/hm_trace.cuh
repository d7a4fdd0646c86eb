// Ray traversal of the scene LBVH (replaces OptiX traceRay + its built-in
// round-cubic curve and triangle intersectors, which the reference reaches
// through owl::traceRay in hair_msnn.cu:62 and optix_common.cuh:189,257).
//
// Node layout (64 B, 4 x float4): child 0 AABB, child 1 AABB, child indices
// (>= 0 internal node, < 0 leaf slot ~i).  A stack of 64 entries per ray; a
// ray whose stack would overflow or whose node count passes a fixed cap is
// reported through the error word instead of looping or writing out of
// bounds.
//
// Curves: uniform cubic B-spline segments (4 control points with radius).
// The intersector transforms the segment's Bezier control points into ray
// space (ray along +z), splits it uniformly into 2^D linear pieces with D
// chosen from the control polygon's flatness (ray-space subdivision of
// Nakamaru & Ohno 2002, with the flatness-to-depth rule and leaf test of
// Pharr, Jakob, Humphreys, PBRT-v3 section 3.7), and intersects each piece as
// a cone: the closest approach of the projected piece to the ray, then the
// front surface of the tube at that point.
#pragma once
#include "hm_scene.h"

namespace hm {

struct Ray {
  f3 o, d;
  float tmin, tmax;
};

struct Hit {
  float t;
  int prim;  // -1: miss
  float u, v;
};

enum { TRACE_ERR_STACK = 1, TRACE_ERR_STEPS = 2 };
constexpr int kStack = 64;
constexpr int kMaxVisits = 1 << 20;


HM_D bool tri_intersect(const SceneDev& s, int t_idx, const Ray& r, float tmax, float* t_out, float* u_out,
                        float* v_out) {
  const int3 tv = ldi3(s.tri + t_idx);
  const f3 v0 = ldf3(s.vtx + tv.x), v1 = ldf3(s.vtx + tv.y), v2 = ldf3(s.vtx + tv.z);
  const f3 e1 = v1 - v0, e2 = v2 - v0;
  const f3 pv = cross(r.d, e2);
  const float det = dot(e1, pv);
  if (fabsf(det) < 1e-20f) return false;
  const float inv = 1.f / det;
  const f3 tv0 = r.o - v0;
  const float u = dot(tv0, pv) * inv;
  if (u < 0.f || u > 1.f) return false;
  const f3 qv = cross(tv0, e1);
  const float v = dot(r.d, qv) * inv;
  if (v < 0.f || u + v > 1.f) return false;
  const float t = dot(e2, qv) * inv;
  if (!(t > r.tmin && t < tmax)) return false;
  *t_out = t;
  *u_out = u;
  *v_out = v;
  return true;
}

// Branchless orthonormal basis around a unit vector (Duff et al., JCGT 2017).
HM_D void onb(f3 n, f3* a, f3* b) {
  const float sign = copysignf(1.f, n.z);
  const float k = -1.f / (sign + n.z);
  const float m = n.x * n.y * k;
  *a = mk(1.f + sign * n.x * n.x * k, sign * m, -sign * n.x);
  *b = mk(m, sign + n.y * n.y * k, -n.y);
}

struct P4 {
  float x, y, z, r;
};
HM_D P4 lerp4(P4 a, P4 b, float t) {
  return P4{a.x + (b.x - a.x) * t, a.y + (b.y - a.y) * t, a.z + (b.z - a.z) * t, a.r + (b.r - a.r) * t};
}

HM_D bool curve_intersect(const SceneDev& s, int seg_idx, const Ray& r, float tmax, float* t_out, float* u_out) {
  const float4* q = s.cp + __ldg(s.seg + seg_idx);
  const float4 q0 = __ldg(q), q1 = __ldg(q + 1), q2 = __ldg(q + 2), q3 = __ldg(q + 3);
  // B-spline -> Bezier
  const float4 w0 = make_float4((q0.x + 4.f * q1.x + q2.x) * (1.f / 6.f), (q0.y + 4.f * q1.y + q2.y) * (1.f / 6.f),
                                (q0.z + 4.f * q1.z + q2.z) * (1.f / 6.f), (q0.w + 4.f * q1.w + q2.w) * (1.f / 6.f));
  const float4 w1 = make_float4((2.f * q1.x + q2.x) * (1.f / 3.f), (2.f * q1.y + q2.y) * (1.f / 3.f),
                                (2.f * q1.z + q2.z) * (1.f / 3.f), (2.f * q1.w + q2.w) * (1.f / 3.f));
  const float4 w2 = make_float4((q1.x + 2.f * q2.x) * (1.f / 3.f), (q1.y + 2.f * q2.y) * (1.f / 3.f),
                                (q1.z + 2.f * q2.z) * (1.f / 3.f), (q1.w + 2.f * q2.w) * (1.f / 3.f));
  const float4 w3 = make_float4((q1.x + 4.f * q2.x + q3.x) * (1.f / 6.f), (q1.y + 4.f * q2.y + q3.y) * (1.f / 6.f),
                                (q1.z + 4.f * q2.z + q3.z) * (1.f / 6.f), (q1.w + 4.f * q2.w + q3.w) * (1.f / 6.f));
  f3 ax, ay;
  onb(r.d, &ax, &ay);
  auto rs = [&](float4 w) {
    f3 p = mk(w.x, w.y, w.z) - r.o;
    return P4{dot(p, ax), dot(p, ay), dot(p, r.d), w.w};
  };
  const P4 b0 = rs(w0), b1 = rs(w1), b2 = rs(w2), b3 = rs(w3);
  const float rmax = fmaxf(fmaxf(b0.r, b1.r), fmaxf(b2.r, b3.r));
  // ray-space bounding rectangle of the control polygon (+ radius) must hold the ray
  if (fminf(fminf(b0.x, b1.x), fminf(b2.x, b3.x)) - rmax > 0.f ||
      fmaxf(fmaxf(b0.x, b1.x), fmaxf(b2.x, b3.x)) + rmax < 0.f ||
      fminf(fminf(b0.y, b1.y), fminf(b2.y, b3.y)) - rmax > 0.f ||
      fmaxf(fmaxf(b0.y, b1.y), fmaxf(b2.y, b3.y)) + rmax < 0.f ||
      fmaxf(fmaxf(b0.z, b1.z), fmaxf(b2.z, b3.z)) + rmax < r.tmin ||
      fminf(fminf(b0.z, b1.z), fminf(b2.z, b3.z)) - rmax > tmax)
    return false;
  // flatness -> subdivision depth (PBRT-v3 3.7): eps = width / 20
  const float l0 = fmaxf(fmaxf(fabsf(b0.x - 2.f * b1.x + b2.x), fabsf(b0.y - 2.f * b1.y + b2.y)),
                         fmaxf(fabsf(b1.x - 2.f * b2.x + b3.x), fabsf(b1.y - 2.f * b2.y + b3.y)));
  const float eps = fmaxf(rmax * 0.1f, 1e-12f);
  const float fr = 1.41421356f * 6.f * l0 / (8.f * eps);
  int depth = fr > 1.f ? (int)lrintf(0.5f * log2f(fr)) : 0;
  depth = min(max(depth, 0), 5);
  const int npieces = 1 << depth;
  const float inv_np = 1.f / (float)npieces;
  bool found = false;
  float best_t = tmax, best_u = 0.f;
  P4 a = b0;
  for (int k = 0; k < npieces; ++k) {
    // Bernstein evaluation at the piece's end
    const float tt = (float)(k + 1) * inv_np, s1 = 1.f - tt;
    const float c0 = s1 * s1 * s1, c1 = 3.f * s1 * s1 * tt, c2 = 3.f * s1 * tt * tt, c3 = tt * tt * tt;
    const P4 b = P4{c0 * b0.x + c1 * b1.x + c2 * b2.x + c3 * b3.x, c0 * b0.y + c1 * b1.y + c2 * b2.y + c3 * b3.y,
                    c0 * b0.z + c1 * b1.z + c2 * b2.z + c3 * b3.z, c0 * b0.r + c1 * b1.r + c2 * b2.r + c3 * b3.r};
    const float sx = b.x - a.x, sy = b.y - a.y;
    const float len2 = sx * sx + sy * sy;
    if (len2 > 0.f) {
      const float w = -(a.x * sx + a.y * sy) / len2;
      if (w >= 0.f && w < 1.f) {
        const P4 pc = lerp4(a, b, w);
        const float d2 = pc.x * pc.x + pc.y * pc.y;
        const float rr = pc.r * pc.r;
        if (d2 < rr) {
          const float t = pc.z - sqrtf(rr - d2);
          if (t > r.tmin && t < best_t) {
            best_t = t;
            best_u = ((float)k + w) * inv_np;
            found = true;
          }
        }
      }
    }
    a = b;
  }
  if (found) {
    *t_out = best_t;
    *u_out = best_u;
  }
  return found;
}

HM_D f3 safe_inv(f3 d) {
  auto inv = [](float x) { return fabsf(x) > 1e-20f ? 1.f / x : copysignf(1e20f, x); };
  return mk(inv(d.x), inv(d.y), inv(d.z));
}

// Slab test of both children of a node; returns entry distances (inf: miss).
HM_D void node_test(const float4* nodes, int ni, const f3& o, const f3& inv, float tmin, float tmax, float* t0,
                    float* t1, int* c0, int* c1) {
  const float4 a = __ldg(nodes + 4 * ni), b = __ldg(nodes + 4 * ni + 1), c = __ldg(nodes + 4 * ni + 2),
               d = __ldg(nodes + 4 * ni + 3);
  // child 0: lo (a.x, a.y, a.z) hi (a.w, b.x, b.y); child 1: lo (b.z, b.w, c.x) hi (c.y, c.z, c.w)
  {
    float tx0 = (a.x - o.x) * inv.x, tx1 = (a.w - o.x) * inv.x;
    float ty0 = (a.y - o.y) * inv.y, ty1 = (b.x - o.y) * inv.y;
    float tz0 = (a.z - o.z) * inv.z, tz1 = (b.y - o.z) * inv.z;
    float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), tmin));
    float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tmax));
    *t0 = tn <= tf ? tn : INFINITY;
  }
  {
    float tx0 = (b.z - o.x) * inv.x, tx1 = (c.y - o.x) * inv.x;
    float ty0 = (b.w - o.y) * inv.y, ty1 = (c.z - o.y) * inv.y;
    float tz0 = (c.x - o.z) * inv.z, tz1 = (c.w - o.z) * inv.z;
    float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), tmin));
    float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tmax));
    *t1 = tn <= tf ? tn : INFINITY;
  }
  *c0 = __float_as_int(d.x);
  *c1 = __float_as_int(d.y);
}

HM_D bool prim_intersect(const SceneDev& s, int prim, const Ray& r, float tmax, float* t, float* u, float* v) {
  if (prim < s.n_seg) {
    *v = 0.f;
    return curve_intersect(s, prim, r, tmax, t, u);
  }
  return tri_intersect(s, prim - s.n_seg, r, tmax, t, u, v);
}

// Work counters of a traversal (COUNT instantiations only).
struct TraceCount {
  uint32_t nodes, prims;
};

// Resumable traversal: one node visit per trav_step(), so a persistent
// kernel can hand a lane a new ray as soon as its previous ray finishes
// (dynamic ray fetching, Aila & Laine, HPG 2009).
struct TravState {
  f3 o, d, inv;
  float tmin;
  Hit h;
  int node;
  int sp;
  int visits;
  int pend;  // parked leaf slot, -1: none
};

HM_D void trav_init(TravState& t, f3 o, f3 d, float tmin, float tmax) {
  t.o = o;
  t.d = d;
  t.inv = mk(fabsf(d.x) > 1e-20f ? 1.f / d.x : copysignf(1e20f, d.x),
             fabsf(d.y) > 1e-20f ? 1.f / d.y : copysignf(1e20f, d.y),
             fabsf(d.z) > 1e-20f ? 1.f / d.z : copysignf(1e20f, d.z));
  t.tmin = tmin;
  t.h = Hit{tmax, -1, 0.f, 0.f};
  t.node = 0;
  t.sp = 0;
  t.visits = 0;
  t.pend = -1;
}

HM_D bool prim_intersect(const SceneDev& s, int prim, const Ray& r, float tmax, float* t, float* u, float* v);

// Leaf-postponing traversal ("while-while", Aila & Laine 2009): an inner
// step only walks boxes; a leaf reached is parked (t.pend = leaf slot) and
// tested later together with the other lanes' parked leaves, so the expensive
// curve test runs with most lanes of the warp active.
//   t.node >= 0: next internal node to visit; t.node < 0: pop next.
//   A lane needs inner steps while nothing is parked and work remains.
HM_D bool trav_needs_step(const TravState& t) { return t.pend < 0 && (t.node >= 0 || t.sp > 0); }
HM_D bool trav_finished(const TravState& t) { return t.pend < 0 && t.node < 0 && t.sp == 0; }

template <bool COUNT>
HM_D void trav_inner_step(const SceneDev& s, TravState& t, int* stack, int* err, TraceCount* cnt) {
  if (++t.visits > kMaxVisits) {
    atomicOr(err, TRACE_ERR_STEPS);
    t.node = -1;
    t.sp = 0;
    return;
  }
  int cur = t.node >= 0 ? t.node : stack[--t.sp];
  if (cur < 0) {  // a leaf left on the stack
    t.pend = ~cur;
    t.node = -1;
    return;
  }
  float t0, t1;
  int c0, c1;
  node_test(s.nodes, cur, t.o, t.inv, t.tmin, t.h.t, &t0, &t1, &c0, &c1);
  if (COUNT) cnt->nodes += 1;
  const bool go0 = t0 < INFINITY, go1 = t1 < INFINITY;
  int next = 0;
  bool have = true;
  if (go0 && go1) {
    if (t.sp >= kStack) {
      atomicOr(err, TRACE_ERR_STACK);
      t.node = -1;
      t.sp = 0;
      return;
    }
    stack[t.sp++] = t0 <= t1 ? c1 : c0;
    next = t0 <= t1 ? c0 : c1;
  } else if (go0) {
    next = c0;
  } else if (go1) {
    next = c1;
  } else {
    have = false;
  }
  if (!have) {
    t.node = -1;
  } else if (next < 0) {
    t.pend = ~next;
    t.node = -1;
  } else {
    t.node = next;
  }
}

// Tests the parked leaf.  Returns true if an any-hit ray is finished.
template <bool ANY_HIT, bool COUNT>
HM_D bool trav_leaf(const SceneDev& s, TravState& t, TraceCount* cnt) {
  if (t.pend < 0) return false;
  const int prim = __ldg(s.prim_of_leaf + t.pend);
  t.pend = -1;
  if (COUNT) cnt->prims += 1;
  float th, u, v;
  if (prim_intersect(s, prim, Ray{t.o, t.d, t.tmin, t.h.t}, t.h.t, &th, &u, &v)) {
    t.h = Hit{th, prim, u, v};
    if (ANY_HIT) return true;
  }
  return false;
}

// Returns true when the ray is finished (result in t.h).
template <bool ANY_HIT, bool COUNT>
HM_D bool trav_step(const SceneDev& s, TravState& t, int* stack, int* err, TraceCount* cnt) {
  if (++t.visits > kMaxVisits) {
    atomicOr(err, TRACE_ERR_STEPS);
    return true;
  }
  const Ray r{t.o, t.d, t.tmin, t.h.t};
  float t0, t1;
  int c0, c1;
  node_test(s.nodes, t.node, t.o, t.inv, t.tmin, t.h.t, &t0, &t1, &c0, &c1);
  if (COUNT) cnt->nodes += 1;
  if (COUNT) cnt->prims += (c0 < 0 && t0 < INFINITY) + (c1 < 0 && t1 < INFINITY);
  if (c0 < 0 && t0 < INFINITY) {
    float th, u, v;
    const int prim = __ldg(s.prim_of_leaf + ~c0);
    if (prim_intersect(s, prim, r, t.h.t, &th, &u, &v)) {
      t.h = Hit{th, prim, u, v};
      if (ANY_HIT) return true;
    }
    t0 = INFINITY;
    if (t1 > t.h.t) t1 = INFINITY;
  }
  if (c1 < 0 && t1 < INFINITY) {
    float th, u, v;
    const int prim = __ldg(s.prim_of_leaf + ~c1);
    if (prim_intersect(s, prim, Ray{t.o, t.d, t.tmin, t.h.t}, t.h.t, &th, &u, &v)) {
      t.h = Hit{th, prim, u, v};
      if (ANY_HIT) return true;
    }
    t1 = INFINITY;
    if (t0 > t.h.t) t0 = INFINITY;
  }
  const bool go0 = t0 < INFINITY, go1 = t1 < INFINITY;
  if (go0 && go1) {
    if (t.sp >= kStack) {
      atomicOr(err, TRACE_ERR_STACK);
      return true;
    }
    stack[t.sp++] = t0 <= t1 ? c1 : c0;
    t.node = t0 <= t1 ? c0 : c1;
  } else if (go0) {
    t.node = c0;
  } else if (go1) {
    t.node = c1;
  } else {
    if (t.sp == 0) return true;
    t.node = stack[--t.sp];
  }
  return false;
}

// ANY_HIT == true: return at the first hit in (tmin, tmax) (shadow rays).
template <bool ANY_HIT, bool COUNT = false>
HM_D Hit trace(const SceneDev& s, const Ray& r, int* err, TraceCount* cnt = nullptr) {
  Hit h{r.tmax, -1, 0.f, 0.f};
  const f3 inv = safe_inv(r.d);
  int stack[kStack];
  int sp = 0;
  int node = 0;
  int visits = 0;
  for (;;) {
    if (++visits > kMaxVisits) {
      atomicOr(err, TRACE_ERR_STEPS);
      return h;
    }
    float t0, t1;
    int c0, c1;
    node_test(s.nodes, node, r.o, inv, r.tmin, h.t, &t0, &t1, &c0, &c1);
    if (COUNT) cnt->nodes += 1;
    if (COUNT) cnt->prims += (c0 < 0 && t0 < INFINITY) + (c1 < 0 && t1 < INFINITY);
    // leaves first
    if (c0 < 0 && t0 < INFINITY) {
      float t, u, v;
      int prim = __ldg(s.prim_of_leaf + ~c0);
      if (prim_intersect(s, prim, r, h.t, &t, &u, &v)) {
        h = Hit{t, prim, u, v};
        if (ANY_HIT) return h;
      }
      t0 = INFINITY;
      if (t1 > h.t) t1 = INFINITY;
    }
    if (c1 < 0 && t1 < INFINITY) {
      float t, u, v;
      int prim = __ldg(s.prim_of_leaf + ~c1);
      if (prim_intersect(s, prim, r, h.t, &t, &u, &v)) {
        h = Hit{t, prim, u, v};
        if (ANY_HIT) return h;
      }
      t1 = INFINITY;
      if (t0 > h.t) t0 = INFINITY;
    }
    const bool go0 = t0 < INFINITY, go1 = t1 < INFINITY;
    if (go0 && go1) {
      int near = t0 <= t1 ? c0 : c1, far = t0 <= t1 ? c1 : c0;
      if (sp >= kStack) {
        atomicOr(err, TRACE_ERR_STACK);
        return h;
      }
      stack[sp++] = far;
      node = near;
    } else if (go0) {
      node = c0;
    } else if (go1) {
      node = c1;
    } else {
      // pop, skipping entries beyond the current closest hit is not possible
      // without their distances; they are re-tested (cheap, child boxes inline)
      if (sp == 0) return h;
      node = stack[--sp];
    }
  }
}

}  // namespace hm
