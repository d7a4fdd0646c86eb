// ORACLE procedural scenes (test infrastructure only).
//
// The synthetic stand-ins for the reference's missing assets, restated on
// the host so that the CPU baseline and the reference arm of the benchmark
// build their scene without the shipped library: straight / curly
// procedural hair (roots on the head's upper cap, B-spline control points),
// the head ellipsoid mesh, a Preetham-Shirley-Smits (1999) sky baked to a
// lat-long map, and the reference's environment sampling tables
// (generateEnvSamplingTables, scene.cpp:349-425).  The arrays equal the
// library's scene generator bit for bit on the same host (a CPU test checks
// it), so the two arms render the same scene.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "hm_oracle_math.h"

using namespace hmo;

namespace {

constexpr float kPiGen = 3.1415926f;  // the reference's Pi (utils.cuh:10)

uint32_t scene_rng(uint32_t seed) { return get_rng((int)seed, 0x4a1u, 0u, 1u, 1u); }

}  // namespace

extern "C" {

// Procedural hair: curly != 0 adds a helix about the running direction.
// cp_out [strands * cps][4] (x, y, z, radius), seg_out [strands * (cps - 3)]
// (first control point of each cubic segment).
void hmo_gen_hair(int curly, int strands, int cps, float length, float radius, float root_min_z, float helix_radius,
                  float helix_pitch, uint32_t seed, const float* head_r3, float* cp_out, int* seg_out) {
  const V3 hr(head_r3[0], head_r3[1], head_r3[2]);
  uint32_t st = scene_rng(seed);
  const float step = length / (float)(cps - 1);
  size_t ncp = 0, nseg = 0;
  auto inside = [&](V3 p, float m) {
    V3 q(p.x / (hr.x + m), p.y / (hr.y + m), p.z / (hr.z + m));
    return dot(q, q) < 1.f;
  };
  for (int k = 0; k < strands; ++k) {
    const float u1 = lcg_randomf(st), u2 = lcg_randomf(st);
    const float z = root_min_z + (1.f - root_min_z) * u1;
    const float r = sqrtf(fmaxf(0.f, 1.f - z * z));
    const float phi = 2.f * kPiGen * u2;
    const V3 n(r * cosf(phi), r * sinf(phi), z);
    V3 p(n.x * hr.x, n.y * hr.y, n.z * hr.z);
    V3 dir = normalize(V3(n.x / hr.x, n.y / hr.y, n.z / hr.z));
    const float jitter = 0.15f * (lcg_randomf(st) - 0.5f);
    const float hphase = 2.f * kPiGen * lcg_randomf(st);
    const int first = (int)ncp;
    for (int i = 0; i < cps; ++i) {
      V3 q = p;
      if (curly) {
        const V3 a = normalize(cross(dir, fabsf(dir.z) < 0.9f ? V3(0.f, 0.f, 1.f) : V3(1.f, 0.f, 0.f)));
        const V3 b = cross(dir, a);
        const float ang = hphase + 2.f * kPiGen * (float)i * step / helix_pitch;
        const float hrad = helix_radius * fminf(1.f, (float)i / 4.f);
        q = p + a * (hrad * cosf(ang)) + b * (hrad * sinf(ang));
      }
      float* c = cp_out + 4 * ncp++;
      c[0] = q.x; c[1] = q.y; c[2] = q.z; c[3] = radius;
      dir = normalize(dir + V3(jitter * dir.y, -jitter * dir.x, -0.12f));
      V3 np = p + dir * step;
      if (inside(np, 0.02f)) {
        const V3 o = normalize(V3(np.x / hr.x, np.y / hr.y, np.z / hr.z));
        np = V3(o.x * (hr.x + 0.021f), o.y * (hr.y + 0.021f), o.z * (hr.z + 0.021f));
        dir = normalize(np - p);
      }
      p = np;
    }
    for (int i = 0; i + 3 < cps; ++i) seg_out[nseg++] = first + i;
  }
}

// Head ellipsoid: a UV sphere of about `triangles` triangles scaled by the
// radii.  Call with NULL outputs for the sizes.
void hmo_gen_ellipsoid(int triangles, const float* radii3, float* vtx, float* nrm, int* tri, int* n_vtx,
                       int* n_tri) {
  const int nu = std::max(3, (int)lrintf(sqrtf((float)triangles / 2.f)));
  const int nv = std::max(2, (int)lrintf((float)triangles / (2.f * (float)nu)) + 1);
  *n_vtx = 2 + (nv - 1) * nu;
  *n_tri = 2 * nu + 2 * nu * (nv - 2);
  if (!vtx) return;
  const V3 R(radii3[0], radii3[1], radii3[2]);
  int iv = 0;
  auto push = [&](float th, float ph) {
    const V3 d(sinf(th) * cosf(ph), sinf(th) * sinf(ph), cosf(th));
    const V3 n = normalize(V3(d.x / R.x, d.y / R.y, d.z / R.z));
    vtx[3 * iv] = d.x * R.x; vtx[3 * iv + 1] = d.y * R.y; vtx[3 * iv + 2] = d.z * R.z;
    nrm[3 * iv] = n.x; nrm[3 * iv + 1] = n.y; nrm[3 * iv + 2] = n.z;
    ++iv;
  };
  push(0.f, 0.f);
  for (int v = 1; v < nv; ++v)
    for (int u = 0; u < nu; ++u) push(kPiGen * (float)v / (float)nv, 2.f * kPiGen * (float)u / (float)nu);
  push(kPiGen, 0.f);
  const int south = iv - 1;
  auto ring = [&](int v, int u) { return 1 + (v - 1) * nu + (u % nu); };
  int it = 0;
  auto tri3 = [&](int a, int b, int c) {
    tri[3 * it] = a; tri[3 * it + 1] = b; tri[3 * it + 2] = c;
    ++it;
  };
  for (int u = 0; u < nu; ++u) tri3(0, ring(1, u), ring(1, u + 1));
  for (int v = 1; v + 1 < nv; ++v)
    for (int u = 0; u < nu; ++u) {
      tri3(ring(v, u), ring(v + 1, u), ring(v + 1, u + 1));
      tri3(ring(v, u), ring(v + 1, u + 1), ring(v, u + 1));
    }
  for (int u = 0; u < nu; ++u) tri3(ring(nv - 1, u), south, ring(nv - 1, u + 1));
}

// Preetham-Shirley-Smits daylight (turbidity T, sun direction) as an RGBA
// lat-long map env [H][W][4]: the Perez distribution of Y, x, y with the
// paper's turbidity fits, xyY -> XYZ -> linear sRGB, normalised to a zenith
// luminance of 1, times `scale`; below the horizon a grey ground at 0.3 x
// the horizon's luminance.
void hmo_bake_sky(float T, const float* sun3, int W, int H, float scale, float* env) {
  const V3 sun = normalize(V3(sun3[0], sun3[1], sun3[2]));
  const double ths = acos(std::min(1.0, std::max(-1.0, (double)sun.z)));
  auto perez = [](const double c[5], double th, double gm) {
    const double ct = std::max(cos(th), 1e-3);
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
    const double Y = Yz * perez(cY, th, gm) / perez(cY, 0.0, ths);
    const double x = xz * perez(cx, th, gm) / perez(cx, 0.0, ths);
    const double y = yz * perez(cy, th, gm) / perez(cy, 0.0, ths);
    const double X = x / y * Y, Z = (1.0 - x - y) / y * Y;
    out[0] = 3.2406 * X - 1.5372 * Y - 0.4986 * Z;
    out[1] = -0.9689 * X + 1.8758 * Y + 0.0415 * Z;
    out[2] = 0.0557 * X - 0.2040 * Y + 1.0570 * Z;
    for (int c = 0; c < 3; ++c) out[c] = std::max(0.0, out[c] / Yz);
  };
  for (int y = 0; y < H; ++y) {
    const double th = M_PI * (y + 0.5) / H;
    for (int x = 0; x < W; ++x) {
      const double ph = 2.0 * M_PI * (x + 0.5) / W;
      const double d[3] = {sin(th) * cos(ph), sin(th) * sin(ph), cos(th)};
      double c[3];
      if (th <= M_PI / 2) {
        const double cg = d[0] * sun.x + d[1] * sun.y + d[2] * sun.z;
        sky(th, acos(std::min(1.0, std::max(-1.0, cg))), c);
      } else {
        double h[3];
        sky(M_PI / 2 - 1e-3, M_PI / 2, h);
        const double g = 0.3 * (0.2126 * h[0] + 0.7152 * h[1] + 0.0722 * h[2]);
        c[0] = g * 1.0;
        c[1] = g * 0.9;
        c[2] = g * 0.8;
      }
      float* e = env + 4 * ((size_t)y * W + x);
      e[0] = (float)(c[0] * scale);
      e[1] = (float)(c[1] * scale);
      e[2] = (float)(c[2] * scale);
      e[3] = 1.f;
    }
  }
}

// generateEnvSamplingTables (scene.cpp:349-425) in its single-precision
// order: conditional pdf / cdf [H][W + 1] (column W = the row's total),
// marginal pdf / cdf [H + 1].
void hmo_env_tables(const float* env, int W, int H, float* cpdf, float* ccdf, float* mpdf, float* mcdf) {
  const int cw = W + 1;
  auto avg = [&](int i) { return (env[4 * i] + env[4 * i + 1] + env[4 * i + 2]) * (1.0f / 3.0f); };
  for (int y = 0; y < H; ++y) {
    const float st = sinf(3.14159f * (y + 0.5f) / H);
    float* p = cpdf + (size_t)y * cw;
    float* c = ccdf + (size_t)y * cw;
    p[0] = avg(y * W) * st;
    c[0] = 0.f;
    for (int x = 1; x < W; ++x) {
      p[x] = avg(y * W + x) * st;
      c[x] = c[x - 1] + p[x - 1] / W;
    }
    const float total = c[W - 1] + p[W - 1] / W;
    p[W] = total;
    if (total > 0.f) {
      const float inv = 1.f / total;
      for (int x = 1; x < W; ++x) c[x] *= inv;
    }
    c[W] = 1.f;
  }
  mpdf[0] = cpdf[W];
  mcdf[0] = 0.f;
  for (int i = 1; i < H; ++i) {
    mpdf[i] = cpdf[(size_t)i * cw + W];
    mcdf[i] = mcdf[i - 1] + mpdf[i - 1] / H;
  }
  const float total = mcdf[H - 1] + mpdf[H - 1] / H;
  mpdf[H] = total;
  if (total > 0.f)
    for (int i = 1; i < H; ++i) mcdf[i] /= total;
  mcdf[H] = 1.f;
}

}  // extern "C"
