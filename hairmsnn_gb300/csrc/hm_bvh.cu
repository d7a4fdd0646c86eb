// Device LBVH over all primitives (hair segments, then head triangles).
// Replaces the OptiX GAS/IAS builds of the reference (owlGroupBuildAccel,
// render_hair_msnn.cu:316-384, 412): GB300 has no RT cores.
//
//   1. prim_bounds_kernel  per-primitive AABB (segment: hull of its 4 Bezier
//                          control points grown by their largest radius;
//                          triangle: its 3 vertices) + per-block scene bounds
//   2. morton_kernel       30-bit Morton code of each AABB centre in the
//                          scene bounds, key = code << 32 | primitive id
//                          (unique keys: no tie handling needed)
//   3. radix sort of the 64-bit keys (cub::DeviceRadixSort, setup only)
//   4. karras_kernel       binary radix tree (Karras, HPG 2012)
//   5. refit_kernel        bottom-up child AABBs, second arrival continues
//   6. wide_gather_kernel / wide_link_kernel
//                          collapse into 8-wide nodes, breadth first: the
//                          wide node of binary node r starts with r's
//                          children and repeatedly opens its internal child
//                          of largest surface area until it has 8; wide
//                          nodes are numbered level by level in the order
//                          their parents list them (an exclusive scan per
//                          level), so the array is the same on every run
//                          and equals the host build
//
// All float arithmetic uses explicitly rounded intrinsics (no contraction),
// so the node array is bit-identical to a host build of the same algorithm.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "hm_scene.h"

namespace hm {

struct Aabb {
  float lo[3], hi[3];
};

// One de Casteljau halving of a cubic Bezier (4 points x (x, y, z, r)):
// the left (right = 0) or right half, explicitly rounded.
HM_D void bezier_half(float w[4][4], int right) {
  for (int k = 0; k < 4; ++k) {
    const float m01 = __fmul_rn(__fadd_rn(w[0][k], w[1][k]), 0.5f);
    const float m12 = __fmul_rn(__fadd_rn(w[1][k], w[2][k]), 0.5f);
    const float m23 = __fmul_rn(__fadd_rn(w[2][k], w[3][k]), 0.5f);
    const float m012 = __fmul_rn(__fadd_rn(m01, m12), 0.5f);
    const float m123 = __fmul_rn(__fadd_rn(m12, m23), 0.5f);
    const float m = __fmul_rn(__fadd_rn(m012, m123), 0.5f);
    if (right) {
      w[0][k] = m; w[1][k] = m123; w[2][k] = m23;
    } else {
      w[1][k] = m01; w[2][k] = m012; w[3][k] = m;
    }
  }
}

HM_D Aabb prim_aabb(const SceneDev& s, int p) {
  Aabb b;
  if (p < s.n_hprim) {
    // hull of the Bezier control points of the segment's part (the curve
    // lies inside it), grown by their largest radius; the B-spline control
    // polygon spans three segments and gave boxes about three times too long
    const int part = p / s.n_seg;
    const float4* c = s.cp + s.seg[p - part * s.n_seg];
    float4 q[4] = {c[0], c[1], c[2], c[3]};
    float w[4][4];
    for (int k = 0; k < 4; ++k) {
      const float q0 = (&q[0].x)[k], q1 = (&q[1].x)[k], q2 = (&q[2].x)[k], q3 = (&q[3].x)[k];
      w[0][k] = __fmul_rn(__fadd_rn(__fadd_rn(q0, __fmul_rn(4.f, q1)), q2), 1.f / 6.f);
      w[1][k] = __fmul_rn(__fadd_rn(__fmul_rn(2.f, q1), q2), 1.f / 3.f);
      w[2][k] = __fmul_rn(__fadd_rn(q1, __fmul_rn(2.f, q2)), 1.f / 3.f);
      w[3][k] = __fmul_rn(__fadd_rn(__fadd_rn(q1, __fmul_rn(4.f, q2)), q3), 1.f / 6.f);
    }
    // part j of 2^L: halve L times, the bits of j from the top choosing the side
    for (int bit = s.seg_split >> 1; bit > 0; bit >>= 1) bezier_half(w, part & bit);
    const float r = fmaxf(fmaxf(w[0][3], w[1][3]), fmaxf(w[2][3], w[3][3]));
    for (int k = 0; k < 3; ++k) {
      b.lo[k] = __fsub_rn(fminf(fminf(w[0][k], w[1][k]), fminf(w[2][k], w[3][k])), r);
      b.hi[k] = __fadd_rn(fmaxf(fmaxf(w[0][k], w[1][k]), fmaxf(w[2][k], w[3][k])), r);
    }
  } else {
    int3 t = s.tri[p - s.n_hprim];
    float3 a = s.vtx[t.x], bb = s.vtx[t.y], c = s.vtx[t.z];
    b.lo[0] = fminf(fminf(a.x, bb.x), c.x);
    b.lo[1] = fminf(fminf(a.y, bb.y), c.y);
    b.lo[2] = fminf(fminf(a.z, bb.z), c.z);
    b.hi[0] = fmaxf(fmaxf(a.x, bb.x), c.x);
    b.hi[1] = fmaxf(fmaxf(a.y, bb.y), c.y);
    b.hi[2] = fmaxf(fmaxf(a.z, bb.z), c.z);
  }
  return b;
}

__global__ void prim_bounds_kernel(SceneDev s, int n, float* __restrict__ block_bounds) {
  __shared__ float red[6][256];
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    Aabb b = prim_aabb(s, p);
    for (int k = 0; k < 3; ++k) {
      lo[k] = fminf(lo[k], b.lo[k]);
      hi[k] = fmaxf(hi[k], b.hi[k]);
    }
  }
  for (int k = 0; k < 3; ++k) {
    red[k][threadIdx.x] = lo[k];
    red[3 + k][threadIdx.x] = hi[k];
  }
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int k = 0; k < 3; ++k) {
        red[k][threadIdx.x] = fminf(red[k][threadIdx.x], red[k][threadIdx.x + w]);
        red[3 + k][threadIdx.x] = fmaxf(red[3 + k][threadIdx.x], red[3 + k][threadIdx.x + w]);
      }
    __syncthreads();
  }
  if (threadIdx.x < 6) block_bounds[blockIdx.x * 6 + threadIdx.x] = red[threadIdx.x][0];
}

HM_HD uint32_t expand_bits10(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

HM_D uint32_t quantize10(float c, float lo, float ext) {
  float q = ext > 0.f ? __fdiv_rn(__fsub_rn(c, lo), ext) : 0.f;
  float v = fminf(fmaxf(__fmul_rn(q, 1024.f), 0.f), 1023.f);
  return (uint32_t)v;
}

__global__ void morton_kernel(SceneDev s, int n, const float* __restrict__ block_bounds, int nblocks,
                              unsigned long long* __restrict__ keys) {
  __shared__ float sb[6];
  if (threadIdx.x < 6) {
    float v = threadIdx.x < 3 ? INFINITY : -INFINITY;
    for (int b = 0; b < nblocks; ++b) {
      float x = block_bounds[b * 6 + threadIdx.x];
      v = threadIdx.x < 3 ? fminf(v, x) : fmaxf(v, x);
    }
    sb[threadIdx.x] = v;
  }
  __syncthreads();
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    Aabb b = prim_aabb(s, p);
    uint32_t q[3];
    for (int k = 0; k < 3; ++k) {
      float c = __fmul_rn(__fadd_rn(b.lo[k], b.hi[k]), 0.5f);
      q[k] = quantize10(c, sb[k], __fsub_rn(sb[3 + k], sb[k]));
    }
    uint32_t code = (expand_bits10(q[0]) << 2) | (expand_bits10(q[1]) << 1) | expand_bits10(q[2]);
    keys[p] = ((unsigned long long)code << 32) | (unsigned long long)(uint32_t)p;
  }
}

HM_D int delta(const unsigned long long* keys, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  return __clzll(keys[i] ^ keys[j]);
}

// Internal node i: children (>= 0 internal, < 0 leaf ~slot), parents.
__global__ void karras_kernel(const unsigned long long* __restrict__ keys, int n, int2* __restrict__ child,
                              int* __restrict__ parent_int, int* __restrict__ parent_leaf) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  int dmin = delta(keys, n, i, i - d);
  int lmax = 2;
  while (delta(keys, n, i, i + lmax * d) > dmin) lmax *= 2;
  int l = 0;
  for (int t = lmax / 2; t >= 1; t /= 2)
    if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
  int j = i + l * d;
  int dnode = delta(keys, n, i, j);
  int s = 0;
  for (int div = 2;; div *= 2) {
    int t = (l + div - 1) / div;
    if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    if (t <= 1) break;
  }
  int gamma = i + s * d + min(d, 0);
  int lo = min(i, j), hi = max(i, j);
  int left = lo == gamma ? ~gamma : gamma;
  int right = hi == gamma + 1 ? ~(gamma + 1) : gamma + 1;
  child[i] = make_int2(left, right);
  if (left < 0) parent_leaf[~left] = i; else parent_int[left] = i;
  if (right < 0) parent_leaf[~right] = i; else parent_int[right] = i;
}

HM_D void write_slot(float4* nodes, int node, int slot, const Aabb& b) {
  float* f = reinterpret_cast<float*>(nodes + 4 * node);
  const int o = slot * 6;
  for (int k = 0; k < 3; ++k) {
    f[o + k] = b.lo[k];
    f[o + 3 + k] = b.hi[k];
  }
}

__global__ void refit_kernel(SceneDev s, const unsigned long long* __restrict__ keys, int n,
                             const int2* __restrict__ child, const int* __restrict__ parent_int,
                             const int* __restrict__ parent_leaf, int* __restrict__ counters,
                             float4* __restrict__ nodes, int* __restrict__ prim_of_leaf) {
  int leaf = blockIdx.x * blockDim.x + threadIdx.x;
  if (leaf >= n) return;
  int prim = (int)(keys[leaf] & 0xffffffffull);
  prim_of_leaf[leaf] = prim;
  Aabb b = prim_aabb(s, prim);
  int node = parent_leaf[leaf];
  int slot = (child[node].x == ~leaf) ? 0 : 1;
  int cur = ~leaf;
  for (;;) {
    write_slot(nodes, node, slot, b);
    __threadfence();
    if (atomicAdd(counters + node, 1) == 0) return;  // first arrival: the sibling finishes
    __threadfence();
    const float* f = reinterpret_cast<const float*>(nodes + 4 * node);
    for (int k = 0; k < 3; ++k) {
      b.lo[k] = fminf(__ldcg(f + k), __ldcg(f + 6 + k));
      b.hi[k] = fmaxf(__ldcg(f + 3 + k), __ldcg(f + 9 + k));
    }
    cur = node;
    if (node == 0) return;
    int p = parent_int[node];
    slot = (child[p].x == cur) ? 0 : 1;
    node = p;
  }
}

__global__ void pack_children_kernel(const int2* __restrict__ child, int n_int, float4* __restrict__ nodes) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_int) return;
  int2 c = child[i];
  nodes[4 * i + 3] = make_float4(__int_as_float(c.x), __int_as_float(c.y), 0.f, 0.f);
}

// Single primitive: a root whose second child is an empty box.
__global__ void single_leaf_kernel(SceneDev s, float4* nodes, int* prim_of_leaf) {
  Aabb b = prim_aabb(s, 0);
  write_slot(nodes, 0, 0, b);
  Aabb e;
  for (int k = 0; k < 3; ++k) {
    e.lo[k] = INFINITY;
    e.hi[k] = -INFINITY;
  }
  write_slot(nodes, 0, 1, e);
  nodes[3] = make_float4(__int_as_float(~0), __int_as_float(~0), 0.f, 0.f);
  prim_of_leaf[0] = 0;
}

// ---- 8-wide collapse
HM_D void read_child(const float4* nodes, int node, int slot, float* lo, float* hi, int* code) {
  const float* f = reinterpret_cast<const float*>(nodes + 4 * (int64_t)node);
  for (int k = 0; k < 3; ++k) {
    lo[k] = f[6 * slot + k];
    hi[k] = f[6 * slot + 3 + k];
  }
  *code = __float_as_int(f[12 + slot]);
}

// Surface area / 2 of a box, explicitly rounded: the collapse's expansion order.
HM_D float half_area(const float* lo, const float* hi) {
  const float ex = __fsub_rn(hi[0], lo[0]), ey = __fsub_rn(hi[1], lo[1]), ez = __fsub_rn(hi[2], lo[2]);
  return __fadd_rn(__fadd_rn(__fmul_rn(ex, ey), __fmul_rn(ey, ez)), __fmul_rn(ex, ez));
}

// One thread per wide node of the level (binary root roots[i]).  The node
// starts with r's two children; while it has fewer than kWide, the internal
// child with the largest surface area (the first of equals) is replaced by
// its first child and its second child is appended.  Writes the boxes and
// leaf codes; internal children keep their binary index for now
// (wide_link_kernel renumbers them) and are counted in n_internal[i].
__global__ void wide_gather_kernel(const float4* __restrict__ bnodes, const int* __restrict__ roots, int n, int wbase,
                                   float4* __restrict__ wnodes, int* __restrict__ n_internal) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int r = roots[i];
  float lo[kWide][3], hi[kWide][3], area[kWide];
  int code[kWide];
  for (int slot = 0; slot < 2; ++slot) {
    read_child(bnodes, r, slot, lo[slot], hi[slot], &code[slot]);
    area[slot] = half_area(lo[slot], hi[slot]);
  }
  int k = 2;
  while (k < kWide) {
    int best = -1;
    float ba = 0.f;
    for (int j = 0; j < k; ++j)
      if (code[j] >= 0 && (best < 0 || area[j] > ba)) {
        best = j;
        ba = area[j];
      }
    if (best < 0) break;
    const int c = code[best];
    read_child(bnodes, c, 0, lo[best], hi[best], &code[best]);
    area[best] = half_area(lo[best], hi[best]);
    read_child(bnodes, c, 1, lo[k], hi[k], &code[k]);
    area[k] = half_area(lo[k], hi[k]);
    ++k;
  }
  int ni = 0;
  for (int j = 0; j < k; ++j) ni += code[j] >= 0;
  for (int j = k; j < kWide; ++j) {
    for (int a = 0; a < 3; ++a) lo[j][a] = hi[j][a] = INFINITY;
    code[j] = -1;
  }
  float* w = reinterpret_cast<float*>(wnodes + kWideF4 * (int64_t)(wbase + i));
  for (int j = 0; j < kWide; ++j) {
    for (int a = 0; a < 3; ++a) {
      w[2 * a * kWide + j] = lo[j][a];
      w[(2 * a + 1) * kWide + j] = hi[j][a];
    }
    w[6 * kWide + j] = __int_as_float(code[j]);
  }
  n_internal[i] = ni;
}

// Internal children of wide node wbase + i become the wide nodes
// next_base + offs[i] + 0, 1, ... (in slot order) and the next level's roots.
__global__ void wide_link_kernel(const int* __restrict__ offs, int n, int wbase, int next_base, float4* __restrict__ wnodes,
                                 int* __restrict__ next_roots) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int* child = reinterpret_cast<int*>(wnodes + kWideF4 * (int64_t)(wbase + i)) + 6 * kWide;
  int m = offs[i];
  for (int j = 0; j < kWide; ++j) {
    const int c = child[j];
    if (c >= 0) {
      next_roots[m] = c;
      child[j] = next_base + m;
      ++m;
    }
  }
}

int build_wide(Scene& sc, cudaStream_t st) {
  const int n_int = std::max(1, sc.n_prims() - 1);
  cudaFree(sc.d_wnodes);
  sc.d_wnodes = nullptr;
  sc.n_wnodes = 0;
  int *ra = nullptr, *rb = nullptr, *cnt = nullptr, *offs = nullptr;
  void* tmp = nullptr;
  size_t tmp_bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, cnt, offs, n_int + 1, st);
  cudaError_t e = cudaMalloc(&sc.d_wnodes, (size_t)n_int * kWideF4 * sizeof(float4));
  if (e == cudaSuccess) e = cudaMalloc(&ra, n_int * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&rb, n_int * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&cnt, (n_int + 1) * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&offs, (n_int + 1) * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&tmp, tmp_bytes);
  int status = HM_OK;
  if (e != cudaSuccess) {
    status = hm_cuda_status(e, "wide bvh alloc");
  } else {
    const int zero = 0;
    cudaMemcpyAsync(ra, &zero, sizeof(int), cudaMemcpyHostToDevice, st);
    int wbase = 0, n = 1;
    for (int level = 0; n > 0 && status == HM_OK; ++level) {
      if (wbase + n > n_int) {
        hm_set_error("wide bvh: node count overflow");
        status = HM_ECAPACITY;
        break;
      }
      wide_gather_kernel<<<(n + 255) / 256, 256, 0, st>>>(sc.d_nodes, ra, n, wbase, sc.d_wnodes, cnt);
      cudaMemsetAsync(cnt + n, 0, sizeof(int), st);
      cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, cnt, offs, n + 1, st);
      wide_link_kernel<<<(n + 255) / 256, 256, 0, st>>>(offs, n, wbase, wbase + n, sc.d_wnodes, rb);
      int next = 0;
      e = cudaMemcpyAsync(&next, offs + n, sizeof(int), cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) {
        status = hm_cuda_status(e, "wide bvh level");
        break;
      }
      wbase += n;
      n = next;
      std::swap(ra, rb);
    }
    sc.n_wnodes = wbase;
  }
  cudaFree(ra); cudaFree(rb); cudaFree(cnt); cudaFree(offs); cudaFree(tmp);
  // the array was sized for the bound (one wide node per binary inner
  // node); keep only what the tree uses
  if (status == HM_OK && sc.n_wnodes < n_int) {
    float4* exact = nullptr;
    e = cudaMalloc(&exact, (size_t)sc.n_wnodes * kWideF4 * sizeof(float4));
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(exact, sc.d_wnodes, (size_t)sc.n_wnodes * kWideF4 * sizeof(float4), cudaMemcpyDeviceToDevice,
                          st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) {
      cudaFree(sc.d_wnodes);
      sc.d_wnodes = exact;
    } else {
      cudaFree(exact);
      status = hm_cuda_status(e, "wide bvh compaction");
    }
  }
  return status;
}

int Scene::build_bvh(cudaStream_t st) {
  const int n = n_prims();
  if (n <= 0) return hm_set_error("scene has no primitives"), HM_EINVAL;
  SceneDev sd = dev();
  const int n_int = std::max(1, n - 1);
  cudaFree(d_nodes);
  cudaFree(d_prim_of_leaf);
  d_nodes = nullptr;
  d_prim_of_leaf = nullptr;
  cudaError_t e = cudaMalloc(&d_nodes, (size_t)n_int * 4 * sizeof(float4));
  if (e == cudaSuccess) e = cudaMalloc(&d_prim_of_leaf, (size_t)n * sizeof(int));
  if (e != cudaSuccess) return hm_cuda_status(e, "bvh alloc");
  n_nodes = n_int;
  if (n == 1) {
    sd.nodes = d_nodes;
    single_leaf_kernel<<<1, 1, 0, st>>>(sd, d_nodes, d_prim_of_leaf);
    HM_CHECK_LAUNCH("single_leaf_kernel");
    return build_wide(*this, st);
  }
  const int nb = std::min(1024, (n + 255) / 256);
  float* bb = nullptr;
  unsigned long long *keys = nullptr, *keys_sorted = nullptr;
  int2* child = nullptr;
  int *par_i = nullptr, *par_l = nullptr, *cnt = nullptr;
  void* tmp = nullptr;
  size_t tmp_bytes = 0;
  cub::DeviceRadixSort::SortKeys(nullptr, tmp_bytes, keys, keys_sorted, n, 0, 62, st);
  e = cudaMalloc(&bb, nb * 6 * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&keys, n * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc(&keys_sorted, n * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc(&child, n_int * sizeof(int2));
  if (e == cudaSuccess) e = cudaMalloc(&par_i, n_int * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&par_l, n * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&cnt, n_int * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&tmp, tmp_bytes);
  int status = HM_OK;
  if (e != cudaSuccess) {
    status = hm_cuda_status(e, "bvh scratch");
  } else {
    prim_bounds_kernel<<<nb, 256, 0, st>>>(sd, n, bb);
    morton_kernel<<<std::min(4096, (n + 255) / 256), 256, 0, st>>>(sd, n, bb, nb, keys);
    cub::DeviceRadixSort::SortKeys(tmp, tmp_bytes, keys, keys_sorted, n, 0, 62, st);
    cudaMemsetAsync(cnt, 0, n_int * sizeof(int), st);
    cudaMemsetAsync(par_i, 0xff, n_int * sizeof(int), st);
    karras_kernel<<<(n_int + 255) / 256, 256, 0, st>>>(keys_sorted, n, child, par_i, par_l);
    refit_kernel<<<(n + 255) / 256, 256, 0, st>>>(sd, keys_sorted, n, child, par_i, par_l, cnt, d_nodes,
                                                  d_prim_of_leaf);
    pack_children_kernel<<<(n_int + 255) / 256, 256, 0, st>>>(child, n_int, d_nodes);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) status = hm_cuda_status(e, "bvh build");
  }
  cudaFree(bb); cudaFree(keys); cudaFree(keys_sorted); cudaFree(child);
  cudaFree(par_i); cudaFree(par_l); cudaFree(cnt); cudaFree(tmp);
  if (status == HM_OK) status = build_wide(*this, st);
  return status;
}

}  // namespace hm
