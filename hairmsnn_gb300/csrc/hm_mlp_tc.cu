// Radiance-cache network forward on the 5th-generation tensor cores.
//
// One persistent CTA of 128 threads per SM slot; each CTA keeps every layer's
// weights in shared memory (loaded once) and walks 128-query tiles:
//   encode   thread t computes the encoded input row of query t of the tile
//            (same per-feature arithmetic as the FP32 encode kernel) and
//            stores it, rounded to FP16 / BF16 / E4M3, as the A operand
//   layers   thread 0 issues tcgen05.mma (M=128, N=width or 16, K=16/32 per
//            instruction) with A and B in shared memory and the FP32
//            accumulator in tensor memory, then tcgen05.commit to an mbarrier
//   epilogue every thread reads its row of the accumulator (tcgen05.ld
//            32x32b), applies ReLU and stores it as the next layer's A
//   output   the 16-column accumulator of the last layer -> out (FP32)
// Layer 0 is split along K into chunks when the encoded row does not fit
// next to the weights.
//
// Operand layout (both A and B, K-major, no swizzle): 8-row x 16-byte core
// matrices; for an R-row operand the byte at (row, kb) sits at
//   ((kb / 16) * (R / 8) + row / 8) * 128 + (row % 8) * 16 + kb % 16,
// so core matrices adjacent in K are 16*R bytes apart (leading byte offset)
// and those adjacent in M/N 128 bytes apart (stride byte offset).
//
// E4M3: weights carry one scale per layer (448 / amax of the layer), the
// activations one scale per query row (448 / amax of the row; for the
// encoded input an upper bound: 1 for Frequency/OneBlob/padding, |x| for
// Identity inputs, the table amax for hash grids).  Scaling rows of A scales
// rows of D, so the epilogue owning the row undoes it exactly.
//
// Every wait on the mbarrier is bounded; on expiry the kernel records the
// fact in a host-mapped flag, stops issuing work, frees its tensor memory
// and returns.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>

#include <string.h>

#include <algorithm>
#include <string>

#include "hm_mlp.cuh"

namespace hm {

enum { TC_FP16 = 1, TC_BF16 = 2, TC_E4M3 = 3 };
constexpr int kTcRows = 128;
constexpr int kTcThreads = 256;
constexpr int kTcSmemMax = 227 * 1024;
constexpr uint32_t kTcWaitLimit = 1u << 20;
constexpr float kE4M3Max = 448.f;

// ------------------------------------------------------------- PTX wrappers
HM_D uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

HM_D void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
HM_D void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
HM_D bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
HM_D bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t limit = kTcWaitLimit) {
  for (uint32_t i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
HM_D void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
HM_D void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// Named barrier over the nthreads threads (whole warps) of one warp group,
// returning the OR of v over them.
HM_D bool group_sync_or(int id, int nthreads, bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 q, %1, 0;\n\t"
      "bar.red.or.pred p, %2, %3, q;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(id), "r"(nthreads)
      : "memory");
  return r != 0;
}
HM_D void group_sync(int id, int nthreads) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory"); }
// The barrier's phase completes once `bytes` of asynchronous copies have
// landed (and the one arrival of this call).
HM_D void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
// One bulk copy global -> shared (16-byte aligned, a multiple of 16 bytes),
// completing on `bar`.
HM_D void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
HM_D void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
HM_D void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// warp-collective
HM_D void tmem_alloc(uint32_t* holder, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(holder)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
HM_D void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

template <bool F8>
HM_D void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
  if (F8)
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
  else
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
HM_D void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
// 16 consecutive FP32 columns of this thread's lane; the wait is in the same
// statement so no use of the registers can be scheduled before it.
HM_D void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Instruction descriptor: D = F32, A/B K-major, formats (kind::f16: 0 F16,
// 1 BF16; kind::f8f6f4: 0 E4M3), N >> 3 at bit 17, M >> 4 at bit 24.
HM_HD uint32_t tc_idesc(int m, int n, int fmt) {
  return (1u << 4) | ((uint32_t)fmt << 7) | ((uint32_t)fmt << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}
// Shared-memory descriptor, no swizzle: start, leading (K) and stride (M/N)
// byte offsets in 16-byte units, descriptor version 1.
HM_D uint64_t tc_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

HM_HD int64_t op_offset(int rows, int row, int kb) {
  return ((int64_t)(kb >> 4) * (rows >> 3) + (row >> 3)) * 128 + (row & 7) * 16 + (kb & 15);
}

// ------------------------------------------------------------ quantisation
template <int PREC>
HM_D uint32_t pack2(float a, float b) {
  if (PREC == TC_BF16) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
  } else {
    __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
  }
}
HM_D uint32_t pack4_e4m3(float a, float b, float c, float d) {
  const uint32_t lo = __nv_cvt_float2_to_fp8x2(make_float2(a, b), __NV_SATFINITE, __NV_E4M3);
  const uint32_t hi = __nv_cvt_float2_to_fp8x2(make_float2(c, d), __NV_SATFINITE, __NV_E4M3);
  return (lo & 0xFFFFu) | (hi << 16);
}

// ---------------------------------------------------------------- encoding
// Features are produced in increasing order and packed through a 128-bit
// shift register into 16-byte groups, one conflict-free store per group
// (the 32 rows of a warp are 32 consecutive 16-byte core-matrix rows);
// 16-bit operands take consecutive features in pairs where they can.
template <int PREC>
struct RowPacker {
  static constexpr int kPer = PREC == TC_E4M3 ? 16 : 8;  // values per 16 bytes
  uint32_t w0 = 0, w1 = 0, w2 = 0, w3 = 0;
  int cnt = 0, group;
  uint8_t* A;
  int row;
  float scale;
  uint8_t* mirror = nullptr;  // training: the row's operand bytes also go here
  // training with E4M3 operands: the row's features, unscaled, as FP16 (the
  // backward pass runs on FP16 operands)
  uint16_t* mirror16 = nullptr;
  HM_D RowPacker(uint8_t* a, int r, int first_group, float sc) : group(first_group), A(a), row(r), scale(sc) {}
  HM_D void push(float v) {
    constexpr int SH = PREC == TC_E4M3 ? 8 : 16;
    if (PREC == TC_E4M3 && mirror16) mirror16[group * kPer + cnt] = __half_as_ushort(__float2half_rn(v));
    uint32_t h;
    if (PREC == TC_E4M3)
      h = (uint32_t)__nv_cvt_float_to_fp8(v * scale, __NV_SATFINITE, __NV_E4M3);
    else if (PREC == TC_BF16)
      h = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v));
    else
      h = (uint32_t)__half_as_ushort(__float2half_rn(v));
    w0 = __funnelshift_r(w0, w1, SH);
    w1 = __funnelshift_r(w1, w2, SH);
    w2 = __funnelshift_r(w2, w3, SH);
    w3 = (w3 >> SH) | (h << (32 - SH));
    if (++cnt == kPer) flush();
  }
  // Two consecutive features: for 16-bit operands at an even fill, one
  // paired conversion (the same round-to-nearest of each value) and one
  // 32-bit step of the register; otherwise two pushes.
  HM_D void push2(float a, float b) {
    if (PREC == TC_E4M3 || (cnt & 1)) {
      push(a);
      push(b);
      return;
    }
    w0 = w1;
    w1 = w2;
    w2 = w3;
    w3 = pack2<PREC>(a, b);
    cnt += 2;
    if (cnt == kPer) flush();
  }
  HM_D void flush() {
    *reinterpret_cast<uint4*>(A + op_offset(kTcRows, row, group * 16)) = make_uint4(w0, w1, w2, w3);
    if (mirror) *reinterpret_cast<uint4*>(mirror + group * 16) = make_uint4(w0, w1, w2, w3);
    ++group;
    cnt = 0;
  }
};

// Encoded features [kb, ke) of one row (k >= n_enc: padding 1; k >= in_pad:
// 0, the extra K columns of the E4M3 layout carry zero weights).
// Identity / OneBlob / hash grid values use the arithmetic of encode_kernel;
// the Frequency pair (sin, cos) of 2^f * pi * x comes from sincospif, whose
// reduction is exact (encode_kernel forms the phase 2^f * x * 3.1415926 in
// FP32 and adds pi/2 for the cosine: at most ~5e-4 apart at 2^11, below the
// 16-bit operand rounding).  OneBlob bins more than two
// bins away from x (circularly) are exactly 0 in encode_kernel's formula and
// are not evaluated.
template <int PREC>
HM_D void enc_range(const MlpDims& d, const float* __restrict__ xin, const float* __restrict__ enc_params, int kb,
                    int ke, RowPacker<PREC>& pk) {
  for (int si = 0; si < d.n_segs; ++si) {
    const EncSeg& s = d.segs[si];
    const int lo = max(kb, s.out_off), hi = min(ke, s.out_off + s.n_out);
    if (lo >= hi) continue;
    const int j0 = lo - s.out_off, j1 = hi - s.out_off;
    if (s.type == ENC_IDENTITY) {
      int j = j0;
      for (; j + 1 < j1; j += 2) pk.push2(xin[s.in_off + j], xin[s.in_off + j + 1]);
      if (j < j1) pk.push(xin[s.in_off + j]);
    } else if (s.type == ENC_FREQUENCY) {
      int u = j0 >> 1;
      int dim = u / s.n_freq, f = u - dim * s.n_freq;
      for (int j = j0; j < j1;) {
        float sn, cs;
        sincospif(ldexpf(xin[s.in_off + dim], f), &sn, &cs);
        if (!(j & 1) && j + 1 < j1) {
          pk.push2(sn, cs);
          j += 2;
        } else {
          if (!(j & 1)) {
            pk.push(sn);
            ++j;
          }
          if (j < j1) {
            pk.push(cs);
            ++j;
          }
        }
        if (++f == s.n_freq) {
          f = 0;
          ++dim;
        }
      }
    } else if (s.type == ENC_ONEBLOB) {
      // the five bins around x (circularly) are evaluated once per input
      // dimension, without branches that would diverge across the rows of
      // a warp; every other bin is 0
      const float nb = (float)s.n_bins;
      int dim = j0 / s.n_bins, b = j0 - dim * s.n_bins;
      int b0 = 0;
      float wv[5];
      auto window = [&](int dm) {
        const float x = xin[s.in_off + dm];
        // bin of x on the period [0, 1) (x itself may lie outside it)
        b0 = (((int)floorf(x * nb)) % s.n_bins + s.n_bins) % s.n_bins;
        const float c0 = oneblob_cdf(0.f, x, nb);
        // mass of window bin t = right edge - left edge; bin t's right edge
        // is bin t+1's left edge (+1 where bin t is the last bin: the edge
        // wraps to 0), so six edge evaluations give the five masses
        float left[5];
        int wb[5];
#pragma unroll
        for (int t = 0; t < 5; ++t) {
          // (b0 - 2 + t) mod n_bins: b0 is in [0, n_bins), so with two or
          // more bins one correction lands in range (one bin: always 0)
          int w = b0 - 2 + t;
          w += w < 0 ? s.n_bins : 0;
          w -= w >= s.n_bins ? s.n_bins : 0;
          wb[t] = s.n_bins == 1 ? 0 : w;
          left[t] = wb[t] == 0 ? c0 : oneblob_cdf((float)wb[t] / nb, x, nb);
        }
        const float right4 = (wb[4] == s.n_bins - 1) ? c0 + 1.f : oneblob_cdf((float)(wb[4] + 1) / nb, x, nb);
#pragma unroll
        for (int t = 0; t < 5; ++t) {
          const float right = t < 4 ? ((wb[t] == s.n_bins - 1) ? left[t + 1] + 1.f : left[t + 1]) : right4;
          wv[t] = right - left[t];
        }
      };
      window(dim);
      auto bin_value = [&](int bb) {
        int dd = bb - b0;
        if (dd > (s.n_bins >> 1)) dd -= s.n_bins;
        if (dd < -(s.n_bins >> 1)) dd += s.n_bins;
        float v = 0.f;
        v = dd == -2 ? wv[0] : v;
        v = dd == -1 ? wv[1] : v;
        v = dd == 0 ? wv[2] : v;
        v = dd == 1 ? wv[3] : v;
        v = dd == 2 ? wv[4] : v;
        return v;
      };
      for (int j = j0; j < j1;) {
        if (b + 1 < s.n_bins && j + 1 < j1) {  // two bins of the same dimension
          pk.push2(bin_value(b), bin_value(b + 1));
          b += 2;
          j += 2;
        } else {
          pk.push(bin_value(b));
          ++b;
          ++j;
        }
        if (b == s.n_bins && j < j1) {
          b = 0;
          ++dim;
          window(dim);
        }
      }
    } else {  // hash grid
      const float* table = enc_params + s.param_off;
      const bool pair_table = s.n_feat == 2 && (reinterpret_cast<uintptr_t>(table) & 7) == 0;
      const float px = xin[s.in_off], py = xin[s.in_off + 1], pz = xin[s.in_off + 2];
      int l = j0 / s.n_feat, f0 = j0 - l * s.n_feat;
      for (int j = j0; j < j1; ++l) {
        const float sc = s.level_scale[l];
        const float fx = fmaf(sc, px, 0.5f), fy = fmaf(sc, py, 0.5f), fz = fmaf(sc, pz, 0.5f);
        const float gx = floorf(fx), gy = floorf(fy), gz = floorf(fz);
        const float wx = fx - gx, wy = fy - gy, wz = fz - gz;
        const uint32_t ix = (uint32_t)(int)gx, iy = (uint32_t)(int)gy, iz = (uint32_t)(int)gz;
        float acc[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) acc[q] = 0.f;
        if (pair_table) {
          // two features per entry: the eight corners' entries are loaded
          // first (eight 8-byte gathers in flight), then accumulated in
          // corner order as below
          float2 tv[8];
#pragma unroll
          for (int c = 0; c < 8; ++c) {
            const uint32_t cx = ix + (c & 1), cy = iy + ((c >> 1) & 1), cz = iz + ((c >> 2) & 1);
            const uint32_t e = s.level_off[l] + grid_index(s, l, cx, cy, cz);
            tv[c] = __ldg(reinterpret_cast<const float2*>(table) + e);
          }
#pragma unroll
          for (int c = 0; c < 8; ++c) {
            const float w = ((c & 1) ? wx : 1.f - wx) * (((c >> 1) & 1) ? wy : 1.f - wy) *
                            (((c >> 2) & 1) ? wz : 1.f - wz);
            acc[0] += w * tv[c].x;
            acc[1] += w * tv[c].y;
          }
        } else {
          for (int c = 0; c < 8; ++c) {
            const uint32_t cx = ix + (c & 1), cy = iy + ((c >> 1) & 1), cz = iz + ((c >> 2) & 1);
            const float w = ((c & 1) ? wx : 1.f - wx) * (((c >> 1) & 1) ? wy : 1.f - wy) *
                            (((c >> 2) & 1) ? wz : 1.f - wz);
            const uint32_t e = s.level_off[l] + grid_index(s, l, cx, cy, cz);
            const float* tv = table + (int64_t)e * s.n_feat;
#pragma unroll
            for (int q = 0; q < 8; ++q)
              if (q < s.n_feat) acc[q] += w * __ldg(tv + q);
          }
        }
#pragma unroll
        for (int q = 0; q < 8; q += 2) {
          const bool ok0 = q >= f0 && q < s.n_feat && j < j1;
          const bool ok1 = q + 1 >= f0 && q + 1 < s.n_feat && j + (ok0 ? 1 : 0) < j1;
          if (ok0 && ok1) {
            pk.push2(acc[q], acc[q + 1]);
            j += 2;
          } else {
            if (ok0) {
              pk.push(acc[q]);
              ++j;
            }
            if (ok1) {
              pk.push(acc[q + 1]);
              ++j;
            }
          }
        }
        f0 = 0;
      }
    }
  }
  int k = max(kb, d.n_enc);
  for (; k + 1 < ke; k += 2) pk.push2(k < d.in_pad ? 1.f : 0.f, k + 1 < d.in_pad ? 1.f : 0.f);
  if (k < ke) pk.push(k < d.in_pad ? 1.f : 0.f);
}

// Upper bound of |feature| over the row (E4M3 input scale).
HM_D float enc_row_bound(const MlpDims& d, const float* __restrict__ xin, float grid_amax) {
  float m = 1.f;
  for (int si = 0; si < d.n_segs; ++si) {
    const EncSeg& s = d.segs[si];
    if (s.type == ENC_IDENTITY)
      for (int k = 0; k < s.n_dims; ++k) m = fmaxf(m, fabsf(xin[s.in_off + k]));
    else if (s.type == ENC_HASHGRID)
      m = fmaxf(m, grid_amax);
  }
  return m;
}

// --------------------------------------------------------------- the kernel
struct TcArgs {
  MlpDims d;
  const uint8_t* blob;
  int64_t blob_bytes;
  int64_t boff[16];
  int N[16], K[16];
  int n_layers;
  int kc0;  // layer-0 K chunk (elements)
  const float* scales;
  const float* enc_params;
  const float* in;
  float* out;
  int out_stride;
  int64_t n;
  int* err;  // host-mapped
  int a_bytes;
  int ncols;
  // training forward (STORE): operands kept for the backward pass
  uint16_t* x16;  // [n][K0]
  uint16_t* h16;  // [L][n][W]
  float* pred;    // [n][16]
  // inference with the encoding done beforehand by tc_encode_kernel: the
  // layer-0 operand of tile t is the tile_bytes at a_pre + t * tile_bytes, in
  // the MMA layout; E4M3 rows carry their activation scale in row_inv_pre
  const uint8_t* a_pre;
  const float* row_inv_pre;
  int64_t tile_bytes;
  // warp-specialised inference: shared-memory bytes of the weights, of one
  // layer-0 operand stage and of one hidden operand; number of stages
  int fz_w, fz_a0, fz_h, fz_stages;
};

// Encoding of every row into the layer-0 operand, in the MMA's shared-memory
// layout one tile after another, so the forward kernel loads a tile (or a K
// chunk of it) with one bulk copy.  One thread per row, 128 rows (one tile)
// per block: the 32 rows of a warp write each 16-byte group as four 128-byte
// runs.  Same arithmetic as the fused encoding (enc_range).
template <int PREC>
__global__ void __launch_bounds__(kTcRows) tc_encode_kernel(const __grid_constant__ TcArgs p, uint8_t* __restrict__ a_out,
                                                            float* __restrict__ row_inv_out) {
  const int row = threadIdx.x;
  const int64_t tile = blockIdx.x;
  const int64_t q = tile * kTcRows + row;
  const bool valid = q < p.n;
  const MlpDims& d = p.d;
  const float* xin = p.in + (valid ? q : 0) * d.in_ch;
  float row_scale = 1.f;
  if (PREC == TC_E4M3) {
    const float bound = valid ? enc_row_bound(d, xin, p.scales[15]) : 1.f;
    row_scale = kE4M3Max / bound;
    if (valid) row_inv_out[q] = bound / kE4M3Max;
  }
  RowPacker<PREC> pk(a_out + tile * p.tile_bytes, row, 0, row_scale);
  const int K0 = p.K[0];
  if (valid) {
    enc_range<PREC>(d, xin, p.enc_params, 0, K0, pk);
  } else {
    for (int k = 0; k < K0; ++k) pk.push(0.f);
  }
}

// 256 threads: thread (warp w, lane i) owns row 32 * (w % 4) + i of the tile
// (tensor-memory lanes are split by warp quadrant) and half h = w / 4 of the
// work on that row: every other 16-byte feature group when encoding, and
// accumulator columns [h * W/2, (h + 1) * W/2) in the epilogues.
template <int PREC, int W, bool STORE>
__global__ void __launch_bounds__(kTcThreads, 2) mlp_tc_fwd_kernel(const __grid_constant__ TcArgs p) {
  constexpr bool F8 = PREC == TC_E4M3;
  constexpr int EB = F8 ? 1 : 2;       // bytes per element
  constexpr int KI = 32 / EB;          // K per MMA instruction
  constexpr int CK = 16 / EB;          // elements per 16-byte core-matrix row
  constexpr int FMT = PREC == TC_BF16 ? 1 : 0;
  constexpr int HW = W / 2;            // accumulator columns per half
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* A = smem;
  uint8_t* Wt = smem + p.a_bytes;
  uint64_t* bar = reinterpret_cast<uint64_t*>(Wt + ((p.blob_bytes + 127) & ~(int64_t)127));
  uint64_t* bar_a = bar + 1;  // bulk copies of pre-encoded operands
  uint32_t* holder = reinterpret_cast<uint32_t*>(bar + 2);
  float* amax_x = reinterpret_cast<float*>(holder + 4);  // [2][128] E4M3 row maxima

  const int tid = threadIdx.x, warp = tid >> 5;
  const int row = ((warp & 3) << 5) | (tid & 31);
  const int half = warp >> 2;
  const MlpDims& d = p.d;
  const int L = p.n_layers - 1;  // index of the output layer

  for (int64_t i = tid; i < p.blob_bytes / 16; i += kTcThreads)
    reinterpret_cast<uint4*>(Wt)[i] = __ldg(reinterpret_cast<const uint4*>(p.blob) + i);
  if (tid == 0) {
    mbar_init(bar, 1);
    mbar_init(bar_a, 1);
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(holder, p.ncols);
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *holder;
  const uint32_t row_taddr = tmem + ((uint32_t)((warp & 3) * 32) << 16);
  const uint32_t a_base = smem_u32(A), w_base = smem_u32(Wt);
  const uint32_t a_lbo = 16 * kTcRows;
  uint32_t phase = 0, phase_a = 0;
  bool failed = false;
  auto w_inv = [&](int l) { return F8 ? __ldg(p.scales + l) : 1.f; };
  const float grid_amax = F8 ? p.scales[15] : 0.f;

  // issue the MMAs of one layer (or layer-0 chunk) and wait for them
  auto run_layer = [&](int l, int k_begin, int k_count, bool accumulate_first) -> bool {
    if (tid == 0) {
      tc_fence_after();
      const uint32_t idesc = tc_idesc(kTcRows, p.N[l], FMT);
      const uint32_t b_lbo = 16 * p.N[l];
      const uint32_t b_base = w_base + (uint32_t)p.boff[l];
      for (int ks = 0; ks < k_count / KI; ++ks) {
        const uint64_t ad = tc_sdesc(a_base + (uint32_t)ks * 2 * a_lbo, a_lbo, 128);
        const uint64_t bd = tc_sdesc(b_base + (uint32_t)((k_begin / KI) + ks) * 2 * b_lbo, b_lbo, 128);
        tc_mma<F8>(tmem, ad, bd, idesc, (accumulate_first || ks > 0) ? 1u : 0u);
      }
      tc_commit(bar);
    }
    // thread 0 (which committed) polls the barrier; the others sleep in the
    // block barrier instead of spinning
    const bool ok = threadIdx.x == 0 ? mbar_wait_bounded(bar, phase) : true;
    phase ^= 1u;
    const bool bad = __syncthreads_or(!ok);
    tc_fence_after();
    return !bad;
  };

  const int64_t n_tiles = (p.n + kTcRows - 1) / kTcRows;
  for (int64_t tile = blockIdx.x; tile < n_tiles && !failed; tile += gridDim.x) {
    const int64_t q = tile * kTcRows + row;
    const bool valid = q < p.n;
    const float* xin = p.in + (valid ? q : 0) * d.in_ch;
    float row_inv = 1.f;  // 1 / activation scale of this row of A
    float row_scale = 1.f;
    if (F8) {
      if (p.a_pre) {
        row_inv = valid ? __ldg(p.row_inv_pre + q) : 1.f;
      } else {
        const float bound = valid ? enc_row_bound(d, xin, grid_amax) : 1.f;
        row_scale = kE4M3Max / bound;
        row_inv = bound / kE4M3Max;
      }
    }
    // ---- layer 0, in K chunks
    const int K0 = p.K[0];
    for (int kc = 0; kc < K0 && !failed; kc += p.kc0) {
      const int kn = min(p.kc0, K0 - kc);
      if (p.a_pre) {
        // the chunk's K range is one contiguous run of the tile in the MMA layout
        if (tid == 0) {
          fence_proxy_async_smem();  // the previous tile's epilogue wrote A through the generic proxy
          const uint32_t bytes = (uint32_t)(kn * EB * kTcRows);
          mbar_arrive_expect_tx(bar_a, bytes);
          bulk_copy_g2s(A, p.a_pre + tile * p.tile_bytes + (int64_t)kc * EB * kTcRows, bytes, bar_a);
        }
        const bool ok = tid == 0 ? mbar_wait_bounded(bar_a, phase_a) : true;
        phase_a ^= 1u;
        if (__syncthreads_or(!ok)) {
          failed = true;
          break;
        }
      } else {
        // the two halves of the row: groups [0, G/2) and [G/2, G) of the chunk
        const int G = kn / CK, gsplit = (G + 1) >> 1;
        const int g0 = half ? gsplit : 0, g1 = half ? G : gsplit;
        RowPacker<PREC> pk(A, row, g0, row_scale);
        if (STORE && valid) {
          if (F8)
            pk.mirror16 = p.x16 + q * K0 + kc;
          else
            pk.mirror = reinterpret_cast<uint8_t*>(p.x16 + q * K0 + kc);
        }
        if (valid) {
          enc_range<PREC>(d, xin, p.enc_params, kc + g0 * CK, kc + g1 * CK, pk);
        } else {
          for (int k = g0 * CK; k < g1 * CK; ++k) pk.push(0.f);
        }
        fence_proxy_async_smem();
        __syncthreads();
      }
      if (!run_layer(0, kc, kn, kc > 0)) failed = true;
    }
    // ---- hidden epilogues and the following layers
    for (int l = 1; l <= L && !failed; ++l) {
      const float sc = row_inv * w_inv(l - 1);
      float v[HW];
#pragma unroll
      for (int c = 0; c < HW / 16; ++c) {
        float t[16];
        tmem_ld16(row_taddr + half * HW + c * 16, t);
#pragma unroll
        for (int e = 0; e < 16; ++e) v[c * 16 + e] = fmaxf(F8 ? t[e] * sc : t[e], 0.f);
      }
      if (F8) {
        float amax = 0.f;
#pragma unroll
        for (int e = 0; e < HW; ++e) amax = fmaxf(amax, v[e]);
        amax_x[half * kTcRows + row] = amax;
        __syncthreads();
        amax = fmaxf(amax_x[row], amax_x[kTcRows + row]);
        const float s = amax > 0.f ? kE4M3Max / amax : 1.f;
        row_inv = amax > 0.f ? amax / kE4M3Max : 1.f;
#pragma unroll
        for (int g = 0; g < HW / 16; ++g) {
          uint32_t word[4];
#pragma unroll
          for (int w4 = 0; w4 < 4; ++w4)
            word[w4] = pack4_e4m3(v[g * 16 + 4 * w4] * s, v[g * 16 + 4 * w4 + 1] * s, v[g * 16 + 4 * w4 + 2] * s,
                                  v[g * 16 + 4 * w4 + 3] * s);
          *reinterpret_cast<uint4*>(A + op_offset(kTcRows, row, half * HW + g * 16)) =
              make_uint4(word[0], word[1], word[2], word[3]);
        }
        if (STORE && valid) {  // the backward pass's FP16 copy of the activations
#pragma unroll
          for (int g = 0; g < HW / 8; ++g) {
            uint32_t word[4];
#pragma unroll
            for (int w2 = 0; w2 < 4; ++w2) word[w2] = pack2<TC_FP16>(v[g * 8 + 2 * w2], v[g * 8 + 2 * w2 + 1]);
            *reinterpret_cast<uint4*>(p.h16 + ((int64_t)(l - 1) * p.n + q) * W + half * HW + g * 8) =
                make_uint4(word[0], word[1], word[2], word[3]);
          }
        }
      } else {
#pragma unroll
        for (int g = 0; g < HW / 8; ++g) {
          uint32_t word[4];
#pragma unroll
          for (int w2 = 0; w2 < 4; ++w2) word[w2] = pack2<PREC>(v[g * 8 + 2 * w2], v[g * 8 + 2 * w2 + 1]);
          *reinterpret_cast<uint4*>(A + op_offset(kTcRows, row, (half * HW + g * 8) * 2)) =
              make_uint4(word[0], word[1], word[2], word[3]);
          if (STORE && valid)
            *reinterpret_cast<uint4*>(p.h16 + ((int64_t)(l - 1) * p.n + q) * W + half * HW + g * 8) =
                make_uint4(word[0], word[1], word[2], word[3]);
        }
      }
      tc_fence_before();
      fence_proxy_async_smem();
      __syncthreads();
      if (!run_layer(l, 0, p.K[l], false)) failed = true;
    }
    if (failed) break;
    // ---- output layer accumulator -> out (columns 0..15, first half of the warps)
    if (half == 0) {
      float t[16];
      tmem_ld16(row_taddr, t);
      const float sc = row_inv * w_inv(L);
      if (valid) {
        if (STORE) {
#pragma unroll
          for (int o = 0; o < 16; ++o) p.pred[q * 16 + o] = t[o] * sc;
        } else {
#pragma unroll
          for (int o = 0; o < 16; ++o)
            if (o < d.out_ch && o < p.out_stride) p.out[q * p.out_stride + o] = t[o] * sc;
        }
      }
    }
    tc_fence_before();
    __syncthreads();
  }
  if (failed && tid == 0) atomicOr(p.err, 1);
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, p.ncols);
}

// ---------------------------------------------- warp-specialised inference
// Encoding and layers overlapped inside one persistent CTA per SM (16-bit
// operands).  24 encoder warps write layer-0 operands into a ring of NS
// stages (each the whole K of one 128-row tile): they form NS teams of
// 4 * P warps, team t encoding the CTA's tiles k = t (mod NS) into stage t
// with P threads per row (each an equal contiguous range of the row's
// 16-byte feature groups; P = 6 / NS with NS 6 or 2, the most stages that
// fit next to the weights, so small operands get one thread per row as in
// tc_encode_kernel).  Two lanes of 4 layer warps walk the layers: lane s
// takes the tiles k = s (mod 2) (with NS even, stage t always feeds lane
// t % 2), with its own hidden operand H[s] (128 x W) and W columns of
// tensor memory; warp w reads tensor-memory lanes 32 * (w % 4) .. (one
// thread per row) and the lane's first thread issues the MMAs.  A team refills its stage as soon as the layer-0 MMAs of its
// previous tile have read it, so encoding runs while the layer warps walk
// layers 1..L, and the two lanes fill each other's waits.  Hand-offs:
// full[t] (team -> layer lane, one arrival after the team's named barrier),
// empty[t] (layer-0 MMAs done -> team), mma[s] (tcgen05.commit).  Every
// mbarrier wait is bounded; an expired wait is reduced over the waiting
// group through its named barrier, the group stops and the waits of the
// groups that depend on it then expire too.  The encoded operands, the MMAs
// and the epilogue arithmetic are those of mlp_tc_fwd_kernel, so the
// outputs are the same bits.
constexpr int kFzLanes = 2;
constexpr int kFzLayWarps = 4;   // per lane
constexpr int kFzEncWarps = 24;  // in all
constexpr int kFzLayThreads = kFzLanes * kFzLayWarps * 32;
constexpr int kFzThreads = kFzLayThreads + kFzEncWarps * 32;
constexpr int kFzMaxStages = kFzEncWarps / 4;
constexpr int kFzMisc = 128;  // 2 * kFzMaxStages + 2 mbarriers + the tensor-memory address

template <int PREC, int W>
__global__ void __launch_bounds__(kFzThreads, 1) mlp_tc_fused_kernel(const __grid_constant__ TcArgs p) {
  static_assert(PREC != TC_E4M3, "16-bit operands only");
  static_assert(8 * (2 * kFzMaxStages + 2) + 4 <= kFzMisc, "barrier area");
  constexpr int CK = 8;  // elements per 16-byte core-matrix row
  constexpr int FMT = PREC == TC_BF16 ? 1 : 0;
  extern __shared__ __align__(1024) uint8_t smem[];
  const int NS = p.fz_stages, P = kFzMaxStages / NS;
  uint8_t* Wt = smem;
  uint8_t* A0 = smem + p.fz_w;
  uint8_t* Hb = A0 + NS * p.fz_a0;
  uint64_t* bars = reinterpret_cast<uint64_t*>(Hb + kFzLanes * p.fz_h);
  uint64_t* full = bars;                 // [NS]
  uint64_t* empty = bars + kFzMaxStages;  // [NS]
  uint64_t* mma = bars + 2 * kFzMaxStages;  // [2]
  uint32_t* holder = reinterpret_cast<uint32_t*>(bars + 2 * kFzMaxStages + 2);

  const int tid = threadIdx.x, warp = tid >> 5, lane_id = tid & 31;
  const MlpDims& d = p.d;
  const int L = p.n_layers - 1;
  const int K0 = p.K[0];
  const int64_t n_tiles = (p.n + kTcRows - 1) / kTcRows;

  for (int64_t i = tid; i < p.blob_bytes / 16; i += kFzThreads)
    reinterpret_cast<uint4*>(Wt)[i] = __ldg(reinterpret_cast<const uint4*>(p.blob) + i);
  if (tid == 0) {
    for (int b = 0; b < 2 * kFzMaxStages + 2; ++b) mbar_init(bars + b, 1);
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(holder, p.ncols);
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *holder;
  bool failed = false;

  if (tid < kFzLayThreads) {
    // ---------------- layer warps of lane s
    const int s = warp / kFzLayWarps, quad = warp % 4, row = quad * 32 + lane_id;
    const int bar_id = 1 + s;
    const bool leader = (warp % kFzLayWarps) == 0 && lane_id == 0;
    const uint32_t tm = tmem + (uint32_t)(s * W);
    const uint32_t row_taddr = tm + ((uint32_t)(quad * 32) << 16);
    uint8_t* Hs = Hb + s * p.fz_h;
    uint64_t* mma_s = mma + s;
    const uint32_t a_lbo = 16 * kTcRows;
    const uint32_t h_base = smem_u32(Hs), w_base = smem_u32(Wt);
    uint32_t ph_mma = 0;
    // the MMAs of layer l over A (k_count elements of K), committed to mma_s
    auto issue = [&](int l, uint32_t a_base, int k_count) {
      tc_fence_after();
      const uint32_t idesc = tc_idesc(kTcRows, p.N[l], FMT);
      const uint32_t b_lbo = 16 * p.N[l];
      const uint32_t b_base = w_base + (uint32_t)p.boff[l];
      for (int ks = 0; ks < k_count / 16; ++ks) {
        const uint64_t ad = tc_sdesc(a_base + (uint32_t)ks * 2 * a_lbo, a_lbo, 128);
        const uint64_t bd = tc_sdesc(b_base + (uint32_t)ks * 2 * b_lbo, b_lbo, 128);
        tc_mma<false>(tm, ad, bd, idesc, ks > 0 ? 1u : 0u);
      }
      tc_commit(mma_s);
    };
    for (int64_t k = s;; k += kFzLanes) {
      const int64_t tile = blockIdx.x + k * (int64_t)gridDim.x;
      if (tile >= n_tiles) break;
      const int st = (int)(k % NS);
      bool ok = true;
      if (leader) {
        ok = mbar_wait_bounded(full + st, (uint32_t)((k / NS) & 1));
        if (ok) {
          issue(0, smem_u32(A0 + st * p.fz_a0), K0);
          ok = mbar_wait_bounded(mma_s, ph_mma);
          if (ok) mbar_arrive(empty + st);  // the stage has been read
        }
      }
      ph_mma ^= 1u;
      if (group_sync_or(bar_id, kFzLayWarps * 32, !ok)) {
        failed = true;
        break;
      }
      tc_fence_after();
      for (int l = 1; l <= L; ++l) {
        // epilogue of layer l - 1: ReLU, rounded to the operand type, as the A of layer l
#pragma unroll
        for (int c = 0; c < W / 16; ++c) {
          float t[16];
          tmem_ld16(row_taddr + c * 16, t);
#pragma unroll
          for (int g = 0; g < 2; ++g) {
            uint32_t word[4];
#pragma unroll
            for (int w2 = 0; w2 < 4; ++w2)
              word[w2] = pack2<PREC>(fmaxf(t[g * 8 + 2 * w2], 0.f), fmaxf(t[g * 8 + 2 * w2 + 1], 0.f));
            *reinterpret_cast<uint4*>(Hs + op_offset(kTcRows, row, (c * 16 + g * 8) * 2)) =
                make_uint4(word[0], word[1], word[2], word[3]);
          }
        }
        tc_fence_before();
        fence_proxy_async_smem();
        group_sync(bar_id, kFzLayWarps * 32);
        if (leader) {
          issue(l, h_base, p.K[l]);
          ok = mbar_wait_bounded(mma_s, ph_mma);
        }
        ph_mma ^= 1u;
        if (group_sync_or(bar_id, kFzLayWarps * 32, !ok)) {
          failed = true;
          break;
        }
        tc_fence_after();
      }
      if (failed) break;
      // output layer accumulator -> out
      float t[16];
      tmem_ld16(row_taddr, t);
      const int64_t q = tile * kTcRows + row;
      if (q < p.n)
        for (int o = 0; o < d.out_ch && o < p.out_stride; ++o) p.out[q * p.out_stride + o] = t[o];
      // the next tile's layer-0 MMAs overwrite these columns
      tc_fence_before();
      group_sync(bar_id, kFzLayWarps * 32);
    }
  } else {
    // ---------------- encoder team t (4 * P warps)
    const int e = tid - kFzLayThreads;
    const int team = e / (kTcRows * P), et = e % (kTcRows * P);
    const int row = et % kTcRows, part = et / kTcRows;
    const int bar_id = 3 + team;
    const bool leader = et == 0;
    uint8_t* As = A0 + team * p.fz_a0;
    const int G = K0 / CK;
    const int g0 = part * G / P, g1 = (part + 1) * G / P;
    uint32_t ph_empty = 0;
    for (int64_t k = team;; k += NS) {
      const int64_t tile = blockIdx.x + k * (int64_t)gridDim.x;
      if (tile >= n_tiles) break;
      if (k >= NS) {  // wait until the layer-0 MMAs of the team's previous tile have read the stage
        const bool ok = leader ? mbar_wait_bounded(empty + team, ph_empty) : true;
        ph_empty ^= 1u;
        if (group_sync_or(bar_id, kTcRows * P, !ok)) {
          failed = true;
          break;
        }
      }
      const int64_t q = tile * kTcRows + row;
      RowPacker<PREC> pk(As, row, g0, 1.f);
      if (q < p.n) {
        enc_range<PREC>(d, p.in + q * d.in_ch, p.enc_params, g0 * CK, g1 * CK, pk);
      } else {
        for (int kk = g0 * CK; kk < g1 * CK; ++kk) pk.push(0.f);
      }
      fence_proxy_async_smem();
      group_sync(bar_id, kTcRows * P);
      if (leader) mbar_arrive(full + team);
    }
  }
  if (failed && lane_id == 0) atomicOr(p.err, 1);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, p.ncols);
}

// ------------------------------------------------------------ weight packing
__global__ void tc_scales_kernel(MlpDims d, const float* __restrict__ params, int n_layers, float* __restrict__ scales) {
  // block l < n_layers: amax of layer l's weights -> 1 / (448 / amax);
  // block n_layers: amax of the encoding parameters (hash tables)
  __shared__ float red[256];
  const int l = blockIdx.x;
  int64_t begin, count;
  if (l < n_layers) {
    const int fan_in = l == 0 ? d.in_pad : d.width;
    const int fan_out = l == n_layers - 1 ? d.out_pad : d.width;
    begin = d.layer_off[l];
    count = (int64_t)fan_in * fan_out;
  } else {
    begin = d.n_net_params;
    count = d.n_enc_params;
  }
  float m = 0.f;
  for (int64_t i = threadIdx.x; i < count; i += blockDim.x) m = fmaxf(m, fabsf(params[begin + i]));
  red[threadIdx.x] = m;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (l < n_layers)
      scales[l] = red[0] > 0.f ? red[0] / kE4M3Max : 1.f;
    else
      scales[15] = red[0];
  }
}

template <int PREC>
__global__ void tc_pack_kernel(MlpDims d, const float* __restrict__ params, int layer, int N, int K,
                               int64_t boff, const float* __restrict__ scales, uint8_t* __restrict__ blob) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)N * K) return;
  const int n = (int)(i / K), k = (int)(i % K);
  const int fan_in = layer == 0 ? d.in_pad : d.width;
  const float w = k < fan_in ? params[d.layer_off[layer] + (int64_t)n * fan_in + k] : 0.f;
  if (PREC == TC_E4M3) {
    const float s = 1.f / scales[layer];
    const uint32_t v = __nv_cvt_float2_to_fp8x2(make_float2(w * s, 0.f), __NV_SATFINITE, __NV_E4M3);
    blob[boff + op_offset(N, n, k)] = (uint8_t)(v & 0xFF);
  } else if (PREC == TC_BF16) {
    __nv_bfloat16 h = __float2bfloat16_rn(w);
    *reinterpret_cast<__nv_bfloat16*>(blob + boff + op_offset(N, n, 2 * k)) = h;
  } else {
    __half h = __float2half_rn(w);
    *reinterpret_cast<__half*>(blob + boff + op_offset(N, n, 2 * k)) = h;
  }
}

// W_l^T for the backward pass: element (n = input, k = output) of layer l.
template <int PREC>
__global__ void tc_pack_t_kernel(MlpDims d, const float* __restrict__ params, int layer, int NT, int KT,
                                 int64_t boff, uint8_t* __restrict__ blob) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)NT * KT) return;
  const int n = (int)(i / KT), k = (int)(i % KT);
  const int fan_in = layer == 0 ? d.in_pad : d.width;
  const float w = n < fan_in ? params[d.layer_off[layer] + (int64_t)k * fan_in + n] : 0.f;
  if (PREC == TC_BF16)
    *reinterpret_cast<__nv_bfloat16*>(blob + boff + op_offset(NT, n, 2 * k)) = __float2bfloat16_rn(w);
  else
    *reinterpret_cast<__half*>(blob + boff + op_offset(NT, n, 2 * k)) = __float2half_rn(w);
}

// ------------------------------------------------------------------ host API
static int tc_kinst(int precision) { return precision == HM_PREC_FP8_E4M3 ? 32 : 16; }
static int round_up(int x, int m) { return (x + m - 1) / m * m; }

bool tc_supported(const MlpDims& d, int precision, std::string* why) {
  if (precision != HM_PREC_FP16 && precision != HM_PREC_BF16 && precision != HM_PREC_FP8_E4M3) {
    if (why) *why = "unknown precision";
    return false;
  }
  if (precision == HM_PREC_FP8_E4M3 && d.width < 32) {
    if (why) *why = "E4M3 needs n_neurons >= 32 (K of one MMA is 32)";
    return false;
  }
  if (d.n_hidden + 1 > 15) {
    if (why) *why = "too many layers";
    return false;
  }
  TcPack pk;
  pk.precision = precision;
  pk.elem_bytes = precision == HM_PREC_FP8_E4M3 ? 1 : 2;
  const int KI = tc_kinst(precision);
  int64_t blob = 0;
  for (int l = 0; l <= d.n_hidden; ++l) {
    const int N = l == d.n_hidden ? d.out_pad : d.width;
    const int K = round_up(l == 0 ? d.in_pad : d.width, KI);
    blob += (int64_t)N * K * pk.elem_bytes;
  }
  const int64_t a_min = (int64_t)kTcRows * std::max(KI, d.width) * pk.elem_bytes;
  if (((blob + 127) & ~127) + a_min + 1152 > kTcSmemMax) {
    if (why) *why = "weights do not fit in shared memory";
    return false;
  }
  return true;
}

int tc_pack_alloc(const MlpDims& d, int precision, TcPack* pk) {
  pk->precision = precision;
  pk->elem_bytes = precision == HM_PREC_FP8_E4M3 ? 1 : 2;
  pk->kinst = tc_kinst(precision);
  pk->n_layers = d.n_hidden + 1;
  int64_t off = 0;
  for (int l = 0; l < pk->n_layers; ++l) {
    pk->N[l] = l == d.n_hidden ? d.out_pad : d.width;
    pk->K[l] = round_up(l == 0 ? d.in_pad : d.width, pk->kinst);
    pk->boff[l] = off;
    off += (int64_t)pk->N[l] * pk->K[l] * pk->elem_bytes;
  }
  pk->bytes = off;
  cudaError_t e = cudaMalloc(&pk->blob, (size_t)off);
  if (e == cudaSuccess) e = cudaMalloc(&pk->scales, 16 * sizeof(float));
  if (e == cudaSuccess && tc_trainable(d, precision)) {
    int64_t ot = 0;
    for (int l = 0; l < pk->n_layers; ++l) {
      pk->NT[l] = pk->K[l];  // the layer's inputs
      pk->KT[l] = pk->N[l];  // the layer's outputs
      pk->boff_t[l] = ot;
      ot += (int64_t)pk->NT[l] * pk->KT[l] * 2;
    }
    pk->bytes_t = ot;
    e = cudaMalloc(&pk->blob_t, (size_t)ot);
  }
  if (e != cudaSuccess) return hm_cuda_status(e, "tensor-core weight blob");
  cudaMemset(pk->scales, 0, 16 * sizeof(float));
  return HM_OK;
}

void tc_pack_free(TcPack* pk) {
  cudaFree(pk->blob);
  cudaFree(pk->scales);
  cudaFree(pk->blob_t);
  pk->blob = nullptr;
  pk->scales = nullptr;
  pk->blob_t = nullptr;
}

int tc_pack(const MlpDims& d, const float* params, TcPack& pk, cudaStream_t st) {
  if (pk.precision == HM_PREC_FP8_E4M3) {
    tc_scales_kernel<<<pk.n_layers + 1, 256, 0, st>>>(d, params, pk.n_layers, pk.scales);
    HM_CHECK_LAUNCH("tc_scales_kernel");
  }
  for (int l = 0; l < pk.n_layers; ++l) {
    const int64_t cnt = (int64_t)pk.N[l] * pk.K[l];
    const int blocks = (int)((cnt + 255) / 256);
    if (pk.precision == HM_PREC_FP8_E4M3)
      tc_pack_kernel<TC_E4M3><<<blocks, 256, 0, st>>>(d, params, l, pk.N[l], pk.K[l], pk.boff[l], pk.scales, pk.blob);
    else if (pk.precision == HM_PREC_BF16)
      tc_pack_kernel<TC_BF16><<<blocks, 256, 0, st>>>(d, params, l, pk.N[l], pk.K[l], pk.boff[l], pk.scales, pk.blob);
    else
      tc_pack_kernel<TC_FP16><<<blocks, 256, 0, st>>>(d, params, l, pk.N[l], pk.K[l], pk.boff[l], pk.scales, pk.blob);
    HM_CHECK_LAUNCH("tc_pack_kernel");
    if (pk.blob_t) {
      const int64_t ct = (int64_t)pk.NT[l] * pk.KT[l];
      const int bt = (int)((ct + 255) / 256);
      if (pk.precision == HM_PREC_BF16)
        tc_pack_t_kernel<TC_BF16><<<bt, 256, 0, st>>>(d, params, l, pk.NT[l], pk.KT[l], pk.boff_t[l], pk.blob_t);
      else
        tc_pack_t_kernel<TC_FP16><<<bt, 256, 0, st>>>(d, params, l, pk.NT[l], pk.KT[l], pk.boff_t[l], pk.blob_t);
      HM_CHECK_LAUNCH("tc_pack_t_kernel");
    }
  }
  return HM_OK;
}

template <int PREC, int W, bool STORE = false>
static int tc_launch(const TcArgs& a, size_t smem, cudaStream_t st) {
  auto kern = mlp_tc_fwd_kernel<PREC, W, STORE>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return hm_cuda_status(e, "mlp_tc_fwd_kernel smem");
  int dev = 0, sms = 0, smem_sm = 0, smem_res = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&smem_res, cudaDevAttrReservedSharedMemoryPerBlock, dev);
  cudaFuncAttributes fa;
  cudaFuncGetAttributes(&fa, kern);
  int per_sm = smem_sm / (int)(smem + smem_res);
  per_sm = std::min(per_sm, 65536 / std::max(1, fa.numRegs * kTcThreads));
  per_sm = std::max(1, std::min(per_sm, 512 / a.ncols));  // tensor-memory columns per SM
  const int64_t tiles = (a.n + kTcRows - 1) / kTcRows;
  const int blocks = (int)std::min<int64_t>(tiles, (int64_t)sms * per_sm);
  kern<<<blocks, kTcThreads, smem, st>>>(a);
  HM_CHECK_LAUNCH("mlp_tc_fwd_kernel");
  return HM_OK;
}

static int tc_args(const MlpDims& d, const TcPack& pk, const float* enc_params, const float* in, float* out,
                   int out_stride, int64_t n, int* err_flag, TcArgs* ap, size_t* smem_out) {
  TcArgs& a = *ap;
  memset(&a, 0, sizeof(a));
  a.d = d;
  a.blob = pk.blob;
  a.blob_bytes = pk.bytes;
  for (int l = 0; l < 16; ++l) {
    a.boff[l] = l < pk.n_layers ? pk.boff[l] : 0;
    a.N[l] = l < pk.n_layers ? pk.N[l] : 0;
    a.K[l] = l < pk.n_layers ? pk.K[l] : 0;
  }
  a.n_layers = pk.n_layers;
  a.scales = pk.scales;
  a.enc_params = enc_params;
  a.in = in;
  a.out = out;
  a.out_stride = out_stride;
  a.n = n;
  a.err = err_flag;
  int ncols = 32;
  while (ncols < std::max(d.width, 16)) ncols *= 2;
  a.ncols = ncols;
  // shared memory: A tile + weights + barrier
  const int eb = pk.elem_bytes;
  const int64_t wbytes = (pk.bytes + 127) & ~(int64_t)127;
  const int64_t misc = 1152;  // barrier, tensor-memory address, E4M3 row maxima
  auto a_bytes_for = [&](int kc) { return (int64_t)kTcRows * std::max(kc, d.width) * eb; };
  auto total = [&](int kc) { return a_bytes_for(kc) + wbytes + misc; };
  // prefer a layer-0 chunk that leaves room for two CTAs per SM
  const int64_t two_per_sm = 113 * 1024;
  int kc0 = pk.K[0];
  while (total(kc0) > two_per_sm && kc0 > pk.kinst) kc0 -= pk.kinst;
  if (total(kc0) > two_per_sm) {
    kc0 = pk.K[0];
    while (total(kc0) > kTcSmemMax && kc0 > pk.kinst) kc0 -= pk.kinst;
  }
  if (total(kc0) > kTcSmemMax) return hm_set_error("mlp: tensor-core tile does not fit"), HM_EUNSUPPORTED;
  a.kc0 = kc0;
  a.a_bytes = (int)a_bytes_for(kc0);
  *smem_out = (size_t)(a.a_bytes + wbytes + misc);
  return HM_OK;
}

int64_t tc_encode_bytes(const MlpDims& d, const TcPack& pk, int64_t n) {
  const int64_t tiles = (n + kTcRows - 1) / kTcRows;
  const int64_t tile_bytes = (int64_t)kTcRows * pk.K[0] * pk.elem_bytes;
  return tiles * tile_bytes + (pk.precision == HM_PREC_FP8_E4M3 ? ((n * 4 + 255) & ~(int64_t)255) : 0);
}

// Form of the 16-bit inferences: 0 automatic (below), 1 never the
// warp-specialised kernel, 2 only it (HM_EUNSUPPORTED where it does not
// fit).  Set by hm_debug_tc_path.
static int g_tc_path = 0;

static bool has_hash_grid(const MlpDims& d) {
  for (int si = 0; si < d.n_segs; ++si)
    if (d.segs[si].type == ENC_HASHGRID) return true;
  return false;
}

// Shared memory of mlp_tc_fused_kernel (0: the network does not fit it).
static int64_t tc_fused_smem(const MlpDims& d, const TcPack& pk, TcArgs* a) {
  if (pk.precision == HM_PREC_FP8_E4M3 || (d.width != 32 && d.width != 64) || pk.N[pk.n_layers - 1] > d.width)
    return 0;
  const int64_t w = (pk.bytes + 1023) & ~(int64_t)1023;
  const int64_t a0 = (int64_t)kTcRows * pk.K[0] * 2;
  const int64_t h = (int64_t)kTcRows * d.width * 2;
  // the most stages (the fewest encoder threads per row) that fit; an even
  // count, so that each stage is read by one layer lane only and every
  // parity wait on it is for the phase after the one that lane last saw
  for (int ns : {6, 2}) {
    const int64_t total = w + ns * a0 + kFzLanes * h + kFzMisc;
    if (total > kTcSmemMax) continue;
    if (a) {
      a->fz_w = (int)w;
      a->fz_a0 = (int)a0;
      a->fz_h = (int)h;
      a->fz_stages = ns;
    }
    return total;
  }
  return 0;
}

template <int PREC, int W>
static int tc_fused_launch(const TcArgs& a, size_t smem, cudaStream_t st) {
  auto kern = mlp_tc_fused_kernel<PREC, W>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return hm_cuda_status(e, "mlp_tc_fused_kernel smem");
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t tiles = (a.n + kTcRows - 1) / kTcRows;
  const int blocks = (int)std::min<int64_t>(tiles, (int64_t)sms);
  kern<<<blocks, kFzThreads, smem, st>>>(a);
  HM_CHECK_LAUNCH("mlp_tc_fused_kernel");
  return HM_OK;
}

bool tc_wants_workspace(const MlpDims& d, const TcPack& pk) {
  if (g_tc_path == 2) return false;
  return g_tc_path == 1 || has_hash_grid(d) || tc_fused_smem(d, pk, nullptr) == 0;
}

int tc_forward(const MlpDims& d, const TcPack& pk, const float* enc_params, const float* in, float* out,
               int out_stride, int64_t n, int* err_flag, cudaStream_t st, uint8_t* work, int64_t work_bytes) {
  if (n <= 0) return HM_OK;
  TcArgs a;
  size_t smem = 0;
  if (int e = tc_args(d, pk, enc_params, in, out, out_stride, n, err_flag, &a, &smem)) return e;
  const bool have_work = work && work_bytes >= tc_encode_bytes(d, pk, n);
  // Automatic choice, from the measured times (2^18 and 2^20 queries, W 64):
  // with a workspace, the encode kernel + layer kernel where the encoding
  // holds a hash grid (its table gathers are latency-bound and want the
  // encode kernel's occupancy: 0.127 / 0.437 ms against 0.136 / 0.510), else
  // the warp-specialised kernel (Frequency / OneBlob: 0.134 / 0.494 ms
  // against 0.151 / 0.515); without one, the warp-specialised kernel
  // wherever it fits (the layer kernel encoding its own tiles: 0.17 /
  // 0.64 ms on either network).
  const bool want_fz = g_tc_path == 2 || (g_tc_path == 0 && (!have_work || !has_hash_grid(d)));
  if (want_fz) {
    const int64_t fz = tc_fused_smem(d, pk, &a);
    if (fz > 0) {
      // both lanes' accumulators
      int ncols = 32;
      while (ncols < 2 * d.width) ncols *= 2;
      a.ncols = ncols;
      if (pk.precision == HM_PREC_BF16)
        return d.width == 32 ? tc_fused_launch<TC_BF16, 32>(a, (size_t)fz, st)
                             : tc_fused_launch<TC_BF16, 64>(a, (size_t)fz, st);
      return d.width == 32 ? tc_fused_launch<TC_FP16, 32>(a, (size_t)fz, st)
                           : tc_fused_launch<TC_FP16, 64>(a, (size_t)fz, st);
    }
    if (g_tc_path == 2) return hm_set_error("mlp: the warp-specialised kernel does not fit this network"), HM_EUNSUPPORTED;
  }
  if (have_work) {
    // encode every row first (high occupancy, no tensor work), then the
    // layers with the layer-0 operand loaded by bulk copies
    const int64_t tiles = (n + kTcRows - 1) / kTcRows;
    a.tile_bytes = (int64_t)kTcRows * pk.K[0] * pk.elem_bytes;
    float* row_inv = pk.precision == HM_PREC_FP8_E4M3 ? reinterpret_cast<float*>(work + tiles * a.tile_bytes)
                                                      : nullptr;
    if (pk.precision == HM_PREC_BF16)
      tc_encode_kernel<TC_BF16><<<(unsigned)tiles, kTcRows, 0, st>>>(a, work, row_inv);
    else if (pk.precision == HM_PREC_FP16)
      tc_encode_kernel<TC_FP16><<<(unsigned)tiles, kTcRows, 0, st>>>(a, work, row_inv);
    else
      tc_encode_kernel<TC_E4M3><<<(unsigned)tiles, kTcRows, 0, st>>>(a, work, row_inv);
    HM_CHECK_LAUNCH("tc_encode_kernel");
    a.a_pre = work;
    a.row_inv_pre = row_inv;
  }
  const int W = d.width;
  switch (pk.precision) {
    case HM_PREC_BF16:
      return W == 16 ? tc_launch<TC_BF16, 16>(a, smem, st) : W == 32 ? tc_launch<TC_BF16, 32>(a, smem, st)
             : W == 64 ? tc_launch<TC_BF16, 64>(a, smem, st) : tc_launch<TC_BF16, 128>(a, smem, st);
    case HM_PREC_FP16:
      return W == 16 ? tc_launch<TC_FP16, 16>(a, smem, st) : W == 32 ? tc_launch<TC_FP16, 32>(a, smem, st)
             : W == 64 ? tc_launch<TC_FP16, 64>(a, smem, st) : tc_launch<TC_FP16, 128>(a, smem, st);
    default:
      return W == 32 ? tc_launch<TC_E4M3, 32>(a, smem, st) : W == 64 ? tc_launch<TC_E4M3, 64>(a, smem, st)
             : tc_launch<TC_E4M3, 128>(a, smem, st);
  }
}

// =================================================================== training
// E4M3 handles train with the E4M3 forward (the operands inference uses)
// and the FP16 backward (dgrad chain and weight gradients on FP16 operands:
// the activations and encoded inputs kept as FP16, W^T packed as FP16).
bool tc_trainable(const MlpDims& d, int precision) {
  return ((precision == HM_PREC_FP16 || precision == HM_PREC_BF16) && d.width >= 16) ||
         (precision == HM_PREC_FP8_E4M3 && d.width >= 32);
}

int tc_train_alloc(const MlpDims& d, int64_t cap, bool need_dx, TcTrainBufs* b) {
  tc_train_free(b);
  const int L = d.n_hidden;
  const int wz = std::max(d.width, 16);
  // encoded inputs at the widest layer-0 pitch (E4M3 pads K to 32)
  cudaError_t e = cudaMalloc(&b->x16, (size_t)cap * round_up(d.in_pad, 32) * 2);
  if (e == cudaSuccess) e = cudaMalloc(&b->h16, (size_t)L * cap * d.width * 2);
  if (e == cudaSuccess) e = cudaMalloc(&b->dz16, (size_t)(L + 1) * cap * wz * 2);
  if (e == cudaSuccess) e = cudaMalloc(&b->pred, (size_t)cap * 16 * sizeof(float));
  if (e == cudaSuccess && need_dx) e = cudaMalloc(&b->dX, (size_t)cap * d.in_pad * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&b->loss_part, 4096 * sizeof(float));
  if (e != cudaSuccess) {
    tc_train_free(b);
    return hm_cuda_status(e, "tensor-core training buffers");
  }
  b->cap = cap;
  return HM_OK;
}

void tc_train_free(TcTrainBufs* b) {
  cudaFree(b->x16);
  cudaFree(b->h16);
  cudaFree(b->dz16);
  cudaFree(b->pred);
  cudaFree(b->dX);
  cudaFree(b->loss_part);
  *b = TcTrainBufs{};
}

int tc_train_forward(const MlpDims& d, const TcPack& pk, const float* enc_params, const float* in, int64_t n,
                     const TcTrainBufs& b, int* err_flag, cudaStream_t st) {
  if (n <= 0) return HM_OK;
  TcArgs a;
  size_t smem = 0;
  if (int e = tc_args(d, pk, enc_params, in, nullptr, 16, n, err_flag, &a, &smem)) return e;
  a.x16 = b.x16;
  a.h16 = b.h16;
  a.pred = b.pred;
  const int W = d.width;
  if (pk.precision == HM_PREC_FP8_E4M3)
    return W == 32 ? tc_launch<TC_E4M3, 32, true>(a, smem, st) : W == 64 ? tc_launch<TC_E4M3, 64, true>(a, smem, st)
           : tc_launch<TC_E4M3, 128, true>(a, smem, st);
  if (pk.precision == HM_PREC_BF16)
    return W == 16 ? tc_launch<TC_BF16, 16, true>(a, smem, st) : W == 32 ? tc_launch<TC_BF16, 32, true>(a, smem, st)
           : W == 64 ? tc_launch<TC_BF16, 64, true>(a, smem, st) : tc_launch<TC_BF16, 128, true>(a, smem, st);
  return W == 16 ? tc_launch<TC_FP16, 16, true>(a, smem, st) : W == 32 ? tc_launch<TC_FP16, 32, true>(a, smem, st)
         : W == 64 ? tc_launch<TC_FP16, 64, true>(a, smem, st) : tc_launch<TC_FP16, 128, true>(a, smem, st);
}

// ---- backward: loss gradient and the dgrad chain, one 128-row tile at a time
// dZ_{L+1} = loss gradient x loss_scale (16 columns); for j = L .. 1:
// dH_j = dZ_{j+1} W_j (A = dZ_{j+1}, B = W_j^T, accumulator in tensor memory),
// dZ_j = dH_j where h_j > 0; and dX = dZ_1 W_0 when the encoding has
// parameters.  Every dZ is rounded to the operand type, kept in shared memory
// as the next A operand and written out for the weight gradients.
struct TcBwdArgs {
  MlpDims d;
  const uint8_t* blob_t;
  int64_t blob_bytes;
  int64_t boff_t[16];
  int NT[16], KT[16];
  int L;
  const uint16_t* h16;
  uint16_t* dz16;
  const float* pred;
  const float* target;
  float* dX;
  float* loss_part;
  int loss;
  float inv_total, loss_scale;
  int64_t n;
  int* err;
  int a_bytes;
  int ncols;
  int wz;  // row pitch of dz16 (max(W, 16))
};

template <int PREC, int W>
__global__ void __launch_bounds__(kTcThreads, 1) mlp_tc_bwd_kernel(const __grid_constant__ TcBwdArgs p) {
  constexpr int FMT = PREC == TC_BF16 ? 1 : 0;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* A = smem;
  uint8_t* Wt = smem + p.a_bytes;
  uint64_t* bar = reinterpret_cast<uint64_t*>(Wt + ((p.blob_bytes + 127) & ~(int64_t)127));
  uint32_t* holder = reinterpret_cast<uint32_t*>(bar + 1);
  float* red = reinterpret_cast<float*>(holder + 4);  // [256] loss partials

  const int tid = threadIdx.x, warp = tid >> 5;
  const int row = ((warp & 3) << 5) | (tid & 31);
  const int half = warp >> 2;
  const MlpDims& d = p.d;
  const int L = p.L;
  for (int64_t i = tid; i < p.blob_bytes / 16; i += kTcThreads)
    reinterpret_cast<uint4*>(Wt)[i] = __ldg(reinterpret_cast<const uint4*>(p.blob_t) + i);
  if (tid == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(holder, p.ncols);
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *holder;
  const uint32_t row_taddr = tmem + ((uint32_t)((warp & 3) * 32) << 16);
  const uint32_t a_base = smem_u32(A), w_base = smem_u32(Wt);
  const uint32_t a_lbo = 16 * kTcRows;
  uint32_t phase = 0;
  bool failed = false;
  float loss_acc = 0.f;

  auto run = [&](int j, int k_count) -> bool {  // MMAs of dH_j = dZ_{j+1} W_j
    if (tid == 0) {
      tc_fence_after();
      const uint32_t idesc = tc_idesc(kTcRows, p.NT[j], FMT);
      const uint32_t b_lbo = 16 * p.NT[j];
      const uint32_t b_base = w_base + (uint32_t)p.boff_t[j];
      for (int ks = 0; ks < k_count / 16; ++ks) {
        const uint64_t ad = tc_sdesc(a_base + (uint32_t)ks * 2 * a_lbo, a_lbo, 128);
        const uint64_t bd = tc_sdesc(b_base + (uint32_t)ks * 2 * b_lbo, b_lbo, 128);
        tc_mma<false>(tmem, ad, bd, idesc, ks > 0 ? 1u : 0u);
      }
      tc_commit(bar);
    }
    // thread 0 (which committed) polls the barrier; the others sleep in the
    // block barrier instead of spinning
    const bool ok = threadIdx.x == 0 ? mbar_wait_bounded(bar, phase) : true;
    phase ^= 1u;
    const bool bad = __syncthreads_or(!ok);
    tc_fence_after();
    return !bad;
  };

  const int64_t n_tiles = (p.n + kTcRows - 1) / kTcRows;
  for (int64_t tile = blockIdx.x; tile < n_tiles && !failed; tile += gridDim.x) {
    const int64_t q = tile * kTcRows + row;
    const bool valid = q < p.n;
    // ---- loss gradient (half 0 of each row): dZ_{L+1}, 16 columns
    if (half == 0) {
      float g[16], pr[16];
#pragma unroll
      for (int o = 0; o < 16; ++o) {
        g[o] = 0.f;
        pr[o] = valid ? p.pred[q * 16 + o] : 0.f;
      }
      if (valid) {
        float tg[16];
        for (int o = 0; o < d.out_ch; ++o) tg[o] = __ldg(p.target + q * d.out_ch + o);
        float v = 0.f;
        loss_grad(p.loss, pr, tg, d.out_ch, p.inv_total, g, &v);
        loss_acc += v;
      }
      uint32_t word[8];
#pragma unroll
      for (int w2 = 0; w2 < 8; ++w2) word[w2] = pack2<PREC>(g[2 * w2] * p.loss_scale, g[2 * w2 + 1] * p.loss_scale);
      *reinterpret_cast<uint4*>(A + op_offset(kTcRows, row, 0)) = make_uint4(word[0], word[1], word[2], word[3]);
      *reinterpret_cast<uint4*>(A + op_offset(kTcRows, row, 16)) = make_uint4(word[4], word[5], word[6], word[7]);
      if (valid) {
        uint4* dst = reinterpret_cast<uint4*>(p.dz16 + ((int64_t)L * p.n + q) * p.wz);
        dst[0] = make_uint4(word[0], word[1], word[2], word[3]);
        dst[1] = make_uint4(word[4], word[5], word[6], word[7]);
      }
    }
    fence_proxy_async_smem();
    __syncthreads();
    int kk = 16;  // K of the next MMA: columns of the dZ in A
    for (int j = L; j >= 0 && !failed; --j) {
      if (j == 0 && !p.dX) break;
      if (!run(j, kk)) {
        failed = true;
        break;
      }
      const int nt = p.NT[j];  // inputs of layer j: W (j >= 1) or K0 (j == 0)
      if (j == 0) {
        // dX (loss-scaled, FP32) for the hash-grid backward
        for (int c = half * 16; c < nt; c += 32) {
          float t[16];
          tmem_ld16(row_taddr + c, t);
          if (valid)
            for (int e = 0; e < 16 && c + e < d.in_pad; ++e) p.dX[q * d.in_pad + c + e] = t[e];
        }
      } else {
        constexpr int HW = W / 2;
        const uint16_t* hrow = p.h16 + ((int64_t)(j - 1) * p.n + (valid ? q : 0)) * W + half * HW;
#pragma unroll
        for (int c = 0; c < HW / 16; ++c) {
          float t[16];
          tmem_ld16(row_taddr + half * HW + c * 16, t);
          uint4 hv[2];
          hv[0] = valid ? __ldg(reinterpret_cast<const uint4*>(hrow + c * 16)) : make_uint4(0, 0, 0, 0);
          hv[1] = valid ? __ldg(reinterpret_cast<const uint4*>(hrow + c * 16 + 8)) : make_uint4(0, 0, 0, 0);
          const uint16_t* hs = reinterpret_cast<const uint16_t*>(hv);
          uint32_t word[8];
#pragma unroll
          for (int w2 = 0; w2 < 8; ++w2) {
            const float a0 = hs[2 * w2] != 0 && !(hs[2 * w2] & 0x8000) ? t[2 * w2] : 0.f;
            const float a1 = hs[2 * w2 + 1] != 0 && !(hs[2 * w2 + 1] & 0x8000) ? t[2 * w2 + 1] : 0.f;
            word[w2] = pack2<PREC>(a0, a1);
          }
          const int col = half * HW + c * 16;
          *reinterpret_cast<uint4*>(A + op_offset(kTcRows, row, col * 2)) =
              make_uint4(word[0], word[1], word[2], word[3]);
          *reinterpret_cast<uint4*>(A + op_offset(kTcRows, row, col * 2 + 16)) =
              make_uint4(word[4], word[5], word[6], word[7]);
          if (valid) {
            uint4* dst = reinterpret_cast<uint4*>(p.dz16 + ((int64_t)(j - 1) * p.n + q) * p.wz + col);
            dst[0] = make_uint4(word[0], word[1], word[2], word[3]);
            dst[1] = make_uint4(word[4], word[5], word[6], word[7]);
          }
        }
        kk = W;
      }
      tc_fence_before();
      fence_proxy_async_smem();
      __syncthreads();
    }
  }
  // per-CTA loss partial, fixed order
  red[tid] = loss_acc;
  __syncthreads();
  if (tid == 0) {
    float s = 0.f;
    for (int i = 0; i < kTcThreads; ++i) s += red[i];
    p.loss_part[blockIdx.x] = s;
  }
  if (failed && tid == 0) atomicOr(p.err, 1);
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, p.ncols);
}

// ---- weight gradients of one layer: dW[o][i] = sum over rows dZ[row][o] h[row][i]
// The batch is split in fixed chunks; a CTA accumulates its chunk in tensor
// memory (A = dZ^T: the layer's outputs padded to 128 rows, B = h^T, K = the
// 128 rows of a tile) and writes an FP32 partial [outputs][inputs].
struct TcWgradArgs {
  const uint16_t* dz;  // [n][dz_pitch], columns = outputs
  int dz_pitch;
  const uint16_t* h;   // [n][h_pitch], columns = inputs
  int h_pitch;
  int n_out, n_in;     // n_in: multiple of 16, <= 256
  int64_t n;
  int64_t chunk;
  float* part;         // [splits][n_out][n_in]
  int* err;
  int ncols;
};

template <int PREC>
__global__ void __launch_bounds__(kTcThreads, 1) mlp_tc_wgrad_kernel(const __grid_constant__ TcWgradArgs p) {
  constexpr int FMT = PREC == TC_BF16 ? 1 : 0;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* A = smem;                        // [128 outputs][128 rows]
  uint8_t* B = smem + kTcRows * kTcRows * 2;  // [n_in][128 rows]
  uint64_t* bar = reinterpret_cast<uint64_t*>(B + (size_t)p.n_in * kTcRows * 2);
  uint32_t* holder = reinterpret_cast<uint32_t*>(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5;
  // A rows beyond the layer's outputs stay zero
  for (int i = tid; i < kTcRows * kTcRows * 2 / 16; i += kTcThreads)
    reinterpret_cast<uint4*>(A)[i] = make_uint4(0, 0, 0, 0);
  if (tid == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(holder, p.ncols);
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *holder;
  const uint32_t a_base = smem_u32(A), b_base = smem_u32(B);
  const uint32_t a_lbo = 16 * kTcRows, b_lbo = 16 * p.n_in;
  uint32_t phase = 0;
  bool failed = false;
  const int64_t r0 = blockIdx.x * p.chunk, r1 = min(p.n, r0 + p.chunk);
  bool first = true;
  for (int64_t t0 = r0; t0 < r1 && !failed; t0 += kTcRows) {
    // transpose the tile's rows into A (dZ^T) and B (h^T): element (feature f,
    // row k) at op_offset(rows_of_operand, f, 2k)
    const int k = tid >> 1, hf = tid & 1;
    const int64_t q = t0 + k;
    const bool valid = q < r1;
    for (int f = hf; f < p.n_out; f += 2) {
      const uint16_t v = valid ? p.dz[q * p.dz_pitch + f] : (uint16_t)0;
      *reinterpret_cast<uint16_t*>(A + op_offset(kTcRows, f, 2 * k)) = v;
    }
    for (int f = hf; f < p.n_in; f += 2) {
      const uint16_t v = valid ? p.h[q * p.h_pitch + f] : (uint16_t)0;
      *reinterpret_cast<uint16_t*>(B + op_offset(p.n_in, f, 2 * k)) = v;
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const uint32_t idesc = tc_idesc(kTcRows, p.n_in, FMT);
      for (int ks = 0; ks < kTcRows / 16; ++ks) {
        const uint64_t ad = tc_sdesc(a_base + (uint32_t)ks * 2 * a_lbo, a_lbo, 128);
        const uint64_t bd = tc_sdesc(b_base + (uint32_t)ks * 2 * b_lbo, b_lbo, 128);
        tc_mma<false>(tmem, ad, bd, idesc, (!first || ks > 0) ? 1u : 0u);
      }
      tc_commit(bar);
    }
    // thread 0 (which committed) polls the barrier; the others sleep in the
    // block barrier instead of spinning
    const bool ok = threadIdx.x == 0 ? mbar_wait_bounded(bar, phase) : true;
    phase ^= 1u;
    if (__syncthreads_or(!ok)) failed = true;
    tc_fence_after();
    first = false;
  }
  // epilogue: row o of the accumulator (tensor-memory lane o) -> part
  if (!failed && !first && warp < 4) {
    const int o = tid;  // lanes 0..127 by warp quadrant
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
    float* dst = p.part + ((int64_t)blockIdx.x * p.n_out + o) * p.n_in;
    for (int c = 0; c < p.n_in; c += 16) {
      float t[16];
      tmem_ld16(taddr + c, t);
      if (o < p.n_out)
#pragma unroll
        for (int e = 0; e < 16; ++e) dst[c + e] = t[e];
    }
  } else if (!failed && first && warp < 4 && tid < p.n_out) {
    float* dst = p.part + ((int64_t)blockIdx.x * p.n_out + tid) * p.n_in;
    for (int c = 0; c < p.n_in; ++c) dst[c] = 0.f;
  }
  if (failed && tid == 0) atomicOr(p.err, 1);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, p.ncols);
}

__global__ void tc_reduce_kernel(const float* __restrict__ part, int splits, int64_t mn, float* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < mn; i += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int k = 0; k < splits; ++k) s += part[(int64_t)k * mn + i];
    out[i] = s;
  }
}

// The same for a layer whose K is padded past its fan-in (E4M3 layer 0):
// partial rows are K wide, the parameter rows fan_in wide.
__global__ void tc_reduce_pad_kernel(const float* __restrict__ part, int splits, int N, int K, int fan_in,
                                     float* __restrict__ out) {
  const int64_t mn = (int64_t)N * K;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)N * fan_in;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t src = (i / fan_in) * K + i % fan_in;
    float s = 0.f;
    for (int k = 0; k < splits; ++k) s += part[(int64_t)k * mn + src];
    out[i] = s;
  }
}

__global__ void tc_loss_reduce_kernel(const float* __restrict__ part, int nb, float* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    float s = 0.f;
    for (int i = 0; i < nb; ++i) s += part[i];
    *out = s;
  }
}

template <int PREC, int W>
static int tc_bwd_launch(const TcBwdArgs& a, size_t smem, cudaStream_t st, int* blocks_out) {
  auto kern = mlp_tc_bwd_kernel<PREC, W>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return hm_cuda_status(e, "mlp_tc_bwd_kernel smem");
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t tiles = (a.n + kTcRows - 1) / kTcRows;
  const int blocks = (int)std::min<int64_t>(std::min<int64_t>(tiles, sms), 4096);
  kern<<<blocks, kTcThreads, smem, st>>>(a);
  HM_CHECK_LAUNCH("mlp_tc_bwd_kernel");
  *blocks_out = blocks;
  return HM_OK;
}

int tc_backward(const MlpDims& d, const TcPack& pk, const TcTrainBufs& b, const float* target, int loss,
                float loss_scale, int64_t n, float* loss_out, float* grads, float** dw_part, int64_t* dw_cap,
                int* err_flag, cudaStream_t st) {
  if (n <= 0) return HM_OK;
  const int L = d.n_hidden;
  const int W = d.width;
  TcBwdArgs a;
  memset(&a, 0, sizeof(a));
  a.d = d;
  a.blob_t = pk.blob_t;
  // layer 0's transposed block (dX) is only loaded when the encoding needs it
  const bool need_dx = b.dX != nullptr;
  a.blob_bytes = need_dx ? pk.bytes_t : pk.bytes_t;
  for (int l = 0; l < 16; ++l) {
    a.boff_t[l] = l < pk.n_layers ? pk.boff_t[l] : 0;
    a.NT[l] = l < pk.n_layers ? pk.NT[l] : 0;
    a.KT[l] = l < pk.n_layers ? pk.KT[l] : 0;
  }
  a.L = L;
  a.h16 = b.h16;
  a.dz16 = b.dz16;
  a.pred = b.pred;
  a.target = target;
  a.dX = b.dX;
  a.loss_part = b.loss_part;
  a.loss = loss;
  a.inv_total = 1.f / ((float)n * (float)d.out_ch);
  a.loss_scale = loss_scale;
  a.n = n;
  a.err = err_flag;
  a.wz = std::max(W, 16);
  int ncols = 32;
  while (ncols < std::max(W, need_dx ? pk.NT[0] : 16)) ncols *= 2;
  a.ncols = ncols;
  a.a_bytes = kTcRows * std::max(W, 16) * 2;
  const size_t smem = (size_t)a.a_bytes + ((pk.bytes_t + 127) & ~(int64_t)127) + 64 + 1024 + 64;
  if (smem > (size_t)kTcSmemMax) return hm_set_error("mlp: backward tile does not fit"), HM_EUNSUPPORTED;
  int blocks = 0;
  int s = HM_OK;
  if (pk.precision == HM_PREC_BF16)
    s = W == 16 ? tc_bwd_launch<TC_BF16, 16>(a, smem, st, &blocks) : W == 32 ? tc_bwd_launch<TC_BF16, 32>(a, smem, st, &blocks)
        : W == 64 ? tc_bwd_launch<TC_BF16, 64>(a, smem, st, &blocks) : tc_bwd_launch<TC_BF16, 128>(a, smem, st, &blocks);
  else
    s = W == 16 ? tc_bwd_launch<TC_FP16, 16>(a, smem, st, &blocks) : W == 32 ? tc_bwd_launch<TC_FP16, 32>(a, smem, st, &blocks)
        : W == 64 ? tc_bwd_launch<TC_FP16, 64>(a, smem, st, &blocks) : tc_bwd_launch<TC_FP16, 128>(a, smem, st, &blocks);
  if (s) return s;
  tc_loss_reduce_kernel<<<1, 32, 0, st>>>(b.loss_part, blocks, loss_out);
  HM_CHECK_LAUNCH("tc_loss_reduce_kernel");
  // weight gradients
  const int64_t chunk = 2048;
  const int splits = (int)((n + chunk - 1) / chunk);
  int64_t need = 0;
  for (int l = 0; l <= L; ++l) need = std::max<int64_t>(need, (int64_t)splits * pk.N[l] * pk.K[l]);
  if (need > *dw_cap) {
    cudaFree(*dw_part);
    *dw_part = nullptr;
    cudaError_t e = cudaMalloc(dw_part, need * sizeof(float));
    if (e != cudaSuccess) return hm_cuda_status(e, "tensor-core dW partials");
    *dw_cap = need;
  }
  for (int l = 0; l <= L; ++l) {
    TcWgradArgs g;
    g.n_out = pk.N[l];
    g.n_in = pk.K[l];
    g.dz = b.dz16 + (int64_t)l * n * std::max(W, 16);
    g.dz_pitch = std::max(W, 16);
    g.h = l == 0 ? b.x16 : b.h16 + (int64_t)(l - 1) * n * W;
    g.h_pitch = l == 0 ? pk.K[0] : W;
    g.n = n;
    g.chunk = chunk;
    g.part = *dw_part;
    g.err = err_flag;
    int nc = 32;
    while (nc < g.n_in) nc *= 2;
    g.ncols = nc;
    const size_t sm = (size_t)kTcRows * kTcRows * 2 + (size_t)g.n_in * kTcRows * 2 + 64;
    if (pk.precision == HM_PREC_BF16) {
      cudaFuncSetAttribute(mlp_tc_wgrad_kernel<TC_BF16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      mlp_tc_wgrad_kernel<TC_BF16><<<splits, kTcThreads, sm, st>>>(g);
    } else {
      cudaFuncSetAttribute(mlp_tc_wgrad_kernel<TC_FP16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      mlp_tc_wgrad_kernel<TC_FP16><<<splits, kTcThreads, sm, st>>>(g);
    }
    HM_CHECK_LAUNCH("mlp_tc_wgrad_kernel");
    // the layer's weights are [out][in_l] with in_l = fan_in (<= K[l]); the
    // partial rows are K[l] wide, the parameters fan_in wide
    const int fan_in = l == 0 ? d.in_pad : W;
    const int64_t mn = (int64_t)pk.N[l] * pk.K[l];
    if (fan_in == pk.K[l]) {
      tc_reduce_kernel<<<256, 256, 0, st>>>(*dw_part, splits, mn, grads + d.layer_off[l]);
      HM_CHECK_LAUNCH("tc_reduce_kernel");
    } else {
      tc_reduce_pad_kernel<<<256, 256, 0, st>>>(*dw_part, splits, pk.N[l], pk.K[l], fan_in, grads + d.layer_off[l]);
      HM_CHECK_LAUNCH("tc_reduce_pad_kernel");
    }
  }
  return HM_OK;
}

// ---- the bounded wait's expiry, exercised on purpose (tests)
// One block: thread 0 sets up an mbarrier that expects one arrival, which
// never comes, and waits on it with the kernels' bounded wait, `limit`
// tries; the expiry is recorded in err and the kernel returns.  Any other
// outcome (the wait completing) is recorded as 2.
__global__ void tc_wait_expiry_kernel(uint32_t limit, int* err) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
    *err = mbar_wait_bounded(&bar, 0u, limit) ? 2 : 1;
  }
}

}  // namespace hm

extern "C" int hm_debug_tc_path(int path) {
  if (path < 0 || path > 2) return hm_set_error("hm_debug_tc_path: path out of range"), HM_EINVAL;
  hm::g_tc_path = path;
  return HM_OK;
}

extern "C" int hm_debug_wait_expiry(int tries, void* stream) {
  if (tries < 1 || tries > (1 << 20)) return hm_set_error("hm_debug_wait_expiry: tries out of range"), HM_EINVAL;
  int* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(int));
  if (e != cudaSuccess) return hm_cuda_status(e, "hm_debug_wait_expiry");
  cudaMemsetAsync(d, 0, sizeof(int), (cudaStream_t)stream);
  hm::tc_wait_expiry_kernel<<<1, 32, 0, (cudaStream_t)stream>>>((uint32_t)tries, d);
  int h = 0;
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
  cudaFree(d);
  if (e != cudaSuccess) return hm_cuda_status(e, "hm_debug_wait_expiry");
  if (h == 1) return hm_set_error("hm_debug_wait_expiry: the bounded wait expired"), HM_ETIMEOUT;
  return hm_set_error("hm_debug_wait_expiry: the wait did not expire (%d)", h), HM_EINVAL;
}
