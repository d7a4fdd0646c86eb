// OpenEXR reader for environment maps (host code).
//
// The reference loads its maps with tinyexr's LoadEXR (model.cpp:158-181):
// a single-part image as RGBA float rows, first stored scanline first; a
// missing A reads 1, a luminance-only (Y) image is copied to R, G, B.  This
// is a reader of my own for the format's published layout: magic and
// version, the attribute header (channels, compression, dataWindow), the
// scanline offset table, and chunks of (y, size, data) with the channels of
// each line stored one after another in name order.  Pixel types HALF,
// FLOAT and UINT; compressions NONE, RLE, ZIPS and ZIP (zlib streams,
// decoded by the inflate below, then the format's byte predictor and
// even/odd de-interleave).  PIZ, PXR24, B44 and DWA, tiled and multi-part
// files are refused with a message.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "hm_common.cuh"
#include "hm_exr.h"

namespace hm {
namespace {

// ---------------------------------------------------------------- inflate
// RFC 1950 (zlib wrapper) / RFC 1951 (deflate) decoder.
struct BitReader {
  const uint8_t* p;
  size_t n, pos = 0;
  uint32_t bitbuf = 0;
  int bitcnt = 0;
  bool overrun = false;
  int need(int k) {
    while (bitcnt < k) {
      uint32_t b = 0;
      if (pos < n) b = p[pos++];
      else overrun = true;
      bitbuf |= b << bitcnt;
      bitcnt += 8;
    }
    return 0;
  }
  uint32_t bits(int k) {
    if (k == 0) return 0;
    need(k);
    const uint32_t v = bitbuf & ((1u << k) - 1u);
    bitbuf >>= k;
    bitcnt -= k;
    return v;
  }
  void align() {
    bitbuf = 0;
    bitcnt = 0;
  }
};

// Canonical Huffman decoding table: counts per length and symbols in order.
struct Huffman {
  uint16_t count[16];
  uint16_t symbol[320];
  bool build(const uint8_t* lengths, int n) {
    memset(count, 0, sizeof(count));
    for (int i = 0; i < n; ++i) count[lengths[i]]++;
    count[0] = 0;
    int left = 1;
    for (int len = 1; len < 16; ++len) {
      left <<= 1;
      left -= count[len];
      if (left < 0) return false;  // over-subscribed
    }
    uint16_t offs[16];
    offs[1] = 0;
    for (int len = 1; len < 15; ++len) offs[len + 1] = offs[len] + count[len];
    for (int i = 0; i < n; ++i)
      if (lengths[i]) symbol[offs[lengths[i]]++] = (uint16_t)i;
    return true;
  }
  int decode(BitReader& br) const {
    int code = 0, first = 0, index = 0;
    for (int len = 1; len < 16; ++len) {
      code |= (int)br.bits(1);
      const int c = count[len];
      if (code - c < first) return symbol[index + (code - first)];
      index += c;
      first += c;
      first <<= 1;
      code <<= 1;
    }
    return -1;
  }
};

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                               35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193,
                                257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_block(BitReader& br, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out, size_t cap) {
  for (;;) {
    const int sym = lit.decode(br);
    if (sym < 0 || br.overrun) return false;
    if (sym < 256) {
      if (out.size() >= cap) return false;
      out.push_back((uint8_t)sym);
    } else if (sym == 256) {
      return true;
    } else {
      const int li = sym - 257;
      if (li >= 29) return false;
      const size_t len = kLenBase[li] + br.bits(kLenExtra[li]);
      const int ds = dist.decode(br);
      if (ds < 0 || ds >= 30) return false;
      const size_t d = kDistBase[ds] + br.bits(kDistExtra[ds]);
      if (d > out.size() || out.size() + len > cap) return false;
      const size_t from = out.size() - d;
      for (size_t k = 0; k < len; ++k) out.push_back(out[from + k]);
    }
  }
}

// zlib stream -> bytes (at most cap); false on any malformed input.
bool zlib_decompress(const uint8_t* src, size_t n, size_t cap, std::vector<uint8_t>& out) {
  out.clear();
  if (n < 2) return false;
  const uint8_t cmf = src[0], flg = src[1];
  if ((cmf & 15) != 8 || ((cmf << 8) | flg) % 31 != 0 || (flg & 32)) return false;
  BitReader br{src + 2, n - 2};
  for (int guard = 0; guard < (1 << 24); ++guard) {
    const uint32_t final = br.bits(1);
    const uint32_t type = br.bits(2);
    if (type == 0) {
      br.align();
      if (br.pos + 4 > br.n) return false;
      const uint32_t len = br.p[br.pos] | (br.p[br.pos + 1] << 8);
      const uint32_t nlen = br.p[br.pos + 2] | (br.p[br.pos + 3] << 8);
      br.pos += 4;
      if ((len ^ 0xffffu) != nlen || br.pos + len > br.n || out.size() + len > cap) return false;
      out.insert(out.end(), br.p + br.pos, br.p + br.pos + len);
      br.pos += len;
    } else if (type == 1) {
      uint8_t l[288], d[30];
      for (int i = 0; i < 144; ++i) l[i] = 8;
      for (int i = 144; i < 256; ++i) l[i] = 9;
      for (int i = 256; i < 280; ++i) l[i] = 7;
      for (int i = 280; i < 288; ++i) l[i] = 8;
      for (int i = 0; i < 30; ++i) d[i] = 5;
      Huffman lit, dist;
      lit.build(l, 288);
      dist.build(d, 30);
      if (!inflate_block(br, lit, dist, out, cap)) return false;
    } else if (type == 2) {
      const int hlit = (int)br.bits(5) + 257, hdist = (int)br.bits(5) + 1, hclen = (int)br.bits(4) + 4;
      static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
      uint8_t cl[19] = {0};
      for (int i = 0; i < hclen; ++i) cl[order[i]] = (uint8_t)br.bits(3);
      Huffman clh;
      if (!clh.build(cl, 19)) return false;
      uint8_t lens[320] = {0};
      int i = 0;
      while (i < hlit + hdist) {
        const int sym = clh.decode(br);
        if (sym < 0 || br.overrun) return false;
        if (sym < 16) {
          lens[i++] = (uint8_t)sym;
        } else {
          int rep = 0;
          uint8_t val = 0;
          if (sym == 16) {
            if (i == 0) return false;
            val = lens[i - 1];
            rep = 3 + (int)br.bits(2);
          } else if (sym == 17) {
            rep = 3 + (int)br.bits(3);
          } else {
            rep = 11 + (int)br.bits(7);
          }
          if (i + rep > hlit + hdist) return false;
          while (rep--) lens[i++] = val;
        }
      }
      Huffman lit, dist;
      if (!lit.build(lens, hlit) || !dist.build(lens + hlit, hdist)) return false;
      if (!inflate_block(br, lit, dist, out, cap)) return false;
    } else {
      return false;
    }
    if (br.overrun) return false;
    if (final) return true;
  }
  return false;
}

// ---------------------------------------------------------------- EXR
float half_to_float(uint16_t h) {
  const uint32_t s = (uint32_t)(h >> 15) << 31;
  const int e = (h >> 10) & 31;
  const uint32_t m = h & 1023;
  uint32_t bits;
  if (e == 0) {
    if (m == 0) {
      bits = s;
    } else {  // subnormal: m * 2^-24
      const float f = (float)m * 5.9604644775390625e-8f;
      memcpy(&bits, &f, 4);
      bits |= s;
    }
  } else if (e == 31) {
    bits = s | 0x7f800000u | (m << 13);
  } else {
    bits = s | ((uint32_t)(e - 15 + 127) << 23) | (m << 13);
  }
  float f;
  memcpy(&f, &bits, 4);
  return f;
}

struct Channel {
  std::string name;
  int type;  // 0 uint, 1 half, 2 float
  int xs, ys;
};

// The format's reordering for RLE / ZIP(S): a byte predictor, then the
// first half of the bytes holds the even positions and the second the odd.
void undo_predictor_interleave(std::vector<uint8_t>& b) {
  for (size_t i = 1; i < b.size(); ++i) b[i] = (uint8_t)(b[i - 1] + b[i] - 128);
  std::vector<uint8_t> t(b.size());
  const size_t half = (b.size() + 1) / 2;
  for (size_t i = 0; i < b.size(); ++i) t[i] = (i & 1) ? b[half + i / 2] : b[i / 2];
  b.swap(t);
}

bool rle_decompress(const uint8_t* src, size_t n, size_t cap, std::vector<uint8_t>& out) {
  out.clear();
  size_t i = 0;
  while (i < n) {
    const int c = (int8_t)src[i++];
    if (c < 0) {
      const size_t k = (size_t)(-c);
      if (i + k > n || out.size() + k > cap) return false;
      out.insert(out.end(), src + i, src + i + k);
      i += k;
    } else {
      if (i >= n || out.size() + (size_t)c + 1 > cap) return false;
      out.insert(out.end(), (size_t)c + 1, src[i++]);
    }
  }
  return true;
}

}  // namespace

int exr_load_rgba(const std::string& data, std::vector<float4>* rgba, int* width, int* height, std::string* err) {
  auto fail = [&](const std::string& m) {
    *err = m;
    return HM_EPARSE;
  };
  const uint8_t* p = (const uint8_t*)data.data();
  const size_t n = data.size();
  if (n < 8 || p[0] != 0x76 || p[1] != 0x2f || p[2] != 0x31 || p[3] != 0x01) return fail("not an OpenEXR file");
  const uint32_t ver = p[4] | (p[5] << 8) | (p[6] << 16) | ((uint32_t)p[7] << 24);
  if ((ver & 0xff) != 2) return fail("unsupported OpenEXR version");
  if (ver & 0x200) {
    *err = "tiled OpenEXR images are not supported";
    return HM_EUNSUPPORTED;
  }
  if (ver & 0x1800) {
    *err = "multi-part / deep OpenEXR images are not supported";
    return HM_EUNSUPPORTED;
  }
  size_t pos = 8;
  auto rd_str = [&](std::string* s) {
    const size_t start = pos;
    while (pos < n && p[pos] != 0) ++pos;
    if (pos >= n) return false;
    s->assign((const char*)p + start, pos - start);
    ++pos;
    return true;
  };
  auto rd_i32 = [&](size_t at) {
    int32_t v;
    memcpy(&v, p + at, 4);
    return v;
  };
  std::vector<Channel> ch;
  int compression = -1;
  int32_t dw[4] = {0, 0, -1, -1};
  for (;;) {
    if (pos >= n) return fail("truncated OpenEXR header");
    if (p[pos] == 0) {
      ++pos;
      break;
    }
    std::string name, type;
    if (!rd_str(&name) || !rd_str(&type) || pos + 4 > n) return fail("truncated OpenEXR header");
    const int32_t size = rd_i32(pos);
    pos += 4;
    if (size < 0 || pos + (size_t)size > n) return fail("bad OpenEXR attribute size");
    const size_t end = pos + size;
    if (name == "channels" && type == "chlist") {
      size_t q = pos;
      while (q < end && p[q] != 0) {
        Channel c;
        const size_t s0 = q;
        while (q < end && p[q] != 0) ++q;
        if (q + 17 > end) return fail("bad OpenEXR channel list");
        c.name.assign((const char*)p + s0, q - s0);
        ++q;
        c.type = rd_i32(q);
        c.xs = rd_i32(q + 8);
        c.ys = rd_i32(q + 12);
        q += 16;
        if (c.type < 0 || c.type > 2) return fail("bad OpenEXR pixel type");
        if (c.xs != 1 || c.ys != 1) {
          *err = "sub-sampled OpenEXR channels are not supported";
          return HM_EUNSUPPORTED;
        }
        ch.push_back(c);
      }
    } else if (name == "compression" && type == "compression" && size >= 1) {
      compression = p[pos];
    } else if (name == "dataWindow" && type == "box2i" && size >= 16) {
      for (int k = 0; k < 4; ++k) dw[k] = rd_i32(pos + 4 * k);
    }
    pos = end;
  }
  if (ch.empty()) return fail("OpenEXR file without channels");
  const int64_t w = (int64_t)dw[2] - dw[0] + 1, h = (int64_t)dw[3] - dw[1] + 1;
  if (w <= 0 || h <= 0 || w > 16384 || h > 16384) return fail("bad OpenEXR data window");
  int lines = 1;
  switch (compression) {
    case 0: case 1: case 2: lines = 1; break;
    case 3: lines = 16; break;
    default:
      *err = "OpenEXR compression " + std::to_string(compression) + " is not supported (NONE, RLE, ZIPS, ZIP are)";
      return HM_EUNSUPPORTED;
  }
  int64_t line_bytes = 0;
  for (const Channel& c : ch) line_bytes += w * (c.type == 1 ? 2 : 4);
  const int64_t chunks = (h + lines - 1) / lines;
  if (pos + 8 * (size_t)chunks > n) return fail("truncated OpenEXR offset table");
  std::vector<uint64_t> offs(chunks);
  memcpy(offs.data(), p + pos, 8 * chunks);
  // channel index of R, G, B, A (or Y)
  int iR = -1, iG = -1, iB = -1, iA = -1, iY = -1;
  for (size_t k = 0; k < ch.size(); ++k) {
    const std::string& nm = ch[k].name;
    if (nm == "R") iR = (int)k;
    if (nm == "G") iG = (int)k;
    if (nm == "B") iB = (int)k;
    if (nm == "A") iA = (int)k;
    if (nm == "Y") iY = (int)k;
  }
  if ((iR < 0 || iG < 0 || iB < 0) && iY < 0) return fail("OpenEXR image has neither R, G, B nor Y channels");
  rgba->assign((size_t)w * h, make_float4(0.f, 0.f, 0.f, 1.f));
  std::vector<uint8_t> buf;
  for (int64_t c = 0; c < chunks; ++c) {
    const uint64_t o = offs[c];
    if (o + 8 > n) return fail("bad OpenEXR chunk offset");
    const int32_t y0 = rd_i32(o), sz = rd_i32(o + 4);
    if (sz < 0 || o + 8 + (uint64_t)sz > n) return fail("bad OpenEXR chunk size");
    const int64_t row0 = (int64_t)y0 - dw[1];
    if (row0 < 0 || row0 >= h) return fail("bad OpenEXR chunk line");
    const int64_t nl = std::min<int64_t>(lines, h - row0);
    const size_t raw = (size_t)(nl * line_bytes);
    const uint8_t* src = p + o + 8;
    if ((size_t)sz == raw || compression == 0) {  // stored (also when compression did not pay)
      if ((size_t)sz < raw) return fail("short OpenEXR chunk");
      buf.assign(src, src + raw);
    } else if (compression == 1) {
      if (!rle_decompress(src, sz, raw, buf) || buf.size() != raw) return fail("bad OpenEXR RLE chunk");
      undo_predictor_interleave(buf);
    } else {
      if (!zlib_decompress(src, sz, raw, buf) || buf.size() != raw) return fail("bad OpenEXR ZIP chunk");
      undo_predictor_interleave(buf);
    }
    size_t q = 0;
    for (int64_t l = 0; l < nl; ++l) {
      float4* row = rgba->data() + (size_t)(row0 + l) * w;
      for (size_t k = 0; k < ch.size(); ++k) {
        const int t = ch[k].type;
        for (int64_t x = 0; x < w; ++x) {
          float v;
          if (t == 1) {
            uint16_t hv;
            memcpy(&hv, buf.data() + q, 2);
            v = half_to_float(hv);
            q += 2;
          } else if (t == 2) {
            memcpy(&v, buf.data() + q, 4);
            q += 4;
          } else {
            uint32_t u;
            memcpy(&u, buf.data() + q, 4);
            v = (float)u;
            q += 4;
          }
          float4& px = row[x];
          const int ki = (int)k;
          if (ki == iR) px.x = v;
          if (ki == iG) px.y = v;
          if (ki == iB) px.z = v;
          if (ki == iA) px.w = v;
          if (ki == iY && iR < 0) px.x = px.y = px.z = v;
        }
      }
    }
  }
  *width = (int)w;
  *height = (int)h;
  return HM_OK;
}

}  // namespace hm
