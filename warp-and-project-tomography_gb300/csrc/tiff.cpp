// TIFF projection stacks (the reference's input through CImg's libtiff
// loader: WaP_Tomo.h:7-8 enables it, CImg.h:47445-47500 load_tiff and
// 47562-47700 _load_tiff).  CImg reads every directory (page) of the file as
// one z slice and stores each sample value cast to float, with no scaling
// and no photometric inversion; grey images (one sample per pixel) are the
// projection-stack case.  This reader covers baseline TIFF and the common
// extensions: little- and big-endian files, strips or tiles, 8/16/32/64-bit
// unsigned, signed or IEEE samples, no compression, PackBits, LZW and
// Deflate (Deflate through the system's zlib, opened at run time), with the
// horizontal-differencing predictor.  Every offset and length read from the
// file is checked against its size; a malformed or unsupported file is
// WAP_EIO with no partial output.  Pages are at most kMaxSide pixels a side
// and a stack at most kMaxSamples samples (WAP_ETOOBIG beyond), so a header
// cannot ask for an unbounded allocation; a failed host allocation is
// WAP_ENOMEM (WAP_CATCH).
#include <dlfcn.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "c_boundary.h"
#include "wap/wap_io.h"

namespace {

constexpr uint32_t kMaxSide = 1u << 20;       // pixels per page side
constexpr uint64_t kMaxSamples = 1ull << 33;  // samples per stack (32 GB as float)

struct Ifd {
  uint32_t w = 0, h = 0, bps = 1, spp = 1, fmt = 1, comp = 1, planar = 1, pred = 1, rps = 0xffffffffu, tw = 0,
           th = 0;
  bool tiled = false;
  std::vector<uint64_t> offs, counts;
};

struct File {
  std::vector<uint8_t> b;
  bool le = true;
  bool ok(uint64_t off, uint64_t len) const { return off <= b.size() && len <= b.size() - off; }
  uint32_t u16(uint64_t o) const {
    return le ? (uint32_t)b[o] | (uint32_t)b[o + 1] << 8 : (uint32_t)b[o] << 8 | (uint32_t)b[o + 1];
  }
  uint32_t u32(uint64_t o) const {
    return le ? (uint32_t)b[o] | (uint32_t)b[o + 1] << 8 | (uint32_t)b[o + 2] << 16 | (uint32_t)b[o + 3] << 24
              : (uint32_t)b[o] << 24 | (uint32_t)b[o + 1] << 16 | (uint32_t)b[o + 2] << 8 | (uint32_t)b[o + 3];
  }
};

bool read_file(const char *path, std::vector<uint8_t> &out) {
  FILE *f = std::fopen(path, "rb");
  if (!f) return false;
  const bool seek = std::fseek(f, 0, SEEK_END) == 0;
  const long n = seek ? std::ftell(f) : -1;
  bool good = n >= 8 && std::fseek(f, 0, SEEK_SET) == 0;
  if (good) {
    out.resize((size_t)n);
    good = std::fread(out.data(), 1, (size_t)n, f) == (size_t)n;
  }
  std::fclose(f);
  return good;
}

// Values of an entry of type SHORT or LONG (count n), inline or at an offset.
bool entry_values(const File &F, uint64_t e, std::vector<uint64_t> &v) {
  const uint32_t type = F.u16(e + 2), n = F.u32(e + 4);
  const uint32_t sz = type == 3 ? 2 : type == 4 ? 4 : 0;
  if (!sz || n == 0 || n > (1u << 26)) return false;
  uint64_t at = e + 8;
  if ((uint64_t)n * sz > 4) {
    at = F.u32(e + 8);
    if (!F.ok(at, (uint64_t)n * sz)) return false;
  }
  v.resize(n);
  for (uint32_t i = 0; i < n; ++i) v[i] = sz == 2 ? F.u16(at + 2 * i) : F.u32(at + 4 * i);
  return true;
}

bool parse(const File &F, std::vector<Ifd> &ifds) {
  uint64_t off = F.u32(4);
  while (off != 0) {
    if (ifds.size() > 100000 || !F.ok(off, 2)) return false;
    const uint32_t n = F.u16(off);
    if (!F.ok(off + 2, (uint64_t)n * 12 + 4)) return false;
    Ifd d;
    for (uint32_t i = 0; i < n; ++i) {
      const uint64_t e = off + 2 + 12 * (uint64_t)i;
      const uint32_t tag = F.u16(e);
      std::vector<uint64_t> v;
      switch (tag) {
        case 256: case 257: case 258: case 259: case 262: case 277: case 278: case 284: case 317: case 322:
        case 323: case 339:
          if (!entry_values(F, e, v)) return false;
          break;
        case 273: case 279: case 324: case 325:
          if (!entry_values(F, e, v)) return false;
          break;
        default:
          continue;
      }
      const uint32_t x = (uint32_t)v[0];
      switch (tag) {
        case 256: d.w = x; break;
        case 257: d.h = x; break;
        case 258: d.bps = x; break;
        case 259: d.comp = x; break;
        case 277: d.spp = x; break;
        case 278: d.rps = x; break;
        case 284: d.planar = x; break;
        case 317: d.pred = x; break;
        case 322: d.tw = x; d.tiled = true; break;
        case 323: d.th = x; d.tiled = true; break;
        case 339: d.fmt = x; break;
        case 273: case 324: d.offs = v; break;
        case 279: case 325: d.counts = v; break;
        default: break;
      }
    }
    ifds.push_back(d);
    off = F.u32(off + 2 + 12 * (uint64_t)n);
  }
  return !ifds.empty();
}

bool unpackbits(const uint8_t *s, size_t n, std::vector<uint8_t> &out, size_t want) {
  out.clear();
  size_t i = 0;
  while (i < n && out.size() < want) {
    const int c = (int8_t)s[i++];
    if (c >= 0) {
      if (i + c + 1 > n) return false;
      out.insert(out.end(), s + i, s + i + c + 1);
      i += c + 1;
    } else if (c != -128) {
      if (i >= n) return false;
      out.insert(out.end(), (size_t)(1 - c), s[i++]);
    }
  }
  return out.size() >= want;
}

// TIFF LZW: MSB-first codes of 9..12 bits, 256 = clear, 257 = end; the code
// width grows when the next free entry reaches 2^bits - 1 (the decoder sits
// one entry behind the encoder, which switches at 2^bits).
bool unlzw(const uint8_t *s, size_t n, std::vector<uint8_t> &out, size_t want) {
  out.clear();
  std::vector<uint16_t> prefix(4096);
  std::vector<uint8_t> suffix(4096), first(4096);
  std::vector<uint16_t> len(4096);
  for (int c = 0; c < 256; ++c) {
    prefix[c] = 0xffff;
    suffix[c] = first[c] = (uint8_t)c;
    len[c] = 1;
  }
  int nbits = 9, next = 258, prev = -1;
  uint64_t bitpos = 0;
  std::vector<uint8_t> tmp;
  auto emit = [&](int code) {
    const size_t L = len[code], at = out.size();
    out.resize(at + L);
    for (size_t k = L; k-- > 0;) {
      out[at + k] = suffix[code];
      code = prefix[code];
    }
  };
  while (out.size() < want) {
    if (bitpos + nbits > (uint64_t)n * 8) break;
    int code = 0;
    for (int k = 0; k < nbits; ++k, ++bitpos) code = code << 1 | ((s[bitpos >> 3] >> (7 - (bitpos & 7))) & 1);
    if (code == 257) break;
    if (code == 256) {
      nbits = 9;
      next = 258;
      prev = -1;
      continue;
    }
    if (prev < 0) {
      if (code > 255) return false;
      emit(code);
      prev = code;
      continue;
    }
    if (code > next || next >= 4096) return false;
    const uint8_t head = code < next ? first[code] : first[prev];
    prefix[next] = (uint16_t)prev;
    suffix[next] = head;
    first[next] = first[prev];
    len[next] = (uint16_t)(len[prev] + 1);
    if (len[next] == 0) return false;
    ++next;
    emit(code);
    prev = code;
    if (next >= (1 << nbits) - 1 && nbits < 12) ++nbits;
  }
  return out.size() >= want;
}

// zlib's uncompress, opened at run time (no link-time dependency).
bool inflate_zlib(const uint8_t *s, size_t n, std::vector<uint8_t> &out, size_t want) {
  typedef int (*uncompress_fn)(unsigned char *, unsigned long *, const unsigned char *, unsigned long);
  static uncompress_fn fn = [] {
    void *h = dlopen("libz.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!h) h = dlopen("libz.so", RTLD_NOW | RTLD_LOCAL);
    return h ? (uncompress_fn)dlsym(h, "uncompress") : (uncompress_fn) nullptr;
  }();
  if (!fn) return false;
  out.assign(want, 0);
  unsigned long got = (unsigned long)want;
  const int rc = fn(out.data(), &got, s, (unsigned long)n);
  return (rc == 0 || rc == -5 /* Z_BUF_ERROR: a strip may carry padding */) && got >= want;
}

// One page into h_out (w*h floats).
bool load_page(const File &F, const Ifd &d, float *h_out, std::string &why) {
  const uint32_t bytes = d.bps / 8;
  if (d.spp != 1 || (d.bps != 8 && d.bps != 16 && d.bps != 32 && d.bps != 64) ||
      !(d.fmt == 1 || d.fmt == 2 || d.fmt == 3) || (d.fmt == 3 && d.bps < 32)) {
    why = "unsupported sample layout (one sample per pixel of 8/16/32/64 bits is read)";
    return false;
  }
  if (d.pred != 1 && !(d.pred == 2 && d.fmt != 3)) {
    why = "unsupported predictor";
    return false;
  }
  const uint32_t bw = d.tiled ? d.tw : d.w, bh = d.tiled ? d.th : (d.rps < d.h ? d.rps : d.h);
  if (bw == 0 || bh == 0 || (d.tiled && (d.tw % 16 || d.th % 16))) {
    why = "bad strip or tile size";
    return false;
  }
  const uint32_t across = (d.w + bw - 1) / bw, down = (d.h + bh - 1) / bh;
  if (d.offs.size() < (size_t)across * down || d.counts.size() < d.offs.size()) {
    why = "missing strip or tile offsets";
    return false;
  }
  const size_t blk = (size_t)bw * bh * bytes;
  std::vector<uint8_t> raw;
  for (uint32_t by = 0; by < down; ++by)
    for (uint32_t bx = 0; bx < across; ++bx) {
      const size_t q = (size_t)by * across + bx;
      const uint64_t off = d.offs[q], cnt = d.counts[q];
      // rows of this block that hold pixels (a last strip may be short)
      const uint32_t rows = d.tiled ? bh : std::min<uint32_t>(bh, d.h - by * bh);
      const size_t need = (size_t)bw * rows * bytes;
      if (!F.ok(off, cnt)) {
        why = "strip or tile outside the file";
        return false;
      }
      const uint8_t *src = F.b.data() + off;
      bool good = true;
      if (d.comp == 1) {
        good = cnt >= need;
        if (good) raw.assign(src, src + need);
      } else if (d.comp == 32773) {
        good = unpackbits(src, cnt, raw, need);
      } else if (d.comp == 5) {
        good = unlzw(src, cnt, raw, need);
      } else if (d.comp == 8 || d.comp == 32946) {
        good = inflate_zlib(src, cnt, raw, need);
      } else {
        why = "unsupported compression " + std::to_string(d.comp);
        return false;
      }
      if (!good) {
        why = "corrupt or truncated strip or tile";
        return false;
      }
      (void)blk;
      if (d.pred == 2) {  // horizontal differencing, per row, in sample units of the file's byte order
        for (uint32_t r = 0; r < rows; ++r) {
          uint8_t *row = raw.data() + (size_t)r * bw * bytes;
          for (uint32_t c = 1; c < bw; ++c) {
            if (bytes == 1) {
              row[c] = (uint8_t)(row[c] + row[c - 1]);
            } else {
              uint64_t a = 0, p = 0;
              for (uint32_t k = 0; k < bytes; ++k) {
                const uint32_t sh = F.le ? 8 * k : 8 * (bytes - 1 - k);
                a |= (uint64_t)row[c * bytes + k] << sh;
                p |= (uint64_t)row[(c - 1) * bytes + k] << sh;
              }
              a += p;
              for (uint32_t k = 0; k < bytes; ++k)
                row[c * bytes + k] = (uint8_t)(a >> (F.le ? 8 * k : 8 * (bytes - 1 - k)));
            }
          }
        }
      }
      for (uint32_t r = 0; r < rows; ++r) {
        const uint32_t y = by * bh + r;
        if (y >= d.h) break;
        for (uint32_t c = 0; c < bw; ++c) {
          const uint32_t x = bx * bw + c;
          if (x >= d.w) break;
          const uint8_t *p = raw.data() + ((size_t)r * bw + c) * bytes;
          uint64_t u = 0;
          for (uint32_t k = 0; k < bytes; ++k) u |= (uint64_t)p[k] << (F.le ? 8 * k : 8 * (bytes - 1 - k));
          float v;
          if (d.fmt == 3) {
            if (bytes == 4) {
              uint32_t u32 = (uint32_t)u;
              float f;
              std::memcpy(&f, &u32, 4);
              v = f;
            } else {
              double g;
              std::memcpy(&g, &u, 8);
              v = (float)g;
            }
          } else if (d.fmt == 2) {
            const int64_t sv = bytes == 8 ? (int64_t)u : (int64_t)(u << (64 - 8 * bytes)) >> (64 - 8 * bytes);
            v = (float)sv;
          } else {
            v = (float)u;
          }
          h_out[(size_t)y * d.w + x] = v;
        }
      }
    }
  return true;
}

int open_tiff(const char *path, File &F, std::vector<Ifd> &ifds) {
  if (!path || !read_file(path, F.b)) return WAP_EIO;
  if (F.b[0] == 'I' && F.b[1] == 'I') F.le = true;
  else if (F.b[0] == 'M' && F.b[1] == 'M') F.le = false;
  else return WAP_EIO;
  if (F.u16(2) != 42) return WAP_EIO;  // classic TIFF (BigTIFF is 43)
  if (!parse(F, ifds)) return WAP_EIO;
  const Ifd &d0 = ifds[0];
  for (const Ifd &d : ifds)
    if (d.w != d0.w || d.h != d0.h || d.w == 0 || d.h == 0) return WAP_EIO;
  if (d0.w > kMaxSide || d0.h > kMaxSide || (uint64_t)d0.w * d0.h * ifds.size() > kMaxSamples) return WAP_ETOOBIG;
  return WAP_OK;
}

}  // namespace

extern "C" int wap_tiff_info(const char *path, int *dims4, int *bits, int *sample_format) try {
  File F;
  std::vector<Ifd> ifds;
  const int rc = open_tiff(path, F, ifds);
  if (rc != WAP_OK) return rc;
  if (dims4) {
    dims4[0] = (int)ifds[0].w;
    dims4[1] = (int)ifds[0].h;
    dims4[2] = (int)ifds.size();
    dims4[3] = (int)ifds[0].spp;
  }
  if (bits) *bits = (int)ifds[0].bps;
  if (sample_format) *sample_format = (int)ifds[0].fmt;
  return WAP_OK;
} WAP_CATCH

extern "C" int wap_tiff_load(const char *path, float *h_out, size_t count) try {
  File F;
  std::vector<Ifd> ifds;
  const int rc = open_tiff(path, F, ifds);
  if (rc != WAP_OK) return rc;
  const size_t page = (size_t)ifds[0].w * ifds[0].h;
  if (!h_out || count < page * ifds.size()) return WAP_EINVAL;
  std::vector<float> tmp(page * ifds.size());
  std::string why;
  for (size_t z = 0; z < ifds.size(); ++z)
    if (!load_page(F, ifds[z], tmp.data() + z * page, why)) return WAP_EIO;
  std::memcpy(h_out, tmp.data(), tmp.size() * sizeof(float));
  return WAP_OK;
} WAP_CATCH
