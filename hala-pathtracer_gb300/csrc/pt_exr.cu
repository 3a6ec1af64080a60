// pt_exr.cu -- OpenEXR HDRI reader of the C ABI (host code only):
// pt_exr_read_rgb and pt_renderer_set_envmap_file, the file form of
// HalaRenderer::set_envmap(&hdri_file, rotation) (src/bin/hala-pathtracer.rs:203).
//
// The reference decodes its HDRIs with the `exr` crate (1.72.0,
// Cargo.lock:502-504) inside its renderer crate. This reader covers what
// HDRI files use: single-part scanline images; HALF, FLOAT and UINT channels;
// compression NONE, RLE, ZIPS and ZIP. Tiled, deep and multi-part files and
// the PIZ / PXR24 / B44 / DWA codecs are refused with a reason. It reads the
// same subset as the Python loader (exr.py) and gives the same floats.
//
// File layout (OpenEXR 2): magic 20000630, version word, attributes
// (name\0 type\0 int32 size, value) up to an empty name, a table of chunk
// offsets (uint64 each), then chunks: int32 first line, int32 data size,
// data. A block holds 1 line (NONE, RLE, ZIPS) or 16 lines (ZIP); within a
// block the data is stored line by line, channels in channel-list order.
// RLE and ZIP data is byte-reordered (even bytes, then odd) and delta-coded
// before compression; a chunk whose size equals the raw size is stored raw.
//
// ZIP and ZIPS chunks are zlib streams (RFC 1950) of DEFLATE data (RFC 1951);
// the inflater below is written from those two specifications.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "pt_impl.h"

namespace {

// ------------------------------------------------------------------ inflate
struct BitReader {
  const uint8_t* p;
  size_t n, pos = 0;
  uint32_t bitbuf = 0;
  int bitcnt = 0;
  bool overrun = false;
  BitReader(const uint8_t* data, size_t size) : p(data), n(size) {}
  uint32_t bits(int need) {  // LSB-first, need <= 24
    while (bitcnt < need) {
      uint32_t b = 0;
      if (pos < n) b = p[pos++];
      else overrun = true;
      bitbuf |= b << bitcnt;
      bitcnt += 8;
    }
    uint32_t v = bitbuf & ((1u << need) - 1u);
    bitbuf >>= need;
    bitcnt -= need;
    return v;
  }
  void align() {
    bitbuf = 0;
    bitcnt = 0;
  }
};

// Canonical Huffman code of RFC 1951 3.2.2: codes of each length are
// consecutive integers, shorter codes first, symbols in order within a length.
struct Huffman {
  uint16_t count[16];      // codes of each length
  uint16_t symbol[320];    // symbols ordered by (length, value)
  bool build(const uint8_t* lengths, int nsym) {
    std::memset(count, 0, sizeof(count));
    for (int s = 0; s < nsym; ++s) count[lengths[s]]++;
    count[0] = 0;
    int left = 1;  // over-subscription check
    for (int len = 1; len < 16; ++len) {
      left <<= 1;
      left -= count[len];
      if (left < 0) return false;
    }
    uint16_t offs[16];
    offs[1] = 0;
    for (int len = 1; len < 15; ++len) offs[len + 1] = offs[len] + count[len];
    for (int s = 0; s < nsym; ++s)
      if (lengths[s]) symbol[offs[lengths[s]]++] = (uint16_t)s;
    return true;
  }
  // Reads one symbol a bit at a time: the first `count[len]` codes of length
  // len start at `first`; code values are read most significant bit first.
  int decode(BitReader& br) const {
    int code = 0, first = 0, index = 0;
    for (int len = 1; len < 16; ++len) {
      code |= (int)br.bits(1);
      const int c = count[len];
      if (code - first < c) return symbol[index + (code - first)];
      index += c;
      first = (first + c) << 1;
      code <<= 1;
      if (br.overrun) return -1;
    }
    return -1;
  }
};

const uint16_t LEN_BASE[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t LEN_EXTRA[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t DIST_BASE[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t DIST_EXTRA[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6,
                                6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_codes(BitReader& br, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out, size_t limit) {
  for (;;) {
    int sym = lit.decode(br);
    if (sym < 0) return false;
    if (sym < 256) {
      if (out.size() >= limit) return false;
      out.push_back((uint8_t)sym);
    } else if (sym == 256) {
      return true;
    } else {
      sym -= 257;
      if (sym >= 29) return false;
      const size_t len = LEN_BASE[sym] + br.bits(LEN_EXTRA[sym]);
      const int ds = dist.decode(br);
      if (ds < 0 || ds >= 30) return false;
      const size_t d = DIST_BASE[ds] + br.bits(DIST_EXTRA[ds]);
      if (d > out.size() || out.size() + len > limit) return false;
      const size_t from = out.size() - d;
      for (size_t k = 0; k < len; ++k) out.push_back(out[from + k]);  // overlapping copies repeat
    }
    if (br.overrun) return false;
  }
}

struct FixedCodes {
  Huffman lit, dist;
  FixedCodes() {
    uint8_t l[288];
    for (int s = 0; s < 144; ++s) l[s] = 8;
    for (int s = 144; s < 256; ++s) l[s] = 9;
    for (int s = 256; s < 280; ++s) l[s] = 7;
    for (int s = 280; s < 288; ++s) l[s] = 8;
    lit.build(l, 288);
    uint8_t d[30];
    for (int s = 0; s < 30; ++s) d[s] = 5;
    dist.build(d, 30);
  }
};

// zlib stream -> at most `limit` bytes. False on any format error.
bool zlib_inflate(const uint8_t* data, size_t size, std::vector<uint8_t>& out, size_t limit) {
  out.clear();
  if (size < 6) return false;
  const uint8_t cmf = data[0], flg = data[1];
  if ((cmf & 0x0F) != 8 || (cmf >> 4) > 7 || ((cmf << 8) | flg) % 31 != 0 || (flg & 0x20)) return false;
  BitReader br(data + 2, size - 2);
  bool last = false;
  while (!last) {
    last = br.bits(1) != 0;
    const uint32_t type = br.bits(2);
    if (type == 0) {  // stored
      br.align();
      if (br.pos + 4 > br.n) return false;
      const uint32_t len = br.p[br.pos] | (br.p[br.pos + 1] << 8);
      const uint32_t nlen = br.p[br.pos + 2] | (br.p[br.pos + 3] << 8);
      br.pos += 4;
      if ((len ^ 0xFFFFu) != nlen || br.pos + len > br.n || out.size() + len > limit) return false;
      out.insert(out.end(), br.p + br.pos, br.p + br.pos + len);
      br.pos += len;
    } else if (type == 1) {  // fixed codes, RFC 1951 3.2.6
      static const FixedCodes fixed;  // built once (thread-safe static initialisation)
      if (!inflate_codes(br, fixed.lit, fixed.dist, out, limit)) return false;
    } else if (type == 2) {  // dynamic codes, RFC 1951 3.2.7
      const int nlen = (int)br.bits(5) + 257, ndist = (int)br.bits(5) + 1, ncode = (int)br.bits(4) + 4;
      if (nlen > 286 || ndist > 30) return false;
      static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
      uint8_t cl[19] = {0};
      for (int k = 0; k < ncode; ++k) cl[order[k]] = (uint8_t)br.bits(3);
      Huffman clh;
      if (!clh.build(cl, 19)) return false;
      uint8_t lengths[320] = {0};
      int k = 0;
      while (k < nlen + ndist) {
        int sym = clh.decode(br);
        if (sym < 0) return false;
        if (sym < 16) {
          lengths[k++] = (uint8_t)sym;
          continue;
        }
        uint8_t val = 0;
        int rep;
        if (sym == 16) {
          if (k == 0) return false;
          val = lengths[k - 1];
          rep = 3 + (int)br.bits(2);
        } else if (sym == 17) {
          rep = 3 + (int)br.bits(3);
        } else {
          rep = 11 + (int)br.bits(7);
        }
        if (k + rep > nlen + ndist) return false;
        while (rep--) lengths[k++] = val;
      }
      if (lengths[256] == 0) return false;  // no end-of-block code
      Huffman lit, dist;
      if (!lit.build(lengths, nlen) || !dist.build(lengths + nlen, ndist)) return false;
      if (!inflate_codes(br, lit, dist, out, limit)) return false;
    } else {
      return false;
    }
    if (br.overrun) return false;
  }
  // Adler-32 of the output (RFC 1950), big-endian after the deflate data
  br.align();
  if (br.pos + 4 > br.n) return false;
  uint32_t a = 1, b = 0;
  for (uint8_t c : out) {
    a = (a + c) % 65521u;
    b = (b + a) % 65521u;
  }
  const uint32_t want = ((uint32_t)br.p[br.pos] << 24) | ((uint32_t)br.p[br.pos + 1] << 16) |
                        ((uint32_t)br.p[br.pos + 2] << 8) | br.p[br.pos + 3];
  return ((b << 16) | a) == want;
}

// ------------------------------------------------------------------ OpenEXR
// IEEE binary16 -> binary32, exact (every half is a float).
float half_to_float(uint16_t h) {
  const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
  uint32_t exp = (h >> 10) & 0x1Fu, man = h & 0x3FFu;
  uint32_t bits;
  if (exp == 0x1F) {
    bits = sign | 0x7F800000u | (man << 13);  // inf / NaN
  } else if (exp != 0) {
    bits = sign | ((exp + 112u) << 23) | (man << 13);
  } else if (man == 0) {
    bits = sign;
  } else {  // subnormal: normalise
    int e = -1;
    do {
      ++e;
      man <<= 1;
    } while ((man & 0x400u) == 0);
    bits = sign | ((uint32_t)(112 - e) << 23) | ((man & 0x3FFu) << 13);
  }
  float f;
  std::memcpy(&f, &bits, 4);
  return f;
}

struct Reader {
  const std::vector<uint8_t>& b;
  size_t pos = 0;
  bool ok = true;
  explicit Reader(const std::vector<uint8_t>& buf) : b(buf) {}
  template <class T>
  T get() {
    T v{};
    if (pos + sizeof(T) > b.size()) {
      ok = false;
      return v;
    }
    std::memcpy(&v, b.data() + pos, sizeof(T));  // little-endian file, little-endian hosts (x86-64, aarch64)
    pos += sizeof(T);
    return v;
  }
  std::string cstr() {
    std::string s;
    while (pos < b.size() && b[pos]) s.push_back((char)b[pos++]);
    if (pos >= b.size()) ok = false;
    ++pos;
    return s;
  }
};

struct Channel {
  std::string name;
  int32_t type;  // 0 UINT, 1 HALF, 2 FLOAT
};

// Undoes the predictor (delta) and the even/odd byte reordering of RLE / ZIP data.
void undo_predictor_reorder(std::vector<uint8_t>& t) {
  for (size_t i = 1; i < t.size(); ++i) t[i] = (uint8_t)(t[i - 1] + t[i] - 128);
  std::vector<uint8_t> out(t.size());
  const size_t half = (t.size() + 1) / 2;
  for (size_t i = 0; i < half; ++i) out[2 * i] = t[i];
  for (size_t i = half; i < t.size(); ++i) out[2 * (i - half) + 1] = t[i];
  t.swap(out);
}

bool rle_decode(const uint8_t* d, size_t n, std::vector<uint8_t>& out, size_t expected) {
  out.clear();
  size_t i = 0;
  while (i < n) {
    const int c = (int8_t)d[i++];
    if (c < 0) {
      const size_t k = (size_t)(-c);
      if (i + k > n || out.size() + k > expected) return false;
      out.insert(out.end(), d + i, d + i + k);
      i += k;
    } else {
      if (i >= n || out.size() + (size_t)c + 1 > expected) return false;
      out.insert(out.end(), (size_t)c + 1, d[i++]);
    }
  }
  return out.size() == expected;
}

// Reads an OpenEXR file into RGB float triples (row 0 = top). A single Y
// channel is repeated into R, G and B. Returns an empty string on success.
std::string exr_read_rgb(const char* path, std::vector<float>& rgb, uint32_t& W, uint32_t& H) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return std::string("cannot open ") + path;
  std::vector<uint8_t> buf;
  uint8_t tmp[1 << 16];
  size_t got;
  while ((got = std::fread(tmp, 1, sizeof(tmp), f)) > 0) buf.insert(buf.end(), tmp, tmp + got);
  std::fclose(f);
  Reader rd(buf);
  if (rd.get<int32_t>() != 20000630) return "not an OpenEXR file";
  const uint32_t version = rd.get<uint32_t>();
  if (version & 0x200u) return "tiled OpenEXR files are not supported";
  if (version & 0x1800u) return "deep or multi-part OpenEXR files are not supported";
  std::vector<Channel> chans;
  int comp = -1;
  int32_t win[4] = {0, 0, -1, -1};
  bool have_win = false;
  for (;;) {
    if (rd.pos >= buf.size()) return "truncated header";
    if (buf[rd.pos] == 0) {
      ++rd.pos;
      break;
    }
    const std::string name = rd.cstr(), type = rd.cstr();
    const int32_t size = rd.get<int32_t>();
    if (!rd.ok || size < 0 || rd.pos + (size_t)size > buf.size()) return "truncated header";
    const size_t vend = rd.pos + (size_t)size;
    if (name == "channels") {
      while (rd.pos < vend && buf[rd.pos] != 0) {
        Channel c;
        c.name = rd.cstr();
        c.type = rd.get<int32_t>();
        rd.pos += 4;  // pLinear + reserved
        const int32_t xs = rd.get<int32_t>(), ys = rd.get<int32_t>();
        if (xs != 1 || ys != 1) return "channel " + c.name + " is subsampled";
        if (c.type < 0 || c.type > 2) return "unknown pixel type";
        chans.push_back(c);
      }
    } else if (name == "compression") {
      comp = buf[rd.pos];
    } else if (name == "dataWindow") {
      for (int k = 0; k < 4; ++k) win[k] = rd.get<int32_t>();
      have_win = true;
    }
    rd.pos = vend;
  }
  if (chans.empty() || comp < 0 || !have_win) return "header lacks channels, compression or dataWindow";
  if (comp > 3) return "compression " + std::to_string(comp) + " is not supported (NONE, RLE, ZIPS, ZIP are)";
  const int64_t w64 = (int64_t)win[2] - win[0] + 1, h64 = (int64_t)win[3] - win[1] + 1;
  if (w64 <= 0 || h64 <= 0 || w64 * h64 > (1ll << 28)) return "empty or oversized data window";
  W = (uint32_t)w64;
  H = (uint32_t)h64;
  // the channels that make RGB: by the last component of the name
  auto suffix = [](const std::string& n) {
    size_t d = n.rfind('.');
    return d == std::string::npos ? n : n.substr(d + 1);
  };
  int idx[3] = {-1, -1, -1}, yi = -1;
  for (size_t c = 0; c < chans.size(); ++c) {
    const std::string s = suffix(chans[c].name);
    if (s == "R") idx[0] = (int)c;
    else if (s == "G") idx[1] = (int)c;
    else if (s == "B") idx[2] = (int)c;
    else if (s == "Y") yi = (int)c;
  }
  if (idx[0] < 0 || idx[1] < 0 || idx[2] < 0) {
    if (yi < 0) return "no RGB or Y channels";
    idx[0] = idx[1] = idx[2] = yi;
  }
  const int lpb = comp == 3 ? 16 : 1;
  const size_t nblocks = (H + lpb - 1) / lpb;
  std::vector<uint64_t> offsets(nblocks);
  for (size_t k = 0; k < nblocks; ++k) offsets[k] = rd.get<uint64_t>();
  if (!rd.ok) return "truncated offset table";
  size_t px_bytes = 0;
  for (const Channel& c : chans) px_bytes += c.type == 1 ? 2 : 4;
  const size_t row_bytes = px_bytes * W;
  rgb.assign((size_t)W * H * 3, 0.0f);
  std::vector<uint8_t> raw;
  std::vector<uint32_t> seen(H, 0);
  for (uint64_t off : offsets) {
    if (off + 8 > buf.size()) return "chunk offset outside the file";
    int32_t y, size;
    std::memcpy(&y, buf.data() + off, 4);
    std::memcpy(&size, buf.data() + off + 4, 4);
    if (size < 0 || off + 8 + (uint64_t)size > buf.size()) return "truncated chunk";
    const int64_t y0 = (int64_t)y - win[1];
    if (y0 < 0 || y0 >= (int64_t)H) return "chunk outside the data window";
    const uint32_t lines = (uint32_t)std::min<int64_t>(lpb, (int64_t)H - y0);
    const size_t raw_size = row_bytes * lines;
    const uint8_t* data = buf.data() + off + 8;
    if ((size_t)size == raw_size || comp == 0) {
      if ((size_t)size != raw_size) return "corrupt block size";
      raw.assign(data, data + size);
    } else if (comp == 1) {
      if (!rle_decode(data, (size_t)size, raw, raw_size)) return "corrupt RLE block";
      undo_predictor_reorder(raw);
    } else {
      if (!zlib_inflate(data, (size_t)size, raw, raw_size) || raw.size() != raw_size) return "corrupt ZIP block";
      undo_predictor_reorder(raw);
    }
    size_t p = 0;
    for (uint32_t ly = 0; ly < lines; ++ly) {
      const size_t row = (size_t)(y0 + ly);
      seen[row] = 1;
      for (size_t c = 0; c < chans.size(); ++c) {
        const int t = chans[c].type;
        const size_t bpp = t == 1 ? 2 : 4;
        for (int k = 0; k < 3; ++k) {
          if (idx[k] != (int)c) continue;
          float* dst = rgb.data() + row * W * 3 + k;
          const uint8_t* src = raw.data() + p;
          for (uint32_t x = 0; x < W; ++x) {
            float v;
            if (t == 1) {
              uint16_t h;
              std::memcpy(&h, src + 2 * x, 2);
              v = half_to_float(h);
            } else if (t == 2) {
              std::memcpy(&v, src + 4 * x, 4);
            } else {
              uint32_t u;
              std::memcpy(&u, src + 4 * x, 4);
              v = (float)u;
            }
            dst[3 * (size_t)x] = v;
          }
        }
        p += bpp * W;
      }
    }
  }
  for (uint32_t y = 0; y < H; ++y)
    if (!seen[y]) return "a line of the data window has no chunk";
  return std::string();
}

void put_error(char* msg, size_t cap, const std::string& s) {
  if (msg && cap) std::snprintf(msg, cap, "%s", s.c_str());
}

}  // namespace

namespace hpt {
bool inflate_zlib(const uint8_t* data, size_t size, std::vector<uint8_t>& out, size_t limit) {
  return zlib_inflate(data, size, out, limit);
}
}  // namespace hpt

extern "C" {

pt_status pt_exr_read_rgb(const char* path, float* rgb, size_t capacity_floats, uint32_t* width, uint32_t* height,
                          char* error_message, size_t error_capacity) try {
  if (error_message && error_capacity) error_message[0] = '\0';
  if (!path || !width || !height) {
    put_error(error_message, error_capacity, "path, width and height must not be null");
    return PT_ERR_INVALID_ARG;
  }
  std::vector<float> px;
  uint32_t W = 0, H = 0;
  const std::string why = exr_read_rgb(path, px, W, H);
  if (!why.empty()) {
    put_error(error_message, error_capacity, why);
    return PT_ERR_INVALID_ARG;
  }
  *width = W;
  *height = H;
  if (!rgb) return PT_OK;  // size query
  if (capacity_floats < px.size()) {
    put_error(error_message, error_capacity, "the output holds fewer than width * height * 3 floats");
    return PT_ERR_INVALID_ARG;
  }
  std::memcpy(rgb, px.data(), px.size() * sizeof(float));
  return PT_OK;
} catch (...) {
  std::string why;
  const pt_status st = host_exception_status(&why);
  put_error(error_message, error_capacity, why);
  return st;
}

pt_status pt_renderer_set_envmap_file(pt_renderer* r, const char* path, float rotation_degrees) try {
  if (!r) return PT_ERR_INVALID_ARG;
  std::vector<float> px;
  uint32_t W = 0, H = 0;
  if (!path) return pt_renderer_set_envmap(r, nullptr, 0, 0, rotation_degrees);
  const std::string why = exr_read_rgb(path, px, W, H);
  if (!why.empty()) {
    r->err = "HDRI " + std::string(path) + ": " + why;
    return PT_ERR_INVALID_ARG;
  }
  return pt_renderer_set_envmap(r, px.data(), W, H, rotation_degrees);
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}

}  // extern "C"
