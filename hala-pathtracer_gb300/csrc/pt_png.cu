// pt_png.cu -- PNG decoding for the C ABI (host code only): material
// textures of glTF scenes (pt_gltf.cu), pt_png_read_rgba8, and
// pt_renderer_load_blue_noise_texture, the file form of
// HalaRenderer::load_blue_noise_texture (src/bin/hala-pathtracer.rs:195).
//
// Non-interlaced PNGs (ISO/IEC 15948) of every colour type (grey, RGB,
// palette, grey + alpha, RGBA) at bit depths 1-16 with the five scanline
// filters; image data through the EXR reader's zlib inflater. The float form
// is the Python loader's (png.py): samples / (2^depth - 1), palette entries
// / 255, missing alpha 1. The RGBA8 form is for 8-bit images, as an RGBA8
// UNORM texture holds them.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "pt_impl.h"

namespace {

const uint8_t PNG_SIG[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};

uint32_t be32(const uint8_t* p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }

// Unfiltered scanlines and what is needed to read samples from them.
struct Decoded {
  uint32_t w = 0, h = 0;
  int depth = 0, ctype = 0, nch = 0;
  size_t stride = 0;
  std::vector<uint8_t> rows, plte, trns;
  bool have_trns = false;

  uint32_t sample(uint32_t y, uint32_t x, int ch) const {
    const uint8_t* r = &rows[y * stride];
    if (depth == 16) {
      const size_t o = ((size_t)x * nch + ch) * 2;
      return (uint32_t)r[o] << 8 | r[o + 1];
    }
    if (depth == 8) return r[(size_t)x * nch + ch];
    const size_t bit = ((size_t)x * nch + ch) * depth;  // MSB first
    return (r[bit >> 3] >> (8 - depth - (bit & 7))) & ((1u << depth) - 1u);
  }
};

std::string decode(const uint8_t* buf, size_t size, Decoded& d) {
  if (size < 8 || std::memcmp(buf, PNG_SIG, 8) != 0) return "not a PNG file";
  size_t pos = 8;
  std::vector<uint8_t> idat;
  bool have_hdr = false;
  int interlace = 0;
  while (pos < size) {
    if (pos + 8 > size) return "truncated chunk";
    const uint32_t n = be32(buf + pos);
    const uint8_t* typ = buf + pos + 4;
    if ((size_t)n > size - pos - 8) return "truncated chunk";
    const uint8_t* data = buf + pos + 8;
    pos += 12 + (size_t)n;
    if (!std::memcmp(typ, "IHDR", 4)) {
      if (n < 13) return "short IHDR";
      d.w = be32(data);
      d.h = be32(data + 4);
      d.depth = data[8];
      d.ctype = data[9];
      interlace = data[12];
      have_hdr = true;
    } else if (!std::memcmp(typ, "PLTE", 4)) {
      d.plte.assign(data, data + n);
    } else if (!std::memcmp(typ, "tRNS", 4)) {
      d.trns.assign(data, data + n);
      d.have_trns = true;
    } else if (!std::memcmp(typ, "IDAT", 4)) {
      idat.insert(idat.end(), data, data + n);
    } else if (!std::memcmp(typ, "IEND", 4)) {
      break;
    }
  }
  if (!have_hdr) return "missing IHDR";
  if (interlace) return "interlaced PNGs are not supported";
  switch (d.ctype) {
    case 0: d.nch = 1; break;
    case 2: d.nch = 3; break;
    case 3: d.nch = 1; break;
    case 4: d.nch = 2; break;
    case 6: d.nch = 4; break;
    default: return "unknown colour type " + std::to_string(d.ctype);
  }
  if (!(d.depth == 1 || d.depth == 2 || d.depth == 4 || d.depth == 8 || d.depth == 16)) return "bad bit depth";
  if (d.w == 0 || d.h == 0 || (uint64_t)d.w * d.h > (1ull << 26)) return "image size 0 or above 2^26 pixels";
  if (d.ctype == 3 && d.plte.size() < 3) return "palette image without PLTE";
  const int bits = d.depth * d.nch;
  d.stride = ((size_t)d.w * bits + 7) / 8;
  const size_t bpp = std::max(1, bits / 8);
  std::vector<uint8_t> raw;
  const size_t want = (d.stride + 1) * d.h;
  if (!hpt::inflate_zlib(idat.data(), idat.size(), raw, 2 * want + 65536) || raw.size() < want)
    return "corrupt image data";
  d.rows.assign(d.stride * d.h, 0);
  std::vector<uint8_t> prev(d.stride, 0);
  for (uint32_t y = 0; y < d.h; ++y) {
    const uint8_t f = raw[y * (d.stride + 1)];
    const uint8_t* in = &raw[y * (d.stride + 1) + 1];
    uint8_t* r = &d.rows[y * d.stride];
    for (size_t i = 0; i < d.stride; ++i) {
      const int a = i >= bpp ? r[i - bpp] : 0, b = prev[i], c = i >= bpp ? prev[i - bpp] : 0;
      int pred;
      switch (f) {
        case 0: pred = 0; break;
        case 1: pred = a; break;
        case 2: pred = b; break;
        case 3: pred = (a + b) >> 1; break;
        case 4: {
          const int pp = a + b - c, pa = std::abs(pp - a), pb = std::abs(pp - b), pc = std::abs(pp - c);
          pred = (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
          break;
        }
        default: return "unknown filter type " + std::to_string(f);
      }
      r[i] = (uint8_t)(in[i] + pred);
    }
    std::memcpy(prev.data(), r, d.stride);
  }
  if (d.ctype == 3) {
    const size_t npal = d.plte.size() / 3;
    for (uint32_t y = 0; y < d.h; ++y)
      for (uint32_t x = 0; x < d.w; ++x)
        if (d.sample(y, x, 0) >= npal) return "palette index out of range";
  }
  return "";
}

std::vector<uint8_t> read_file(const char* path, std::string& why) {
  std::vector<uint8_t> out;
  FILE* f = std::fopen(path, "rb");
  if (!f) {
    why = "cannot open the file";
    return out;
  }
  uint8_t buf[1 << 16];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) out.insert(out.end(), buf, buf + n);
  std::fclose(f);
  return out;
}

void put_error(char* msg, size_t cap, const std::string& s) {
  if (!msg || !cap) return;
  const size_t n = std::min(cap - 1, s.size());
  std::memcpy(msg, s.data(), n);
  msg[n] = '\0';
}

}  // namespace

namespace hpt {

std::string png_decode_float(const uint8_t* data, size_t size, uint32_t& w, uint32_t& h, std::vector<float>& rgba) {
  Decoded d;
  const std::string why = decode(data, size, d);
  if (!why.empty()) return why;
  w = d.w;
  h = d.h;
  const float maxv = d.depth == 16 ? 65535.0f : d.depth == 8 ? 255.0f : (float)((1 << d.depth) - 1);
  auto sample = [&](uint32_t y, uint32_t x, int ch) {
    const uint32_t v = d.sample(y, x, ch);
    return d.ctype == 3 ? (float)v : (float)v / maxv;
  };
  rgba.assign((size_t)d.w * d.h * 4, 0.0f);
  for (uint32_t y = 0; y < d.h; ++y)
    for (uint32_t x = 0; x < d.w; ++x) {
      float* o = &rgba[((size_t)y * d.w + x) * 4];
      if (d.ctype == 3) {
        const size_t i = d.sample(y, x, 0);
        for (int k = 0; k < 3; ++k) o[k] = (float)d.plte[3 * i + k] / 255.0f;
        o[3] = (float)((d.have_trns && i < d.trns.size()) ? d.trns[i] : 255) / 255.0f;
      } else if (d.nch == 1) {
        o[0] = o[1] = o[2] = sample(y, x, 0);
        o[3] = 1.0f;
      } else if (d.nch == 2) {
        o[0] = o[1] = o[2] = sample(y, x, 0);
        o[3] = sample(y, x, 1);
      } else {
        for (int k = 0; k < d.nch; ++k) o[k] = sample(y, x, k);
        if (d.nch == 3) o[3] = 1.0f;
      }
    }
  return "";
}

std::string png_decode_rgba8(const uint8_t* data, size_t size, uint32_t& w, uint32_t& h, std::vector<uint8_t>& rgba) {
  Decoded d;
  const std::string why = decode(data, size, d);
  if (!why.empty()) return why;
  if (d.ctype != 3 && d.depth != 8) return "an 8-bit image is needed (this one has " + std::to_string(d.depth) +
                                           "-bit samples)";
  w = d.w;
  h = d.h;
  rgba.assign((size_t)d.w * d.h * 4, 0);
  for (uint32_t y = 0; y < d.h; ++y)
    for (uint32_t x = 0; x < d.w; ++x) {
      uint8_t* o = &rgba[((size_t)y * d.w + x) * 4];
      if (d.ctype == 3) {
        const size_t i = d.sample(y, x, 0);
        for (int k = 0; k < 3; ++k) o[k] = d.plte[3 * i + k];
        o[3] = (d.have_trns && i < d.trns.size()) ? d.trns[i] : 255;
      } else if (d.nch == 1) {
        o[0] = o[1] = o[2] = (uint8_t)d.sample(y, x, 0);
        o[3] = 255;
      } else if (d.nch == 2) {
        o[0] = o[1] = o[2] = (uint8_t)d.sample(y, x, 0);
        o[3] = (uint8_t)d.sample(y, x, 1);
      } else {
        for (int k = 0; k < d.nch; ++k) o[k] = (uint8_t)d.sample(y, x, k);
        if (d.nch == 3) o[3] = 255;
      }
    }
  return "";
}

}  // namespace hpt

extern "C" {

pt_status pt_png_read_rgba8(const char* path, uint8_t* rgba, size_t capacity_bytes, uint32_t* width,
                            uint32_t* height, char* error_message, size_t error_capacity) try {
  put_error(error_message, error_capacity, "");
  if (!path || !width || !height) {
    put_error(error_message, error_capacity, "path, width and height must not be null");
    return PT_ERR_INVALID_ARG;
  }
  std::string why;
  const std::vector<uint8_t> bytes = read_file(path, why);
  uint32_t W = 0, H = 0;
  std::vector<uint8_t> px;
  if (why.empty()) why = hpt::png_decode_rgba8(bytes.data(), bytes.size(), W, H, px);
  if (!why.empty()) {
    put_error(error_message, error_capacity, std::string("PNG ") + path + ": " + why);
    return PT_ERR_INVALID_ARG;
  }
  *width = W;
  *height = H;
  if (!rgba) return PT_OK;  // size query
  if (capacity_bytes < px.size()) {
    put_error(error_message, error_capacity, "the output holds fewer than width * height * 4 bytes");
    return PT_ERR_INVALID_ARG;
  }
  std::memcpy(rgba, px.data(), px.size());
  return PT_OK;
} catch (...) {
  std::string why;
  const pt_status st = host_exception_status(&why);
  put_error(error_message, error_capacity, why);
  return st;
}

pt_status pt_renderer_load_blue_noise_texture(pt_renderer* r, const char* path) try {
  if (!r) return PT_ERR_INVALID_ARG;
  if (!path) return pt_renderer_set_blue_noise(r, nullptr);
  std::string why;
  const std::vector<uint8_t> bytes = read_file(path, why);
  uint32_t W = 0, H = 0;
  std::vector<uint8_t> px;
  if (why.empty()) why = hpt::png_decode_rgba8(bytes.data(), bytes.size(), W, H, px);
  if (why.empty() && (W < PT_BLUE_NOISE_SIZE || H < PT_BLUE_NOISE_SIZE))
    why = "the texture is " + std::to_string(W) + " x " + std::to_string(H) + ", smaller than " +
          std::to_string(PT_BLUE_NOISE_SIZE) + " x " + std::to_string(PT_BLUE_NOISE_SIZE);
  if (!why.empty()) {
    r->err = std::string("blue-noise texture ") + path + ": " + why;
    return PT_ERR_INVALID_ARG;
  }
  // the texels the shader can fetch: the top-left 1024 x 1024
  std::vector<uint8_t> tex((size_t)PT_BLUE_NOISE_SIZE * PT_BLUE_NOISE_SIZE * 4);
  for (uint32_t y = 0; y < PT_BLUE_NOISE_SIZE; ++y)
    std::memcpy(&tex[(size_t)y * PT_BLUE_NOISE_SIZE * 4], &px[(size_t)y * W * 4], (size_t)PT_BLUE_NOISE_SIZE * 4);
  return pt_renderer_set_blue_noise(r, tex.data());
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}

}  // extern "C"
