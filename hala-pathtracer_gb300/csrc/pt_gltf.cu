// pt_gltf.cu -- glTF 2.0 scene reader of the C ABI (host code only):
// pt_gltf_load and pt_renderer_set_scene_file, the file form of
// HalaScene::new(scene_file) + HalaRenderer::set_scene
// (src/bin/hala-pathtracer.rs:97-99, :198).
//
// The reference reads its scenes with the `gltf` crate (1.4.1) inside its
// renderer crate, which is not part of its checkout, so the mapping from a
// glTF document to pt_scene_desc is this library's own; it is the mapping of
// the Python loader (hala-pathtracer_gb300/gltf.py), restated here so that a
// host without Python (the reference's Rust binary) can load a scene:
//
//   geometry   every TRIANGLES primitive of every mesh node of the default
//              scene, in node order (pre-order walk from the scene's roots);
//              POSITION, NORMAL (area-weighted smooth normals when absent),
//              TANGENT xyz (an orthogonal tangent when absent), TEXCOORD_0
//              (zeros when absent); the node's world matrix is the
//              primitive transform;
//   materials  pbrMetallicRoughness factors, emissiveFactor times
//              KHR_materials_emissive_strength, KHR_materials_ior,
//              KHR_materials_transmission, KHR_materials_clearcoat, alpha
//              (BLEND: opacity = base alpha; MASK: 0/1 against alphaCutoff);
//              `extras` override any pt_material field by name, "type"
//              ("diffuse" | "lambert" | "disney" or 0 | 1) selects the model
//              (default: Disney when metallic, transmissive or clear-coated),
//              "medium" {type absorb | scatter | emissive, color, density,
//              anisotropy} attaches a medium;
//   textures   PNG images (file, data URI or buffer view), baked as factor x
//              texel because the shaders replace the material value with the
//              texel (pathtracer.rgen.glsl:121-133); colour and emission maps
//              go from sRGB to linear; other image formats are skipped;
//   lights     KHR_lights_punctual point / spot / directional, intensity =
//              colour x intensity (or an "rgb" extra); extras {type 1, param0
//              w, param1 h} make a w x h rectangle facing the node's -Z and
//              {type 2, param0 r} a sphere of radius r, with the radiance of a
//              Lambertian emitter of the light's power;
//   cameras    perspective (yfov; extras aperture, focal_distance) and
//              orthographic (xmag, ymag), looking along the node's -Z.
//
// The arithmetic follows the Python loader step for step (double precision
// where it computes in float64, float where it computes in float32), so both
// give the same scene arrays.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "pt_impl.h"

struct pt_gltf_scene {
  std::vector<std::vector<float>> verts;
  std::vector<std::vector<uint32_t>> indices;
  std::vector<std::vector<float>> texels;
  std::vector<pt_primitive> prims;
  std::vector<pt_material> mats;
  std::vector<pt_light> lights;
  std::vector<pt_camera> cams;
  std::vector<pt_texture> texs;
  uint32_t skipped_images = 0;
  pt_scene_desc desc{};
};

namespace {

struct LoadError {
  std::string msg;
};
[[noreturn]] void raise(const std::string& m) { throw LoadError{m}; }

// ------------------------------------------------------------------ JSON (RFC 8259)
struct Json {
  enum Kind { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
  bool b = false;
  double num = 0.0;
  bool integer = false;  // the number was written without fraction or exponent
  std::string str;
  std::vector<Json> arr;
  std::vector<std::pair<std::string, Json>> obj;

  // A later duplicate key replaces an earlier one, as in Python's json.
  const Json* get(const char* key) const {
    if (kind != OBJ) return nullptr;
    for (size_t i = obj.size(); i-- > 0;)
      if (obj[i].first == key) return &obj[i].second;
    return nullptr;
  }
  bool truthy() const {
    switch (kind) {
      case NUL: return false;
      case BOOL: return b;
      case NUM: return num != 0.0;
      case STR: return !str.empty();
      case ARR: return !arr.empty();
      default: return !obj.empty();
    }
  }
};

class JsonParser {
 public:
  JsonParser(const char* p, size_t n) : p_(p), end_(p + n) {}
  Json parse() {
    Json v = value(0);
    ws();
    if (p_ != end_) raise("JSON: extra data after the document");
    return v;
  }

 private:
  const char* p_;
  const char* end_;

  void ws() {
    while (p_ < end_ && (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r')) ++p_;
  }
  bool lit(const char* s) {
    size_t n = std::strlen(s);
    if ((size_t)(end_ - p_) >= n && std::memcmp(p_, s, n) == 0) {
      p_ += n;
      return true;
    }
    return false;
  }
  static void utf8(std::string& out, uint32_t c) {
    if (c < 0x80) {
      out += (char)c;
    } else if (c < 0x800) {
      out += (char)(0xC0 | (c >> 6));
      out += (char)(0x80 | (c & 0x3F));
    } else if (c < 0x10000) {
      out += (char)(0xE0 | (c >> 12));
      out += (char)(0x80 | ((c >> 6) & 0x3F));
      out += (char)(0x80 | (c & 0x3F));
    } else {
      out += (char)(0xF0 | (c >> 18));
      out += (char)(0x80 | ((c >> 12) & 0x3F));
      out += (char)(0x80 | ((c >> 6) & 0x3F));
      out += (char)(0x80 | (c & 0x3F));
    }
  }
  uint32_t hex4() {
    if (end_ - p_ < 4) raise("JSON: truncated \\u escape");
    uint32_t v = 0;
    for (int k = 0; k < 4; ++k) {
      const char c = *p_++;
      v <<= 4;
      if (c >= '0' && c <= '9') v |= (uint32_t)(c - '0');
      else if (c >= 'a' && c <= 'f') v |= (uint32_t)(c - 'a' + 10);
      else if (c >= 'A' && c <= 'F') v |= (uint32_t)(c - 'A' + 10);
      else raise("JSON: bad \\u escape");
    }
    return v;
  }
  std::string string() {
    ++p_;  // opening quote
    std::string out;
    for (;;) {
      if (p_ >= end_) raise("JSON: unterminated string");
      const char c = *p_++;
      if (c == '"') return out;
      if ((unsigned char)c < 0x20) raise("JSON: control character in a string");
      if (c != '\\') {
        out += c;
        continue;
      }
      if (p_ >= end_) raise("JSON: unterminated escape");
      const char e = *p_++;
      switch (e) {
        case '"': out += '"'; break;
        case '\\': out += '\\'; break;
        case '/': out += '/'; break;
        case 'b': out += '\b'; break;
        case 'f': out += '\f'; break;
        case 'n': out += '\n'; break;
        case 'r': out += '\r'; break;
        case 't': out += '\t'; break;
        case 'u': {
          uint32_t cp = hex4();
          if (cp >= 0xD800 && cp < 0xDC00 && end_ - p_ >= 6 && p_[0] == '\\' && p_[1] == 'u') {
            const char* save = p_;
            p_ += 2;
            const uint32_t lo = hex4();
            if (lo >= 0xDC00 && lo < 0xE000) cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
            else p_ = save;
          }
          utf8(out, cp);
          break;
        }
        default: raise("JSON: bad escape");
      }
    }
  }
  Json number() {
    const char* s = p_;
    bool integer = true;
    if (p_ < end_ && *p_ == '-') ++p_;
    if (p_ >= end_ || !(*p_ >= '0' && *p_ <= '9')) raise("JSON: bad number");
    while (p_ < end_ && *p_ >= '0' && *p_ <= '9') ++p_;
    if (p_ < end_ && *p_ == '.') {
      integer = false;
      ++p_;
      while (p_ < end_ && *p_ >= '0' && *p_ <= '9') ++p_;
    }
    if (p_ < end_ && (*p_ == 'e' || *p_ == 'E')) {
      integer = false;
      ++p_;
      if (p_ < end_ && (*p_ == '+' || *p_ == '-')) ++p_;
      while (p_ < end_ && *p_ >= '0' && *p_ <= '9') ++p_;
    }
    Json v;
    v.kind = Json::NUM;
    v.integer = integer;
    v.num = std::strtod(std::string(s, p_).c_str(), nullptr);  // correctly rounded
    return v;
  }
  Json value(int depth) {
    if (depth > 256) raise("JSON: nesting too deep");
    ws();
    if (p_ >= end_) raise("JSON: unexpected end");
    Json v;
    const char c = *p_;
    if (c == '{') {
      ++p_;
      v.kind = Json::OBJ;
      ws();
      if (p_ < end_ && *p_ == '}') {
        ++p_;
        return v;
      }
      for (;;) {
        ws();
        if (p_ >= end_ || *p_ != '"') raise("JSON: expected a key");
        std::string k = string();
        ws();
        if (p_ >= end_ || *p_ != ':') raise("JSON: expected ':'");
        ++p_;
        v.obj.emplace_back(std::move(k), value(depth + 1));
        ws();
        if (p_ < end_ && *p_ == ',') {
          ++p_;
          continue;
        }
        if (p_ < end_ && *p_ == '}') {
          ++p_;
          return v;
        }
        raise("JSON: expected ',' or '}'");
      }
    }
    if (c == '[') {
      ++p_;
      v.kind = Json::ARR;
      ws();
      if (p_ < end_ && *p_ == ']') {
        ++p_;
        return v;
      }
      for (;;) {
        v.arr.push_back(value(depth + 1));
        ws();
        if (p_ < end_ && *p_ == ',') {
          ++p_;
          continue;
        }
        if (p_ < end_ && *p_ == ']') {
          ++p_;
          return v;
        }
        raise("JSON: expected ',' or ']'");
      }
    }
    if (c == '"') {
      v.kind = Json::STR;
      v.str = string();
      return v;
    }
    if (lit("true")) {
      v.kind = Json::BOOL;
      v.b = true;
      return v;
    }
    if (lit("false")) {
      v.kind = Json::BOOL;
      return v;
    }
    if (lit("null")) return v;
    // Python's json also takes these three
    v.kind = Json::NUM;
    if (lit("NaN")) {
      v.num = NAN;
      return v;
    }
    if (lit("Infinity")) {
      v.num = INFINITY;
      return v;
    }
    if (lit("-Infinity")) {
      v.num = -INFINITY;
      return v;
    }
    return number();
  }
};

// Value accessors with the Python loader's conversions: float(x) of a number
// or a boolean, int(x) of an integer, a numeric string or a float.
double as_f(const Json* j, double dflt, const char* what) {
  if (!j) return dflt;
  if (j->kind == Json::NUM) return j->num;
  if (j->kind == Json::BOOL) return j->b ? 1.0 : 0.0;
  if (j->kind == Json::STR) {
    char* e = nullptr;
    const double v = std::strtod(j->str.c_str(), &e);
    if (e && *e == '\0' && !j->str.empty()) return v;
  }
  raise(std::string("expected a number for ") + what);
}
long long as_i(const Json* j, long long dflt, const char* what) {
  if (!j) return dflt;
  if (j->kind == Json::NUM && std::isfinite(j->num)) return (long long)j->num;  // int() truncates
  if (j->kind == Json::BOOL) return j->b ? 1 : 0;
  if (j->kind == Json::STR) {
    char* e = nullptr;
    const long long v = std::strtoll(j->str.c_str(), &e, 10);
    if (e && *e == '\0' && !j->str.empty()) return v;
  }
  raise(std::string("expected an integer for ") + what);
}
const Json& at(const Json& arr, long long i, const char* what) {
  if (arr.kind != Json::ARR || i < 0 || (size_t)i >= arr.arr.size()) raise(std::string("bad index into ") + what);
  return arr.arr[(size_t)i];
}
const Json& need(const Json& o, const char* key) {
  const Json* j = o.get(key);
  if (!j) raise(std::string("missing \"") + key + "\"");
  return *j;
}
// str(x).isdigit() of a JSON value: a non-negative integer literal or a
// string of digits
bool digit_text(const Json& j, long long& v) {
  if (j.kind == Json::NUM && j.integer && j.num >= 0.0) {
    v = (long long)j.num;
    return true;
  }
  if (j.kind == Json::STR && !j.str.empty()) {
    for (char c : j.str)
      if (c < '0' || c > '9') return false;
    v = std::strtoll(j.str.c_str(), nullptr, 10);
    return true;
  }
  return false;
}
std::string lower_text(const Json& j) {
  std::string s;
  if (j.kind == Json::STR) s = j.str;
  for (char& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}
// a list of numbers (at least n of them; the first n are used)
void floats(const Json* j, size_t n, double* out, const char* what) {
  if (!j || j->kind != Json::ARR || j->arr.size() < n) raise(std::string("expected ") + std::to_string(n) +
                                                             " numbers for " + what);
  for (size_t k = 0; k < n; ++k) out[k] = as_f(&j->arr[k], 0.0, what);
}

// ------------------------------------------------------------------ files
std::vector<uint8_t> read_file(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) raise("cannot open " + path);
  std::vector<uint8_t> out;
  uint8_t buf[1 << 16];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) out.insert(out.end(), buf, buf + n);
  std::fclose(f);
  return out;
}

// base64 of a data URI; characters outside the alphabet are skipped
std::vector<uint8_t> base64(const std::string& s) {
  std::vector<uint8_t> out;
  uint32_t acc = 0;
  int bits = 0;
  for (char c : s) {
    int v;
    if (c >= 'A' && c <= 'Z') v = c - 'A';
    else if (c >= 'a' && c <= 'z') v = c - 'a' + 26;
    else if (c >= '0' && c <= '9') v = c - '0' + 52;
    else if (c == '+') v = 62;
    else if (c == '/') v = 63;
    else if (c == '=') break;
    else continue;
    acc = (acc << 6) | (uint32_t)v;
    bits += 6;
    if (bits >= 8) {
      bits -= 8;
      out.push_back((uint8_t)(acc >> bits));
    }
  }
  return out;
}

std::vector<uint8_t> uri_bytes(const std::string& uri, const std::string& base) {
  if (uri.compare(0, 5, "data:") == 0) {
    const size_t comma = uri.find(',');
    if (comma == std::string::npos) raise("data URI without ','");
    return base64(uri.substr(comma + 1));
  }
  std::string rel = uri;
  for (size_t k; (k = rel.find("%20")) != std::string::npos;) rel.replace(k, 3, " ");
  return read_file(base.empty() ? rel : base + "/" + rel);
}

// ------------------------------------------------------------------ images
const uint8_t PNG_SIG[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};

struct Image {
  uint32_t w = 0, h = 0;
  std::vector<float> rgba;
};

// float RGBA in [0, 1], as the Python png.read gives it (pt_png.cu)
Image png_read(const std::vector<uint8_t>& buf) {
  Image im;
  const std::string why = hpt::png_decode_float(buf.data(), buf.size(), im.w, im.h, im.rgba);
  if (!why.empty()) raise("PNG: " + why);
  return im;
}

// ------------------------------------------------------------------ document
struct Mat4 {
  double m[4][4];  // row-major
};
Mat4 identity() {
  Mat4 r{};
  for (int k = 0; k < 4; ++k) r.m[k][k] = 1.0;
  return r;
}
Mat4 mul(const Mat4& a, const Mat4& b) {
  Mat4 r{};
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j)
      r.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j] + a.m[i][3] * b.m[3][j];
  return r;
}

struct V3 {
  double x, y, z;
};
V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
// numpy.cross: (a1 b2 - a2 b1, a2 b0 - a0 b2, a0 b1 - a1 b0)
V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
double norm(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
V3 column(const Mat4& M, int k) { return {M.m[0][k], M.m[1][k], M.m[2][k]}; }
V3 scale(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
V3 divide(V3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
void put(float* dst, V3 v) {
  dst[0] = (float)v.x;
  dst[1] = (float)v.y;
  dst[2] = (float)v.z;
}

const double DEG_TO_RAD = M_PI / 180.0;  // math.radians
const double RAD_TO_DEG = 180.0 / M_PI;  // math.degrees

class Doc {
 public:
  Json j;
  std::string base;
  std::vector<std::vector<uint8_t>> buffers;

  explicit Doc(const std::string& path) {
    const size_t slash = path.find_last_of('/');
    base = slash == std::string::npos ? std::string(".") : path.substr(0, slash);
    const std::vector<uint8_t> data = read_file(path);
    std::vector<uint8_t> glb_bin;
    bool have_bin = false;
    if (data.size() >= 4 && !std::memcmp(data.data(), "glTF", 4)) {
      if (data.size() < 12) raise("GLB: truncated header");
      size_t pos = 12;
      bool have_json = false;
      while (pos < data.size()) {
        if (pos + 8 > data.size()) raise("GLB: truncated chunk");
        const uint32_t n = (uint32_t)data[pos] | (uint32_t)data[pos + 1] << 8 | (uint32_t)data[pos + 2] << 16 |
                           (uint32_t)data[pos + 3] << 24;
        const uint8_t* typ = &data[pos + 4];
        const size_t b0 = pos + 8, b1 = std::min(data.size(), b0 + (size_t)n);
        pos = b0 + (size_t)n;
        if (!std::memcmp(typ, "JSON", 4)) {
          j = JsonParser(reinterpret_cast<const char*>(&data[b0]), b1 - b0).parse();
          have_json = true;
        } else if (!std::memcmp(typ, "BIN\0", 4)) {
          glb_bin.assign(data.begin() + b0, data.begin() + b1);
          have_bin = true;
        }
      }
      if (!have_json) raise("GLB without a JSON chunk");
    } else {
      j = JsonParser(reinterpret_cast<const char*>(data.data()), data.size()).parse();
    }
    if (j.kind != Json::OBJ) raise("the document is not a JSON object");
    if (const Json* bs = j.get("buffers")) {
      if (bs->kind != Json::ARR) raise("\"buffers\" is not a list");
      for (size_t i = 0; i < bs->arr.size(); ++i) {
        const Json* uri = bs->arr[i].get("uri");
        if (uri) buffers.push_back(uri_bytes(uri->str, base));
        else if (i == 0 && have_bin) buffers.push_back(glb_bin);
        else raise("buffer " + std::to_string(i) + " has no data");
      }
    }
  }

  // bytes of a buffer view (clamped to its buffer, as a slice) and its stride
  std::pair<std::vector<uint8_t>, size_t> view_bytes(long long vi) const {
    const Json& v = at(need(j, "bufferViews"), vi, "bufferViews");
    const long long bi = as_i(&need(v, "buffer"), 0, "buffer");
    if (bi < 0 || (size_t)bi >= buffers.size()) raise("bad buffer index");
    const std::vector<uint8_t>& b = buffers[(size_t)bi];
    const size_t off = std::min(b.size(), (size_t)std::max(0LL, as_i(v.get("byteOffset"), 0, "byteOffset")));
    const size_t len = (size_t)std::max(0LL, as_i(&need(v, "byteLength"), 0, "byteLength"));
    const size_t e = std::min(b.size(), off + len);
    return {std::vector<uint8_t>(b.begin() + off, b.begin() + e),
            (size_t)std::max(0LL, as_i(v.get("byteStride"), 0, "byteStride"))};
  }

  // accessor -> count x nc doubles (float for normalized integers, as the
  // Python loader divides in float32)
  std::vector<double> accessor(long long ai, size_t& nc_out) const {
    const Json& a = at(need(j, "accessors"), ai, "accessors");
    if (a.get("sparse")) raise("sparse accessors are not supported");
    const long long ct = as_i(&need(a, "componentType"), 0, "componentType");
    size_t isz;
    switch (ct) {
      case 5120: case 5121: isz = 1; break;
      case 5122: case 5123: isz = 2; break;
      case 5125: case 5126: isz = 4; break;
      default: raise("unknown componentType " + std::to_string(ct));
    }
    const std::string type = need(a, "type").str;
    size_t nc;
    if (type == "SCALAR") nc = 1;
    else if (type == "VEC2") nc = 2;
    else if (type == "VEC3") nc = 3;
    else if (type == "VEC4") nc = 4;
    else if (type == "MAT4") nc = 16;
    else raise("unsupported accessor type " + type);
    nc_out = nc;
    const long long count_ll = as_i(&need(a, "count"), 0, "count");
    if (count_ll < 0 || count_ll > (1LL << 31)) raise("bad accessor count");
    const size_t count = (size_t)count_ll, item = isz * nc;
    const Json* bv = a.get("bufferView");
    if (!bv) {  // all zeros; bounded like the largest accessor a buffer could hold
      if (count * nc > (1ull << 28)) raise("accessor " + std::to_string(ai) + " is too large");
      return std::vector<double>(count * nc, 0.0);
    }
    const auto vb = view_bytes(as_i(bv, 0, "bufferView"));
    const std::vector<uint8_t>& raw = vb.first;
    const size_t stride = vb.second ? vb.second : item;
    const size_t off = (size_t)std::max(0LL, as_i(a.get("byteOffset"), 0, "byteOffset"));
    // checked before anything is allocated
    if (count && (off > raw.size() || (count - 1) > (raw.size() - off) / stride ||
                  off + (count - 1) * stride + item > raw.size()))
      raise("accessor " + std::to_string(ai) + " reads past its buffer view");
    std::vector<double> out(count * nc, 0.0);
    const bool normalized = a.get("normalized") && a.get("normalized")->truthy() && ct != 5126;
    for (size_t i = 0; i < count; ++i) {
      const uint8_t* p = raw.data() + off + i * stride;
      for (size_t c = 0; c < nc; ++c, p += isz) {
        double v;
        float scale_f = 1.0f;
        switch (ct) {
          case 5120: v = (int8_t)p[0]; scale_f = 127.0f; break;
          case 5121: v = p[0]; scale_f = 255.0f; break;
          case 5122: v = (int16_t)(uint16_t)(p[0] | p[1] << 8); scale_f = 32767.0f; break;
          case 5123: v = (uint16_t)(p[0] | p[1] << 8); scale_f = 65535.0f; break;
          case 5125: v = (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24; break;
          default: {
            float f;
            std::memcpy(&f, p, 4);
            v = f;
          }
        }
        if (normalized) {
          if (ct == 5125) raise("normalized UNSIGNED_INT accessors are not supported");
          v = std::max((float)v / scale_f, -1.0f);
        }
        out[i * nc + c] = v;
      }
    }
    return out;
  }
};

Mat4 node_matrix(const Json& n) {
  Mat4 M = identity();
  if (const Json* m = n.get("matrix")) {
    double a[16];
    floats(m, 16, a, "matrix");
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c) M.m[r][c] = a[c * 4 + r];  // column-major in the file
    return M;
  }
  double t[3] = {0, 0, 0}, q[4] = {0, 0, 0, 1}, s[3] = {1, 1, 1};
  if (const Json* v = n.get("translation")) floats(v, 3, t, "translation");
  if (const Json* v = n.get("rotation")) floats(v, 4, q, "rotation");
  if (const Json* v = n.get("scale")) floats(v, 3, s, "scale");
  const double x = q[0], y = q[1], z = q[2], w = q[3];
  const double R[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)},
                          {2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)},
                          {2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)}};
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) M.m[r][c] = R[r][c] * s[c];
    M.m[r][3] = t[r];
  }
  return M;
}

// (node index, world matrix) of every node of the default scene, pre-order
void walk(const Json& j, long long i, const Mat4& parent, std::vector<std::pair<long long, Mat4>>& out, int depth) {
  if (depth > 1024) raise("node hierarchy too deep (a cycle?)");
  if (out.size() >= (1u << 20)) raise("more than 2^20 node instances (shared subtrees?)");
  const Json& n = at(need(j, "nodes"), i, "nodes");
  const Mat4 M = mul(parent, node_matrix(n));
  out.emplace_back(i, M);
  if (const Json* ch = n.get("children"))
    for (const Json& c : ch->arr) walk(j, as_i(&c, 0, "children"), M, out, depth + 1);
}

float srgb_to_linear(float c) {
  return c <= 0.04045f ? c / 12.92f : std::pow((c + 0.055f) / 1.055f, 2.4f);
}

pt_material default_material(const float bc[3], uint32_t type) {
  pt_material m{};
  for (int k = 0; k < 3; ++k) {
    m.base_color[k] = bc[k];
    m.clearcoat_tint[k] = 1.0f;
  }
  m.opacity = 1.0f;
  m.ior = 1.5f;
  m.base_color_map_index = m.normal_map_index = m.metallic_roughness_map_index = m.emission_map_index =
      PT_INVALID_INDEX;
  m.type = type;
  m.medium.type = PT_MEDIUM_NONE;
  return m;
}

class Loader {
 public:
  Loader(const Doc& d, pt_gltf_scene& s) : doc_(d), s_(s) {}

  void run() {
    const Json& j = doc_.j;
    if (const Json* ms = j.get("materials"))
      for (const Json& m : ms->arr) s_.mats.push_back(material(m));
    long long default_mat = -1;
    const Json* lights_ext = nullptr;
    if (const Json* e = j.get("extensions"))
      if (const Json* k = e->get("KHR_lights_punctual")) lights_ext = k->get("lights");
    std::vector<std::pair<long long, Mat4>> nodes;
    const Json* scenes = j.get("scenes");
    if (scenes && scenes->kind == Json::ARR && !scenes->arr.empty()) {
      const Json& sc = at(*scenes, as_i(j.get("scene"), 0, "scene"), "scenes");
      for (const Json& r : need(sc, "nodes").arr) walk(j, as_i(&r, 0, "nodes"), identity(), nodes, 0);
    } else if (const Json* ns = j.get("nodes")) {
      for (size_t i = 0; i < ns->arr.size(); ++i) walk(j, (long long)i, identity(), nodes, 0);
    }
    for (const auto& nm : nodes) {
      const Json& n = j.get("nodes")->arr[(size_t)nm.first];
      const Mat4& M = nm.second;
      if (const Json* mesh = n.get("mesh")) {
        const Json& me = at(need(j, "meshes"), as_i(mesh, 0, "mesh"), "meshes");
        for (const Json& prim : need(me, "primitives").arr) {
          if (as_i(prim.get("mode"), 4, "mode") != 4) continue;
          const Json* mi = prim.get("material");
          long long mat;
          if (!mi || mi->kind == Json::NUL) {
            if (default_mat < 0) {
              const float grey[3] = {0.8f, 0.8f, 0.8f};
              pt_material m = default_material(grey, PT_MATERIAL_DIFFUSE);
              pt_material_preprocess(&m);
              s_.mats.push_back(m);
              default_mat = (long long)s_.mats.size() - 1;
            }
            mat = default_mat;
          } else {
            mat = as_i(mi, 0, "material");
          }
          primitive(prim, M, (uint32_t)mat);
        }
      }
      if (const Json* c = n.get("camera"))
        if (s_.cams.size() < PT_MAX_CAMERAS) s_.cams.push_back(camera(at(need(j, "cameras"), as_i(c, 0, "camera"),
                                                                          "cameras"), M));
      const Json* li = nullptr;
      if (const Json* e = n.get("extensions"))
        if (const Json* k = e->get("KHR_lights_punctual")) li = k->get("light");
      if (li && li->kind != Json::NUL && s_.lights.size() < PT_MAX_LIGHTS) {
        if (!lights_ext) raise("a node names a KHR_lights_punctual light but the document has none");
        s_.lights.push_back(light(at(*lights_ext, as_i(li, 0, "light"), "lights"), M));
      }
    }
    if (s_.cams.empty()) raise("the scene has no camera");
  }

 private:
  const Doc& doc_;
  pt_gltf_scene& s_;
  std::map<long long, std::shared_ptr<Image>> images_;  // null: not a PNG
  std::map<std::tuple<long long, int, std::vector<double>>, uint32_t> baked_;

  std::shared_ptr<Image> image(long long ii) {
    auto it = images_.find(ii);
    if (it != images_.end()) return it->second;
    const Json& im = at(need(doc_.j, "images"), ii, "images");
    std::vector<uint8_t> data;
    if (const Json* uri = im.get("uri")) data = uri_bytes(uri->str, doc_.base);
    else data = doc_.view_bytes(as_i(&need(im, "bufferView"), 0, "bufferView")).first;
    std::shared_ptr<Image> out;
    if (data.size() >= 8 && !std::memcmp(data.data(), PNG_SIG, 8)) out = std::make_shared<Image>(png_read(data));
    else ++s_.skipped_images;
    images_[ii] = out;
    return out;
  }

  // factor x texel map of a texture reference; kind 0 sRGB colour, 1
  // metallic (blue) / roughness (green), 2 linear (normal map)
  uint32_t bake(const Json* info, const std::vector<double>& factor, int kind) {
    if (!info || info->kind == Json::NUL) return PT_INVALID_INDEX;
    const Json& tex = at(need(doc_.j, "textures"), as_i(&need(*info, "index"), 0, "index"), "textures");
    const Json* src = tex.get("source");
    if (!src || src->kind == Json::NUL) return PT_INVALID_INDEX;
    const long long si = as_i(src, 0, "source");
    std::vector<double> key_f;
    for (double f : factor) key_f.push_back(std::nearbyint(f * 1e7) / 1e7);  // numpy.round(x, 7)
    const auto key = std::make_tuple(si, kind, key_f);
    auto it = baked_.find(key);
    if (it != baked_.end()) return it->second;
    std::shared_ptr<Image> img = image(si);
    if (!img) return PT_INVALID_INDEX;
    std::vector<float> t = img->rgba;
    const size_t n = (size_t)img->w * img->h;
    if (kind == 0) {
      const float f[3] = {(float)factor[0], (float)factor[1], (float)factor[2]};
      for (size_t p = 0; p < n; ++p)
        for (int k = 0; k < 3; ++k) t[4 * p + k] = srgb_to_linear(t[4 * p + k]) * f[k];
    } else if (kind == 1) {
      const float fm = (float)factor[0], fr = (float)factor[1];
      for (size_t p = 0; p < n; ++p) {
        t[4 * p + 2] *= fm;
        t[4 * p + 1] *= fr;
      }
    }
    s_.texels.push_back(std::move(t));
    pt_texture tx{};
    tx.width = img->w;
    tx.height = img->h;
    s_.texs.push_back(tx);
    const uint32_t idx = (uint32_t)s_.texs.size() - 1;
    baked_[key] = idx;
    return idx;
  }

  pt_material material(const Json& m) {
    static const Json empty_obj = [] {
      Json e;
      e.kind = Json::OBJ;
      return e;
    }();
    const Json* pbr_p = m.get("pbrMetallicRoughness");
    const Json& pbr = pbr_p ? *pbr_p : empty_obj;
    const Json* ext_p = m.get("extensions");
    const Json& ext = ext_p ? *ext_p : empty_obj;
    const Json* extras = m.get("extras");
    if (extras && !extras->truthy()) extras = nullptr;
    double bc[4] = {1, 1, 1, 1};
    bool has_alpha = true;
    if (const Json* v = pbr.get("baseColorFactor")) {
      floats(v, 3, bc, "baseColorFactor");
      has_alpha = v->arr.size() > 3;
      if (has_alpha) bc[3] = as_f(&v->arr[3], 1.0, "baseColorFactor");
    }
    const double metallic = as_f(pbr.get("metallicFactor"), 1.0, "metallicFactor");
    const double rough = as_f(pbr.get("roughnessFactor"), 1.0, "roughnessFactor");
    double emis[3] = {0, 0, 0};
    if (const Json* v = m.get("emissiveFactor")) floats(v, 3, emis, "emissiveFactor");
    double strength = 1.0;
    if (const Json* k = ext.get("KHR_materials_emissive_strength"))
      strength = as_f(k->get("emissiveStrength"), 1.0, "emissiveStrength");
    for (double& e : emis) e = e * strength;
    double ior = 1.5, trans = 0.0, clearcoat = 0.0, cc_rough = 0.0;
    if (const Json* k = ext.get("KHR_materials_ior")) ior = as_f(k->get("ior"), 1.5, "ior");
    if (const Json* k = ext.get("KHR_materials_transmission"))
      trans = as_f(k->get("transmissionFactor"), 0.0, "transmissionFactor");
    if (const Json* k = ext.get("KHR_materials_clearcoat")) {
      clearcoat = as_f(k->get("clearcoatFactor"), 0.0, "clearcoatFactor");
      cc_rough = as_f(k->get("clearcoatRoughnessFactor"), 0.0, "clearcoatRoughnessFactor");
    }
    double opacity = 1.0;
    const Json* mode = m.get("alphaMode");
    const std::string mode_s = mode && mode->kind == Json::STR ? mode->str : "OPAQUE";
    if ((mode_s == "BLEND" || mode_s == "MASK") && !has_alpha) raise("baseColorFactor has no alpha");
    if (mode_s == "BLEND") opacity = bc[3];
    else if (mode_s == "MASK") opacity = bc[3] >= as_f(m.get("alphaCutoff"), 0.5, "alphaCutoff") ? 1.0 : 0.0;
    uint32_t mtype = (metallic > 0 || trans > 0 || clearcoat > 0) ? PT_MATERIAL_DISNEY : PT_MATERIAL_DIFFUSE;
    if (extras)
      if (const Json* t = extras->get("type")) {
        const std::string lt = lower_text(*t);
        long long v;
        if (lt == "diffuse" || lt == "lambert") mtype = PT_MATERIAL_DIFFUSE;
        else if (lt == "disney") mtype = PT_MATERIAL_DISNEY;
        else if (digit_text(*t, v)) mtype = (uint32_t)v;
        else mtype = PT_MATERIAL_DIFFUSE;
      }
    const float bcf[3] = {(float)bc[0], (float)bc[1], (float)bc[2]};
    pt_material mat = default_material(bcf, mtype);
    mat.roughness = (float)rough;
    mat.metallic = (float)metallic;
    mat.specular_transmission = (float)trans;
    mat.ior = (float)ior;
    mat.opacity = (float)opacity;
    put(mat.emission, {emis[0], emis[1], emis[2]});
    mat.clearcoat = (float)clearcoat;
    mat.clearcoat_roughness = (float)cc_rough;
    if (extras) {
      for (const auto& kv : extras->obj) {
        const std::string& name = kv.first;
        const Json& v = kv.second;
        float* scalar = nullptr;
        float* vec = nullptr;
        if (name == "base_color") vec = mat.base_color;
        else if (name == "emission") vec = mat.emission;
        else if (name == "clearcoat_tint") vec = mat.clearcoat_tint;
        else if (name == "opacity") scalar = &mat.opacity;
        else if (name == "anisotropic") scalar = &mat.anisotropic;
        else if (name == "metallic") scalar = &mat.metallic;
        else if (name == "roughness") scalar = &mat.roughness;
        else if (name == "subsurface") scalar = &mat.subsurface;
        else if (name == "specular_tint") scalar = &mat.specular_tint;
        else if (name == "sheen") scalar = &mat.sheen;
        else if (name == "sheen_tint") scalar = &mat.sheen_tint;
        else if (name == "clearcoat") scalar = &mat.clearcoat;
        else if (name == "clearcoat_roughness") scalar = &mat.clearcoat_roughness;
        else if (name == "specular_transmission") scalar = &mat.specular_transmission;
        else if (name == "ior") scalar = &mat.ior;
        else if (name == "ax") scalar = &mat.ax;
        else if (name == "ay") scalar = &mat.ay;
        // "type" and "medium" are read above and below; the map indices are
        // set by the texture references; other names are not material fields
        if (vec) {
          double a[3];
          floats(&v, 3, a, name.c_str());
          put(vec, {a[0], a[1], a[2]});
        } else if (scalar) {
          *scalar = (float)as_f(&v, 0.0, name.c_str());
        }
      }
      const Json* med = extras->get("medium");
      if (med && med->truthy()) {
        const Json* mt = med->get("type");
        long long tv;
        uint32_t type = PT_MEDIUM_ABSORB;  // default "absorb"
        if (mt) {
          const std::string l = lower_text(*mt);
          if (l == "absorb") type = PT_MEDIUM_ABSORB;
          else if (l == "scatter") type = PT_MEDIUM_SCATTER;
          else if (l == "emissive") type = PT_MEDIUM_EMISSIVE;
          else if (digit_text(*mt, tv)) type = (uint32_t)tv;
          else type = PT_MEDIUM_NONE;
        }
        mat.medium.type = type;
        double c[3] = {1, 1, 1};
        if (const Json* cv = med->get("color")) floats(cv, 3, c, "medium color");
        put(mat.medium.color, {c[0], c[1], c[2]});
        mat.medium.density = (float)as_f(med->get("density"), 0.0, "density");
        mat.medium.anisotropy = (float)as_f(med->get("anisotropy"), 0.0, "anisotropy");
      }
    }
    mat.base_color_map_index =
        bake(pbr.get("baseColorTexture"), {mat.base_color[0], mat.base_color[1], mat.base_color[2]}, 0);
    mat.metallic_roughness_map_index = bake(pbr.get("metallicRoughnessTexture"), {mat.metallic, mat.roughness}, 1);
    mat.emission_map_index = bake(m.get("emissiveTexture"), {mat.emission[0], mat.emission[1], mat.emission[2]}, 0);
    mat.normal_map_index = bake(m.get("normalTexture"), {1.0, 1.0, 1.0}, 2);
    pt_material_preprocess(&mat);
    return mat;
  }

  void primitive(const Json& prim, const Mat4& M, uint32_t mat) {
    const Json& attrs = need(prim, "attributes");
    size_t nc;
    const std::vector<double> pos = doc_.accessor(as_i(&need(attrs, "POSITION"), 0, "POSITION"), nc);
    if (nc != 3) raise("POSITION is not VEC3");
    const size_t nv = pos.size() / 3;
    std::vector<uint32_t> idx;
    if (const Json* ij = prim.get("indices")) {
      const std::vector<double> iv = doc_.accessor(as_i(ij, 0, "indices"), nc);
      idx.resize(iv.size());
      for (size_t k = 0; k < iv.size(); ++k) idx[k] = (uint32_t)(int64_t)iv[k];
    } else {
      idx.resize(nv);
      for (size_t k = 0; k < nv; ++k) idx[k] = (uint32_t)k;
    }
    std::vector<double> nrm;
    if (const Json* a = attrs.get("NORMAL")) {
      nrm = doc_.accessor(as_i(a, 0, "NORMAL"), nc);
      if (nc != 3 || nrm.size() != pos.size()) raise("NORMAL does not match POSITION");
    } else {
      // area-weighted face normals summed into each corner (first, second,
      // then third corners of all triangles in turn), normalised
      if (idx.size() % 3) raise("index count is not a multiple of 3");
      const size_t nt = idx.size() / 3;
      nrm.assign(pos.size(), 0.0);
      std::vector<V3> fn(nt);
      for (size_t t = 0; t < nt; ++t) {
        for (int k = 0; k < 3; ++k)
          if (idx[3 * t + k] >= nv) raise("index out of range");
        auto P = [&](uint32_t i) { return V3{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]}; };
        const V3 p0 = P(idx[3 * t]);
        fn[t] = cross(sub(P(idx[3 * t + 1]), p0), sub(P(idx[3 * t + 2]), p0));
      }
      for (int k = 0; k < 3; ++k)
        for (size_t t = 0; t < nt; ++t) {
          double* n = &nrm[3 * (size_t)idx[3 * t + k]];
          n[0] += fn[t].x;
          n[1] += fn[t].y;
          n[2] += fn[t].z;
        }
      for (size_t v = 0; v < nv; ++v) {
        double* n = &nrm[3 * v];
        const double l = std::max(norm({n[0], n[1], n[2]}), 1e-30);
        for (int k = 0; k < 3; ++k) n[k] = n[k] / l;
      }
    }
    std::vector<double> tan(3 * nv);
    if (const Json* a = attrs.get("TANGENT")) {
      const std::vector<double> t4 = doc_.accessor(as_i(a, 0, "TANGENT"), nc);
      if (nc < 3 || t4.size() / nc != nv) raise("TANGENT does not match POSITION");
      for (size_t v = 0; v < nv; ++v)
        for (int k = 0; k < 3; ++k) tan[3 * v + k] = t4[v * nc + k];
    } else {
      for (size_t v = 0; v < nv; ++v) {
        const V3 n{nrm[3 * v], nrm[3 * v + 1], nrm[3 * v + 2]};
        const V3 up = std::fabs(n.z) < 0.999 ? V3{0.0, 0.0, 1.0} : V3{1.0, 0.0, 0.0};
        const V3 t = cross(up, n);
        const double l = norm(t);
        tan[3 * v] = t.x / l;
        tan[3 * v + 1] = t.y / l;
        tan[3 * v + 2] = t.z / l;
      }
    }
    std::vector<double> uv(2 * nv, 0.0);
    if (const Json* a = attrs.get("TEXCOORD_0")) {
      uv = doc_.accessor(as_i(a, 0, "TEXCOORD_0"), nc);
      if (nc != 2 || uv.size() != 2 * nv) raise("TEXCOORD_0 does not match POSITION");
    }
    std::vector<float> verts(11 * nv);
    for (size_t v = 0; v < nv; ++v) {
      float* o = &verts[11 * v];
      for (int k = 0; k < 3; ++k) {
        o[k] = (float)pos[3 * v + k];
        o[3 + k] = (float)nrm[3 * v + k];
        o[6 + k] = (float)tan[3 * v + k];
      }
      o[9] = (float)uv[2 * v];
      o[10] = (float)uv[2 * v + 1];
    }
    pt_primitive p{};
    p.num_vertices = (uint32_t)nv;
    p.num_indices = (uint32_t)idx.size();
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c) p.transform[c * 4 + r] = (float)M.m[r][c];  // column-major
    p.material_index = mat;
    s_.verts.push_back(std::move(verts));
    s_.indices.push_back(std::move(idx));
    s_.prims.push_back(p);
  }

  pt_light light(const Json& L, const Mat4& M) {
    double color[3] = {1, 1, 1};
    if (const Json* c = L.get("color")) floats(c, 3, color, "light color");
    const double inten = as_f(L.get("intensity"), 1.0, "intensity");
    const Json* extras = L.get("extras");
    if (extras && !extras->truthy()) extras = nullptr;
    V3 I;
    if (extras && extras->get("rgb")) {
      double rgb[3];
      floats(extras->get("rgb"), 3, rgb, "rgb");
      I = {rgb[0], rgb[1], rgb[2]};
    } else {
      I = {color[0] * inten, color[1] * inten, color[2] * inten};
    }
    const V3 pos = column(M, 3), X = column(M, 0), Y = column(M, 1), Z = column(M, 2);
    const V3 fwd = divide({-Z.x, -Z.y, -Z.z}, std::max(norm(Z), 1e-30));
    const long long etype = extras ? as_i(extras->get("type"), 0, "light type") : 0;
    pt_light out{};
    if (etype == 1) {  // rectangle
      const double w = as_f(extras->get("param0"), 1.0, "param0"), h = as_f(extras->get("param1"), 1.0, "param1");
      const V3 u = scale(divide(X, norm(X)), w), v = scale(divide(Y, norm(Y)), h);
      const double area = w * h;
      const V3 rad = divide(scale(I, 4.0), std::max(area, 1e-30));
      const V3 corner = sub(sub(pos, scale(u, 0.5)), scale(v, 0.5));
      out.type = PT_LIGHT_QUAD;
      put(out.intensity, rad);
      put(out.position, corner);
      put(out.u, u);
      put(out.v, v);
      out.area = (float)norm(cross(u, v));
      return out;
    }
    if (etype == 2) {  // sphere
      const double r = as_f(extras->get("param0"), 0.1, "param0");
      out.type = PT_LIGHT_SPHERE;
      put(out.intensity, divide(I, M_PI * r * r));
      put(out.position, pos);
      out.radius = (float)r;
      out.area = (float)(4.0 * M_PI * r * r);
      return out;
    }
    const Json* kind_j = L.get("type");
    const std::string kind = kind_j && kind_j->kind == Json::STR ? kind_j->str : "point";
    if (kind == "directional") {
      const double cone = extras ? as_f(extras->get("cone_deg"), 0.0, "cone_deg") : 0.0;
      out.type = PT_LIGHT_DIRECTIONAL;
      put(out.intensity, I);
      put(out.u, divide(fwd, norm(fwd)));
      out.v[0] = cone > 0 ? (float)std::cos(cone * DEG_TO_RAD) : 0.0f;
      return out;
    }
    if (kind == "spot") {
      const Json* spot = L.get("spot");
      const double inner = as_f(spot ? spot->get("innerConeAngle") : nullptr, 0.0, "innerConeAngle") * RAD_TO_DEG;
      const double outer = as_f(spot ? spot->get("outerConeAngle") : nullptr, M_PI / 4, "outerConeAngle") * RAD_TO_DEG;
      out.type = PT_LIGHT_SPOT;
      put(out.intensity, I);
      put(out.position, pos);
      put(out.u, divide(fwd, norm(fwd)));
      out.v[0] = (float)std::cos(inner * DEG_TO_RAD);
      out.v[1] = (float)std::cos(outer * DEG_TO_RAD);
      return out;
    }
    out.type = PT_LIGHT_POINT;
    put(out.intensity, I);
    put(out.position, pos);
    return out;
  }

  pt_camera camera(const Json& c, const Mat4& M) {
    pt_camera cam{};
    V3 ax[3];
    for (int k = 0; k < 3; ++k) ax[k] = divide(column(M, k), norm(column(M, k)));
    put(cam.position, column(M, 3));
    put(cam.right, ax[0]);
    put(cam.up, ax[1]);
    put(cam.forward, {-ax[2].x, -ax[2].y, -ax[2].z});
    const Json* extras = c.get("extras");
    if (extras && !extras->truthy()) extras = nullptr;
    const Json* type = c.get("type");
    if (type && type->kind == Json::STR && type->str == "orthographic") {
      const Json& o = need(c, "orthographic");
      cam.type = PT_CAMERA_ORTHOGRAPHIC;
      cam.yfov = (float)(extras ? as_f(extras->get("yfov"), 0.0, "yfov") : 0.0);
      cam.focal_distance_or_xmag = (float)as_f(&need(o, "xmag"), 0.0, "xmag");
      cam.aperture_or_ymag = (float)as_f(&need(o, "ymag"), 0.0, "ymag");
    } else {
      const Json* p = c.get("perspective");
      cam.type = PT_CAMERA_PERSPECTIVE;
      cam.yfov = (float)as_f(p ? p->get("yfov") : nullptr, 40.0 * DEG_TO_RAD, "yfov");
      cam.focal_distance_or_xmag = (float)(extras ? as_f(extras->get("focal_distance"), 1.0, "focal_distance") : 1.0);
      cam.aperture_or_ymag = (float)(extras ? as_f(extras->get("aperture"), 0.0, "aperture") : 0.0);
    }
    return cam;
  }
};

void set_error(char* buf, size_t cap, const std::string& m) {
  if (buf && cap) {
    const size_t n = std::min(cap - 1, m.size());
    std::memcpy(buf, m.data(), n);
    buf[n] = '\0';
  }
}

}  // namespace

extern "C" {

pt_status pt_gltf_load(const char* path, pt_gltf_scene** out, char* error_message, size_t error_capacity) {
  if (!path || !out) {
    set_error(error_message, error_capacity, "path and out must not be NULL");
    return PT_ERR_INVALID_ARG;
  }
  *out = nullptr;
  std::unique_ptr<pt_gltf_scene> s(new (std::nothrow) pt_gltf_scene());
  if (!s) return PT_ERR_OOM;
  try {
    const Doc doc(path);
    Loader(doc, *s).run();
  } catch (const LoadError& e) {
    set_error(error_message, error_capacity, std::string(path) + ": " + e.msg);
    return PT_ERR_INVALID_ARG;
  } catch (const std::bad_alloc&) {
    set_error(error_message, error_capacity, "out of host memory");
    return PT_ERR_OOM;
  } catch (const std::exception& e) {  // nothing may cross the C boundary
    set_error(error_message, error_capacity, std::string(path) + ": " + e.what());
    return PT_ERR_INVALID_ARG;
  }
  for (size_t i = 0; i < s->prims.size(); ++i) {
    s->prims[i].vertices = s->verts[i].data();
    s->prims[i].indices = s->indices[i].data();
  }
  for (size_t i = 0; i < s->texs.size(); ++i) s->texs[i].rgba = s->texels[i].data();
  pt_scene_desc& d = s->desc;
  d.primitives = s->prims.data();
  d.num_primitives = (uint32_t)s->prims.size();
  d.materials = s->mats.data();
  d.num_materials = (uint32_t)s->mats.size();
  d.lights = s->lights.data();
  d.num_lights = (uint32_t)s->lights.size();
  d.cameras = s->cams.data();
  d.num_cameras = (uint32_t)s->cams.size();
  d.textures = s->texs.data();
  d.num_textures = (uint32_t)s->texs.size();
  *out = s.release();
  set_error(error_message, error_capacity, "");
  return PT_OK;
}

const pt_scene_desc* pt_gltf_scene_desc(const pt_gltf_scene* scene) { return scene ? &scene->desc : nullptr; }

uint32_t pt_gltf_skipped_images(const pt_gltf_scene* scene) { return scene ? scene->skipped_images : 0; }

void pt_gltf_free(pt_gltf_scene* scene) { delete scene; }

pt_status pt_renderer_set_scene_file(pt_renderer* r, const char* path) try {
  if (!r) return PT_ERR_INVALID_ARG;
  char why[512];
  pt_gltf_scene* scene = nullptr;
  const pt_status st = pt_gltf_load(path, &scene, why, sizeof(why));
  if (st != PT_OK) {
    r->err = std::string("scene ") + why;
    return st;
  }
  const pt_status rs = pt_renderer_set_scene(r, &scene->desc);
  pt_gltf_free(scene);
  return rs;
} catch (...) {
  return host_exception_status(r ? &r->err : nullptr);
}

}  // extern "C"
