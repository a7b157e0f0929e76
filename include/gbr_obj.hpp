// gbr_obj.hpp — scene ingest for the C++ API of gbr_engine.hpp: Wavefront
// OBJ + MTL geometry and material loading in the manner of the reference's
// obj_load (obj_load.cpp:181-568), and RGBA8 image decoding for textures
// (PNG through zlib, binary PPM, uncompressed TGA) in place of the
// reference's SFML image loader (texture.cpp:323-358).
//
// As in the reference: one object per `usemtl` section, with the material's
// map_Kd texture, or a 32x32 texture of its Kd colour, or magenta when the
// material has neither; positions scaled by the container's requested scale;
// vt and vn taken as written (the atlas upload flips rows as the reference).
// Beyond the reference, which requires triangulated v/vt/vn faces: polygons
// are split into fans, faces without vt get (0, 0) and faces without vn get
// the face normal, and negative (relative) indices are resolved.  Textures must
// be square powers of two from 16 to 2048 in the atlas; other images are
// resampled (nearest texel) to the next power of two in that range.
//
// Header-only; PNG decoding needs zlib (link -lz).
#ifndef GBR_OBJ_HPP
#define GBR_OBJ_HPP

#include <zlib.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "gbr_engine.hpp"

namespace openclrenderer {

// ---- images ----------------------------------------------------------------------
namespace image_detail {

inline uint32_t be32(const uint8_t* p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }

inline bool read_file(const std::string& path, std::vector<uint8_t>& out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  out.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
  return true;
}

inline int paeth(int a, int b, int c) {
  const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
  return (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
}

// PNG: 8-bit grey, grey+alpha, RGB, RGBA and palette images, not interlaced.
inline bool decode_png(const std::vector<uint8_t>& d, int& w, int& h, std::vector<uint8_t>& rgba, std::string& err) {
  static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
  if (d.size() < 8 || std::memcmp(d.data(), sig, 8) != 0) return err = "not a PNG", false;
  size_t pos = 8;
  int depth = 0, ctype = -1, interlace = 0;
  std::vector<uint8_t> idat, plte, trns;
  while (pos + 12 <= d.size()) {
    const uint32_t len = be32(&d[pos]);
    const std::string type(reinterpret_cast<const char*>(&d[pos + 4]), 4);
    if (pos + 12 + (size_t)len > d.size()) return err = "truncated PNG chunk", false;
    const uint8_t* c = &d[pos + 8];
    if (type == "IHDR" && len >= 13) {
      w = (int)be32(c);
      h = (int)be32(c + 4);
      depth = c[8];
      ctype = c[9];
      interlace = c[12];
    } else if (type == "PLTE") {
      plte.assign(c, c + len);
    } else if (type == "tRNS") {
      trns.assign(c, c + len);
    } else if (type == "IDAT") {
      idat.insert(idat.end(), c, c + len);
    } else if (type == "IEND") {
      break;
    }
    pos += 12 + len;
  }
  if (w <= 0 || h <= 0 || w > 16384 || h > 16384) return err = "bad PNG size", false;
  if (depth != 8 || interlace != 0) return err = "only 8-bit, non-interlaced PNG", false;
  const int chans = ctype == 0 ? 1 : ctype == 2 ? 3 : ctype == 3 ? 1 : ctype == 4 ? 2 : ctype == 6 ? 4 : 0;
  if (!chans) return err = "unsupported PNG colour type", false;
  const size_t stride = (size_t)w * chans;
  std::vector<uint8_t> raw((stride + 1) * h);
  uLongf raw_len = (uLongf)raw.size();
  if (uncompress(raw.data(), &raw_len, idat.data(), (uLong)idat.size()) != Z_OK || raw_len != raw.size())
    return err = "PNG inflate failed", false;
  std::vector<uint8_t> img(stride * h);
  for (int y = 0; y < h; y++) {
    const uint8_t ft = raw[y * (stride + 1)];
    const uint8_t* src = &raw[y * (stride + 1) + 1];
    uint8_t* cur = &img[y * stride];
    const uint8_t* prev = y ? &img[(y - 1) * stride] : nullptr;
    for (size_t i = 0; i < stride; i++) {
      const int a = i >= (size_t)chans ? cur[i - chans] : 0, b = prev ? prev[i] : 0;
      const int cc = (prev && i >= (size_t)chans) ? prev[i - chans] : 0;
      int v = src[i];
      switch (ft) {
        case 0: break;
        case 1: v += a; break;
        case 2: v += b; break;
        case 3: v += (a + b) / 2; break;
        case 4: v += paeth(a, b, cc); break;
        default: return err = "bad PNG filter", false;
      }
      cur[i] = (uint8_t)v;
    }
  }
  rgba.assign((size_t)w * h * 4, 255);
  for (size_t p = 0; p < (size_t)w * h; p++) {
    const uint8_t* s = &img[p * chans];
    uint8_t* o = &rgba[p * 4];
    switch (ctype) {
      case 0: o[0] = o[1] = o[2] = s[0]; break;
      case 4: o[0] = o[1] = o[2] = s[0]; o[3] = s[1]; break;
      case 2: o[0] = s[0]; o[1] = s[1]; o[2] = s[2]; break;
      case 6: std::memcpy(o, s, 4); break;
      case 3:
        if ((size_t)s[0] * 3 + 2 >= plte.size()) return err = "PNG palette index out of range", false;
        o[0] = plte[s[0] * 3]; o[1] = plte[s[0] * 3 + 1]; o[2] = plte[s[0] * 3 + 2];
        if (s[0] < trns.size()) o[3] = trns[s[0]];
        break;
    }
  }
  return true;
}

// binary PPM (P6, maxval 255)
inline bool decode_ppm(const std::vector<uint8_t>& d, int& w, int& h, std::vector<uint8_t>& rgba, std::string& err) {
  std::string head(d.begin(), d.begin() + std::min<size_t>(d.size(), 64));
  std::istringstream in(head);
  std::string magic;
  int maxval = 0;
  in >> magic >> w >> h >> maxval;
  if (magic != "P6" || w <= 0 || h <= 0 || maxval != 255) return err = "only binary PPM with maxval 255", false;
  const size_t off = (size_t)in.tellg() + 1;
  if (off + (size_t)w * h * 3 > d.size()) return err = "truncated PPM", false;
  rgba.assign((size_t)w * h * 4, 255);
  for (size_t p = 0; p < (size_t)w * h; p++) std::memcpy(&rgba[p * 4], &d[off + p * 3], 3);
  return true;
}

// uncompressed TGA, 24 or 32 bits, either row order
inline bool decode_tga(const std::vector<uint8_t>& d, int& w, int& h, std::vector<uint8_t>& rgba, std::string& err) {
  if (d.size() < 18 || d[2] != 2) return err = "only uncompressed true-colour TGA", false;
  w = d[12] | d[13] << 8;
  h = d[14] | d[15] << 8;
  const int bpp = d[16] / 8;
  const bool top = (d[17] & 0x20) != 0;
  const size_t off = 18 + d[0];
  if ((bpp != 3 && bpp != 4) || off + (size_t)w * h * bpp > d.size()) return err = "bad TGA", false;
  rgba.assign((size_t)w * h * 4, 255);
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) {
      const uint8_t* s = &d[off + ((size_t)(top ? y : h - 1 - y) * w + x) * bpp];
      uint8_t* o = &rgba[((size_t)y * w + x) * 4];
      o[0] = s[2]; o[1] = s[1]; o[2] = s[0];
      if (bpp == 4) o[3] = s[3];
    }
  return true;
}

}  // namespace image_detail

// Decode an image file to RGBA8, rows top to bottom.
inline bool load_image_rgba(const std::string& path, int& w, int& h, std::vector<uint8_t>& rgba,
                            std::string* error = nullptr) {
  std::vector<uint8_t> d;
  std::string err;
  bool ok = false;
  if (!image_detail::read_file(path, d)) {
    err = "cannot read " + path;
  } else if (d.size() >= 8 && d[0] == 137 && d[1] == 'P') {
    ok = image_detail::decode_png(d, w, h, rgba, err);
  } else if (d.size() >= 2 && d[0] == 'P' && d[1] == '6') {
    ok = image_detail::decode_ppm(d, w, h, rgba, err);
  } else {
    ok = image_detail::decode_tga(d, w, h, rgba, err);
  }
  if (!ok && error) *error = path + ": " + err;
  return ok;
}

// A square power-of-two edge in 16..2048 for a w x h image, and the image
// resampled to it (nearest texel).
inline int atlas_edge(int w, int h) {
  int e = 16;
  while (e < w || e < h) e *= 2;
  return e > 2048 ? 2048 : e;
}
inline std::vector<uint8_t> resample_square(const std::vector<uint8_t>& rgba, int w, int h, int edge) {
  if (w == edge && h == edge) return rgba;
  std::vector<uint8_t> out((size_t)edge * edge * 4);
  for (int y = 0; y < edge; y++)
    for (int x = 0; x < edge; x++) {
      const int sx = (int)((int64_t)x * w / edge), sy = (int)((int64_t)y * h / edge);
      std::memcpy(&out[((size_t)y * edge + x) * 4], &rgba[((size_t)sy * w + sx) * 4], 4);
    }
  return out;
}

// texture::set_location + load: decode a file into a texture (cached by path
// in the context, as make_new_cached).
inline texture* texture_from_file(texture_context& ctx, std::map<std::string, texture*>& cache,
                                  const std::string& path, std::string* error) {
  auto it = cache.find(path);
  if (it != cache.end()) return it->second;
  int w = 0, h = 0;
  std::vector<uint8_t> px;
  if (!load_image_rgba(path, w, h, px, error)) return nullptr;
  const int edge = atlas_edge(w, h);
  texture* t = ctx.make_new();
  t->set_pixels(edge, resample_square(px, w, h, edge).data());
  cache[path] = t;
  return t;
}

// ---- OBJ / MTL -----------------------------------------------------------------
struct obj_material {
  std::string map_kd;
  float kd[3] = {0, 0, 0};
  bool has_kd = false;
};

inline std::map<std::string, obj_material> parse_mtl(const std::string& path) {
  std::map<std::string, obj_material> mats;
  std::ifstream f(path);
  std::string line, cur;
  while (std::getline(f, line)) {
    std::istringstream in(line);
    std::string key;
    in >> key;
    if (key == "newmtl") {
      in >> cur;
      mats[cur];
    } else if (key == "map_Kd" && !cur.empty()) {
      std::string rest;
      std::getline(in, rest);
      const size_t a = rest.find_first_not_of(" \t"), b = rest.find_last_not_of(" \t\r");
      mats[cur].map_kd = a == std::string::npos ? "" : rest.substr(a, b - a + 1);
    } else if (key == "Kd" && !cur.empty()) {
      obj_material& m = mats[cur];
      in >> m.kd[0] >> m.kd[1] >> m.kd[2];
      m.has_kd = true;
    }
  }
  return mats;
}

// obj_load (obj_load.cpp:181-568): appends one object per usemtl section to c.
// Returns false (with *error set) when the file cannot be read or is malformed.
inline bool obj_load(objects_container* c, texture_context& tex_ctx, const std::string& filename, float scale,
                     std::string* error = nullptr) {
  std::ifstream f(filename);
  if (!f) {
    if (error) *error = filename + " could not be opened";
    return false;
  }
  const size_t slash = filename.find_last_of('/');
  const std::string dir = slash == std::string::npos ? "." : filename.substr(0, slash);
  const size_t dot = filename.find_last_of('.');
  std::map<std::string, obj_material> mats = parse_mtl(filename.substr(0, dot) + ".mtl");
  std::vector<float> v, vt, vn;
  struct Section {
    std::string mtl;
    std::vector<gbr_triangle> tris;
  };
  std::vector<Section> sections(1);
  std::string line;
  auto resolve = [](long i, size_t n) -> long { return i > 0 ? i - 1 : (i < 0 ? (long)n + i : -1); };
  while (std::getline(f, line)) {
    if (line.size() < 2) continue;
    std::istringstream in(line);
    std::string key;
    in >> key;
    if (key == "v") {
      float a = 0, b = 0, cc = 0;
      in >> a >> b >> cc;
      v.insert(v.end(), {a, b, cc});
    } else if (key == "vt") {
      float a = 0, b = 0;
      in >> a >> b;
      vt.insert(vt.end(), {a, b});
    } else if (key == "vn") {
      float a = 0, b = 0, cc = 0;
      in >> a >> b >> cc;
      vn.insert(vn.end(), {a, b, cc});
    } else if (key == "usemtl") {
      std::string name;
      in >> name;
      if (!sections.back().tris.empty() || !sections.back().mtl.empty()) sections.push_back(Section());
      sections.back().mtl = name;
    } else if (key == "f") {
      struct Corner { long v, t, n; };
      std::vector<Corner> poly;
      std::string tok;
      while (in >> tok) {
        Corner k{-1, -1, -1};
        long parts[3] = {0, 0, 0};
        int np = 0;
        size_t s = 0;
        while (np < 3) {
          const size_t e = tok.find('/', s);
          const std::string piece = tok.substr(s, e == std::string::npos ? std::string::npos : e - s);
          parts[np++] = piece.empty() ? 0 : std::strtol(piece.c_str(), nullptr, 10);
          if (e == std::string::npos) break;
          s = e + 1;
        }
        k.v = resolve(parts[0], v.size() / 3);
        k.t = np > 1 ? resolve(parts[1], vt.size() / 2) : -1;
        k.n = np > 2 ? resolve(parts[2], vn.size() / 3) : -1;
        if (k.v < 0 || (size_t)k.v >= v.size() / 3 || (size_t)(k.t + 1) > vt.size() / 2 + 1 ||
            (size_t)(k.n + 1) > vn.size() / 3 + 1) {
          if (error) *error = filename + ": face index out of range: " + line;
          return false;
        }
        poly.push_back(k);
      }
      for (size_t i = 1; i + 1 < poly.size(); i++) {  // fan
        const Corner cs[3] = {poly[0], poly[i], poly[i + 1]};
        gbr_triangle t;
        std::memset(&t, 0, sizeof t);
        float p[3][3];
        for (int k = 0; k < 3; k++)
          for (int a = 0; a < 3; a++) p[k][a] = v[cs[k].v * 3 + a];
        const float e1[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
        const float e2[3] = {p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2]};
        float fnrm[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        const float fl = std::sqrt(fnrm[0] * fnrm[0] + fnrm[1] * fnrm[1] + fnrm[2] * fnrm[2]);
        for (float& x : fnrm) x = fl > 0 ? x / fl : 0.f;
        for (int k = 0; k < 3; k++) {
          gbr_vertex& vx = t.vertices[k];
          for (int a = 0; a < 3; a++) vx.pos[a] = p[k][a] * scale;  // implement scale here (obj_load.cpp:437)
          if (cs[k].t >= 0) { vx.vt[0] = vt[cs[k].t * 2]; vx.vt[1] = vt[cs[k].t * 2 + 1]; }
          for (int a = 0; a < 3; a++) vx.normal[a] = cs[k].n >= 0 ? vn[cs[k].n * 3 + a] : fnrm[a];
        }
        sections.back().tris.push_back(t);
      }
    }
  }
  std::map<std::string, texture*> cache;
  for (const Section& sec : sections) {
    if (sec.tris.empty()) continue;
    texture* tex = nullptr;
    const auto m = mats.find(sec.mtl);
    if (m != mats.end() && !m->second.map_kd.empty()) tex = texture_from_file(tex_ctx, cache, dir + "/" + m->second.map_kd, error);
    if (!tex) {
      // the material's Kd as a 32x32 texture, else magenta (obj_load.cpp:508-540)
      const bool kd = m != mats.end() && m->second.has_kd;
      const std::string key = kd ? "kd:" + std::to_string(m->second.kd[0]) + "," + std::to_string(m->second.kd[1]) +
                                       "," + std::to_string(m->second.kd[2])
                                 : "kd:magenta";
      auto it = cache.find(key);
      if (it != cache.end()) {
        tex = it->second;
      } else {
        tex = tex_ctx.make_new();
        if (kd)
          tex->set_create_colour((uint8_t)(m->second.kd[0] * 255.f), (uint8_t)(m->second.kd[1] * 255.f),
                                 (uint8_t)(m->second.kd[2] * 255.f), 255, 32);
        else
          tex->set_create_colour(255, 0, 255, 255, 32);
        cache[key] = tex;
      }
    }
    c->add_object(sec.tris, tex);
  }
  return true;
}

// Let object_context::load_active load objects_container::set_file files.
inline void install_obj_loader(object_context& ctx) {
  ctx.file_loader = [](objects_container* c, texture_context& t, const std::string& f, float s, std::string* e) {
    return obj_load(c, t, f, s, e);
  };
}

}  // namespace openclrenderer

#endif  // GBR_OBJ_HPP
