// gbr_obj.hpp — scene ingest for the C++ API of gbr_engine.hpp: Wavefront
// OBJ + MTL geometry and material loading in the manner of the reference's
// obj_load (obj_load.cpp:181-568), and RGBA8 image decoding for textures
// (PNG through zlib, binary PPM, uncompressed TGA) in place of the
// reference's SFML image loader (texture.cpp:323-358).
//
// obj_load follows the reference's parsing and material rules as they are
// written (the comment above it lists them), so that on the files the
// reference accepts it yields the same objects, triangles and texture choices;
// it also reads polygons, relative indices and faces without vt or vn.
// Textures must be square powers of two from 16 to 2048 in the atlas; other
// images are resampled (nearest texel) to the next power of two in that range.
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

// texture::set_location + load: decode the image file at path into t, made
// square for the atlas.
inline bool texture_load_file(texture* t, const std::string& path, std::string* error) {
  int w = 0, h = 0;
  std::vector<uint8_t> px;
  if (!load_image_rgba(path, w, h, px, error)) return false;
  const int edge = atlas_edge(w, h);
  t->set_pixels(edge, resample_square(px, w, h, edge).data());
  t->set_location(path);
  return true;
}

// The context's texture for an image file: make_new_cached(cache_name) (a new
// texture when unique), located at path and decoded unless it already holds
// that file's pixels (obj_load.cpp:452-460).  A new texture that cannot be
// decoded is removed again and nullptr returned.
inline texture* texture_file(texture_context& ctx, const std::string& cache_name, const std::string& path, bool unique,
                             std::string* error) {
  bool fresh = true;
  texture* t = unique ? ctx.make_new() : ctx.make_new_cached(cache_name, &fresh);
  if (fresh || t->rgba.empty() || t->location != path) {
    if (!texture_load_file(t, path, error)) {
      if (fresh) ctx.destroy(t);
      return nullptr;
    }
  }
  return t;
}

// ---- OBJ / MTL -----------------------------------------------------------------
// The rules of the reference's loader, stated on their own (obj_load.cpp:18-168).
namespace obj_detail {

inline bool read_lines(const std::string& path, std::vector<std::string>& out) {
  std::ifstream f(path);
  if (!f.is_open()) return false;
  std::string line;
  while (std::getline(f, line)) out.push_back(line);
  return true;
}

inline bool file_exists(const std::string& path) { return std::ifstream(path).good(); }

// get_file_name (util.hpp:23-28): the text after the last '/' or '\'
inline std::string file_name(const std::string& path) { return path.substr(path.find_last_of("/\\") + 1); }

// is_samemtl (obj_load.cpp:26-29): a "newmtl " line whose text after its last
// space begins with name
inline bool is_samemtl(const std::string& line, const std::string& name) {
  return line.compare(0, 7, "newmtl ") == 0 && line.compare(line.find_last_of(' ') + 1, name.size(), name) == 0;
}

// retrieve_diffuse_new (obj_load.cpp:32-50): the text after the last space of
// the first "map_Kd " line at or after the material's newmtl line (the search
// runs on into later materials), else ""
inline std::string diffuse_name(const std::vector<std::string>& mtl, const std::string& name) {
  bool found = false;
  for (const std::string& l : mtl) {
    found = found || is_samemtl(l, name);
    if (found && l.compare(0, 7, "map_Kd ") == 0) return l.substr(l.find_last_of(' ') + 1);
  }
  return "";
}

// retrieve_bumpmap (obj_load.cpp:53-79): the material's own "map_Bump " file,
// else "None"
inline std::string bumpmap_name(const std::vector<std::string>& mtl, const std::string& name) {
  bool found = false;
  for (const std::string& l : mtl) {
    if (is_samemtl(l, name)) {
      found = true;
      continue;
    }
    if (found && l.compare(0, 9, "map_Bump ") == 0) return l.substr(l.find_last_of(' ') + 1);
    if (found && l.compare(0, 7, "newmtl ") == 0) return "None";
  }
  return "None";
}

// split (util.hpp:4-20): fields between single spaces, a trailing empty field dropped
inline std::vector<std::string> split_spaces(const std::string& s) {
  std::vector<std::string> out;
  size_t a = 0;
  while (a < s.size()) {
    const size_t b = s.find(' ', a);
    out.push_back(s.substr(a, b == std::string::npos ? std::string::npos : b - a));
    if (b == std::string::npos) break;
    a = b + 1;
  }
  return out;
}

// get_Kd (obj_load.cpp:83-116): the first line beginning "Kd" at or after the
// material's newmtl line, its fields 1-3 read as doubles rounded to float
inline bool get_kd(const std::vector<std::string>& mtl, const std::string& name, float kd[3]) {
  bool found = false;
  for (const std::string& l : mtl) {
    if (is_samemtl(l, name)) {
      found = true;
      continue;
    }
    if (!found || l.compare(0, 2, "Kd") != 0) continue;
    const std::vector<std::string> f = split_spaces(l);
    if (f.size() < 4) return false;
    for (int k = 0; k < 3; k++) kd[k] = (float)std::strtod(f[k + 1].c_str(), nullptr);
    return true;
  }
  return false;
}

// decompose_attribute (obj_load.cpp:121-141): n values, each read from just
// after the line's next space; the whole line as integers when it has no '.',
// else as doubles rounded to float.  (A missing space wraps the position to
// the start of the line, as the reference's int arithmetic does.)
inline void attributes(const std::string& s, float* out, int n) {
  const bool real = s.find('.') != std::string::npos;
  size_t p = s.find(' ');
  for (int i = 0; i < n; i++) {
    const char* t = s.c_str() + (p + 1);
    out[i] = real ? (float)std::strtod(t, nullptr) : (float)std::atoi(t);
    p = s.find(' ', p + 1);
  }
}

// col2cachename (texture.cpp:9-12): the cache name of a colour texture
inline std::string colour_cache_name(float r, float g, float b, float a) {
  return "CACHE" + std::to_string(r) + std::to_string(g) + std::to_string(b) + std::to_string(a);
}

// float to sf::Uint8 as the reference's sf::Color(float, ...) converts it
inline uint8_t colour_byte(float x) { return (uint8_t)(int32_t)x; }

}  // namespace obj_detail

// obj_load (obj_load.cpp:181-568): appends one object per usemtl section to c
// and returns true; false (with *error set) when the file cannot be opened, a
// face index is out of range or an image cannot be decoded.
//
// The reference's rules, as it states them (on the files it accepts, with
// triangulated v/vt/vn faces and positive indices, the result is the same):
// lines classified by their first characters ("f ", "v ", "vt ", "vn ", "use",
// "g "); attribute values as decompose_attribute reads them; face indices
// resolved after the whole file is read; objects only for usemtl sections
// (faces before the first usemtl belong to none), empty ones included, named
// by the section's group when there are as many "g " lines as usemtl lines;
// the diffuse texture is the material's map_Kd file (dir/name, else
// dir/basename), else a 32x32 texture of Kd*255 (cached by colour), else a new
// magenta 32x32 texture; a map_Bump file becomes the object's bump texture
// (descriptor has_bump) and the container's set_normal file its normal map,
// both cached by path; positions x requested_scale, vt and vn as written.
// Beyond the reference: polygons become fans, relative (negative) indices
// resolve against the counts so far, faces without vt get (0, 0) and faces
// without vn the face normal.
inline bool obj_load(objects_container* c, texture_context& tex_ctx, const std::string& filename, float scale,
                     std::string* error = nullptr) {
  std::vector<std::string> lines, mtl;
  if (!obj_detail::read_lines(filename, lines)) {
    if (error) *error = filename + " could not be opened";
    return false;
  }
  obj_detail::read_lines(filename.substr(0, filename.find_last_of('.')) + ".mtl", mtl);  // none: no materials
  const size_t slash = filename.find_last_of('/');
  const std::string dir = slash == std::string::npos ? "." : filename.substr(0, slash);

  struct Corner {
    long v, t, n;  // 0-based; -1 = absent (t, n)
  };
  struct Tri {
    Corner k[3];
  };
  std::vector<float> v, vt, vn;
  std::vector<Tri> faces;
  std::vector<size_t> use_pos;
  std::vector<std::string> use_name, group_name;
  for (const std::string& ln : lines) {
    const auto at = [&](size_t i) { return i < ln.size() ? ln[i] : '\0'; };
    if (at(0) == 'f' && at(1) == ' ') {
      std::istringstream in(ln.substr(2));
      std::vector<Corner> poly;
      std::string tok;
      // 1-based, or negative = relative to the elements read so far, 0 = absent
      const auto idx = [](long i, size_t n) -> long { return i > 0 ? i - 1 : (i < 0 ? (long)n + i : -1); };
      while (in >> tok) {
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
        Corner k;
        k.v = parts[0] ? idx(parts[0], v.size() / 3) : -2;
        k.t = np > 1 ? idx(parts[1], vt.size() / 2) : -1;
        k.n = np > 2 ? idx(parts[2], vn.size() / 3) : -1;
        poly.push_back(k);
      }
      for (size_t i = 1; i + 1 < poly.size(); i++) faces.push_back(Tri{{poly[0], poly[i], poly[i + 1]}});
    } else if (at(0) == 'v' && at(1) == ' ') {
      float a[3];
      obj_detail::attributes(ln, a, 3);
      v.insert(v.end(), a, a + 3);
    } else if (at(0) == 'v' && at(1) == 't' && at(2) == ' ') {
      float a[2];
      obj_detail::attributes(ln, a, 2);
      vt.insert(vt.end(), a, a + 2);
    } else if (at(0) == 'v' && at(1) == 'n' && at(2) == ' ') {
      float a[3];
      obj_detail::attributes(ln, a, 3);
      vn.insert(vn.end(), a, a + 3);
    } else if (at(0) == 'u' && at(1) == 's' && at(2) == 'e') {
      use_pos.push_back(faces.size());
      use_name.push_back(ln.substr(ln.find_last_of(' ') + 1));
    } else if (at(0) == 'g' && at(1) == ' ') {
      group_name.push_back(ln.substr(ln.find_last_of(' ') + 1));
    }
  }

  // resolve: positions x scale (w = 0 x scale, as mult), vt and vn as written
  const size_t nv = v.size() / 3, nvt = vt.size() / 2, nvn = vn.size() / 3;
  std::vector<gbr_triangle> tris(faces.size());
  for (size_t f = 0; f < faces.size(); f++) {
    const Corner* cs = faces[f].k;
    for (int k = 0; k < 3; k++)
      if (cs[k].v < 0 || (size_t)cs[k].v >= nv || cs[k].t < -1 || cs[k].t >= (long)nvt || cs[k].n < -1 ||
          cs[k].n >= (long)nvn) {
        if (error) *error = filename + ": face index out of range in face " + std::to_string(f + 1);
        return false;
      }
    gbr_triangle& t = tris[f];
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
      vx.pos[3] = 0.f * scale;
      if (cs[k].t >= 0) { vx.vt[0] = vt[cs[k].t * 2]; vx.vt[1] = vt[cs[k].t * 2 + 1]; }
      for (int a = 0; a < 3; a++) vx.normal[a] = cs[k].n >= 0 ? vn[cs[k].n * 3 + a] : fnrm[a];
    }
  }

  // one object per usemtl section, with its textures
  use_pos.push_back(tris.size());
  const bool using_groups = use_name.size() == group_name.size();
  const bool unique = c->textures_are_unique;
  for (size_t i = 0; i + 1 < use_pos.size(); i++) {
    const std::string tex_name = obj_detail::diffuse_name(mtl, use_name[i]);
    const std::string bump_name = obj_detail::bumpmap_name(mtl, use_name[i]);
    std::string full = dir + "/" + tex_name;
    const std::string cache_name = full;
    bool exists = obj_detail::file_exists(full);
    if (!exists && !tex_name.empty()) {
      full = dir + "/" + obj_detail::file_name(tex_name);
      exists = obj_detail::file_exists(full);
    }
    texture* tex = nullptr;
    float kd[3];
    if (!tex_name.empty() && exists) {
      if (!(tex = texture_file(tex_ctx, cache_name, full, unique, error))) return false;
    } else if (obj_detail::get_kd(mtl, use_name[i], kd)) {
      const float r = kd[0] * 255.f, g = kd[1] * 255.f, b = kd[2] * 255.f;
      tex = unique ? tex_ctx.make_new() : tex_ctx.make_new_cached(obj_detail::colour_cache_name(r, g, b, 255.f));
      tex->set_create_colour(obj_detail::colour_byte(r), obj_detail::colour_byte(g), obj_detail::colour_byte(b), 255,
                             32);
    } else {
      tex = tex_ctx.make_new();
      tex->set_create_colour(255, 0, 255, 255, 32);
    }
    texture* bump = nullptr;
    if (bump_name != "None") {
      const std::string bump_full = dir + "/" + bump_name;
      if (!(bump = texture_file(tex_ctx, bump_full, bump_full, false, error))) return false;
    }
    texture* normal = nullptr;
    if (!c->normal_map_file.empty() &&
        !(normal = texture_file(tex_ctx, c->normal_map_file, c->normal_map_file, false, error)))
      return false;
    c->add_object(std::vector<gbr_triangle>(tris.begin() + use_pos[i], tris.begin() + use_pos[i + 1]), tex);
    object& o = c->objs.back();
    o.object_name = using_groups ? group_name[i] : "";
    o.bump = bump;
    o.has_bump = bump != nullptr;
    o.normal_map = normal;
  }
  c->current_scale = scale;
  c->requested_scale = 1.f;
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
