// obj_shim.hpp — TEST INFRASTRUCTURE ONLY: the engine classes that the
// reference's OBJ loader (obj_load.cpp:1-568, extracted by obj_build.py)
// touches, reduced to the members it reads and writes, so that the loader
// compiles on the host from its own source as the parity pin of
// include/gbr_obj.hpp.  The reference's triangle.hpp, vertex.hpp, vec.hpp and
// util.hpp compile unchanged (with objinc/ standing in for <cl/cl.h> and the
// unvendored <vec/vec.hpp>); what lives in files that need SFML, OpenCL or the
// rest of the engine is restated here, each item citing what it follows:
//   vertex accessors       vertex.cpp:134-153, 170-203 (plain stores and loads)
//   texture                texture.hpp / texture.cpp:25-45, 128-146 (location,
//                          cache name, the colour a blank texture is made of)
//   texture_context        texture_context.cpp:16-49 (make_new, make_new_cached)
//   col2cachename          texture.cpp:9-12
//   object, objects_container, object_context: the fields obj_load sets
//   lg::log, sf::Clock, sf::Color: no-ops / a plain RGBA byte colour
// No texture is decoded: the harness reports where each texture comes from.
#pragma once

#include <cassert>
#include <cstdint>
#include <cstdlib>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include <cl/cl.h>
#include <vec/vec.hpp>

#include "triangle.hpp"  // util.hpp has no include guard: the loader source includes it
#include "vec.hpp"

inline cl_float4 vertex::get_pos() const { return pos; }
inline cl_float4 vertex::get_normal() const { return normal; }
inline cl_float2 vertex::get_vt() const { return vt; }
inline void vertex::set_pos(cl_float4 val) { pos = val; }
inline void vertex::set_normal(cl_float4 val) { normal = val; }
inline void vertex::set_vt(cl_float2 vtm) { vt = vtm; }

namespace lg {
template <typename... T>
inline void log(T&&...) {}
}  // namespace lg

namespace sf {
struct Clock {};
struct Color {
  uint8_t r, g, b, a;
  Color(uint8_t r_, uint8_t g_, uint8_t b_, uint8_t a_ = 255) : r(r_), g(g_), b(b_), a(a_) {}
};
}  // namespace sf

struct texture {
  int id = -1;
  int type = 0;
  bool is_unique = false;
  bool cacheable = true;
  std::string texture_location;
  std::string cache_name;
  bool blank = false;  // set_create_colour was called: a w x h texture of colour
  uint8_t colour[4] = {0, 0, 0, 0};
  int w = 0, h = 0;
  void set_location(const std::string& loc) { texture_location = loc; }
  void set_cache_name(const std::string& name) { cache_name = name; }
  void set_create_colour(sf::Color col, int w_, int h_) {
    blank = true;
    colour[0] = col.r;
    colour[1] = col.g;
    colour[2] = col.b;
    colour[3] = col.a;
    w = w_;
    h = h_;
  }
};

struct texture_context {
  std::vector<std::unique_ptr<texture>> all_textures;
  int gid = 0;
  texture* make_new() {
    all_textures.emplace_back(new texture());
    all_textures.back()->id = gid++;
    return all_textures.back().get();
  }
  texture* make_new_cached(const std::string& loc) {
    for (auto& i : all_textures)
      if (i->cacheable && !i->is_unique && i->texture_location == loc) return i.get();
    texture* tex = make_new();
    tex->set_location(loc);
    tex->set_cache_name(loc);
    return tex;
  }
};

inline std::string col2cachename(const vec4f& col) {
  return std::string("CACHE") + std::to_string(col.x()) + std::to_string(col.y()) + std::to_string(col.z()) +
         std::to_string(col.w());
}

struct object {
  std::string object_name;
  std::vector<triangle> tri_list;
  int tri_num = 0;
  cl_uint tid = 0, bid = 0, rid = 0;
  cl_uint has_bump = 0;
  cl_float4 pos = {{0.f}}, rot = {{0.f}};
  int isloaded = 0;
};

struct object_context {
  texture_context tex_ctx;
};

struct objects_container {
  object_context* parent = nullptr;
  cl_uint id = 0;
  std::string file;
  std::string normal_map;
  cl_float4 pos = {{0.f}}, rot = {{0.f}};
  float current_scale = 1.f;
  float requested_scale = 1.f;
  bool textures_are_unique = false;
  bool isloaded = false;
  std::vector<object> objs;
};
