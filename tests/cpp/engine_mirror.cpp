// engine_mirror.cpp — test driver for include/gbr_engine.hpp: builds a scene
// from a binary scene file through the OpenCLRenderer-shaped C++ API
// (object_context, objects_container, texture_context, light, engine), runs
// the reference's frame (generate_realtime_shadowing + draw_bulk_objs_n) and
// writes depth, id and RGBA8 to an output file.
//
// Scene file (little endian): "GBRS", u32 n_objects, u32 n_textures,
// u32 n_lights, f32 cam[8], i32 width, i32 height, f32 hfov, u32 use_linear,
// f32 clear[4]; textures: i32 edge + edge*edge*4 bytes; objects: f32 pos[4],
// f32 quat[4], f32 scale, specular, spec_mult, diffuse, i32 feature_flag,
// i32 texture, u32 ntris, ntris * 144-byte triangles; lights: 64-byte lights.
//
// Optional third argument: "aa" runs engine::do_pseudo_aa after the frame;
// "mb" draws a first frame from a camera moved by (6, -4, 15) and turned by
// (0.012, -0.02, 0.005), swaps buffers, draws the frame from the scene's camera
// and runs engine::do_motion_blur(0.75, 0.6); "ssr" runs
// engine::draw_screenspace_reflections after the frame; "blend other.bin"
// loads a second context, draws it (its lights join the list, as the
// reference's light list is global) from its own camera and renders this one
// with object_context::set_blend_render_context(other).
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gbr_engine.hpp"

using namespace openclrenderer;

template <class T>
static bool rd(FILE* f, T* v, size_t n = 1) { return fread(v, sizeof(T), n, f) == n; }

struct Header {
  uint32_t nobj = 0, ntex = 0, nl = 0, use_linear = 1;
  float cam[8], hfov = 90.f, clear[4];
  int32_t W = 0, H = 0;
};

// Reads a scene file into ctx (objects, textures) and the global light list.
static int load(const char* path, object_context& ctx, Header& h) {
  FILE* f = fopen(path, "rb");
  if (!f) return 2;
  char magic[4];
  if (!rd(f, magic, 4) || memcmp(magic, "GBRS", 4) || !rd(f, &h.nobj) || !rd(f, &h.ntex) || !rd(f, &h.nl) ||
      !rd(f, h.cam, 8) || !rd(f, &h.W) || !rd(f, &h.H) || !rd(f, &h.hfov) || !rd(f, &h.use_linear) ||
      !rd(f, h.clear, 4))
    return 3;
  std::vector<texture*> texs;
  for (uint32_t i = 0; i < h.ntex; i++) {
    int32_t edge = 0;
    if (!rd(f, &edge)) return 3;
    std::vector<uint8_t> px((size_t)edge * edge * 4);
    if (!rd(f, px.data(), px.size())) return 3;
    texture* t = ctx.tex_ctx.make_new();
    t->set_pixels(edge, px.data());
    texs.push_back(t);
  }
  for (uint32_t i = 0; i < h.nobj; i++) {
    float pos[4], quat[4], scale, spec, spec_mult, diffuse;
    int32_t ff, tex;
    uint32_t nt;
    if (!rd(f, pos, 4) || !rd(f, quat, 4) || !rd(f, &scale) || !rd(f, &spec) || !rd(f, &spec_mult) ||
        !rd(f, &diffuse) || !rd(f, &ff) || !rd(f, &tex) || !rd(f, &nt))
      return 3;
    std::vector<gbr_triangle> tris(nt);
    if (nt && !rd(f, tris.data(), nt)) return 3;
    objects_container* c = ctx.make_new();
    c->add_object(tris, tex >= 0 ? texs[tex] : nullptr);
    c->set_pos(float4{pos[0], pos[1], pos[2], pos[3]});
    c->set_rot_quat(float4{quat[0], quat[1], quat[2], quat[3]});
    c->set_dynamic_scale(scale);
    c->set_specular(spec);
    c->set_spec_mult(spec_mult);
    c->set_diffuse(diffuse);
    c->set_two_sided((ff & FLAG_TWO_SIDED) != 0);
    c->set_is_static((ff & FLAG_IS_STATIC) != 0);
    c->set_does_not_receive_dynamic_shadows((ff & FLAG_NO_DYN_SHADOWS) != 0);
    c->set_ss_reflective((ff & FLAG_SS_REFLECTIVE) != 0);
    // an object that reflects, with a texture, uses that texture as its reflection map
    if ((ff & FLAG_SS_REFLECTIVE) && tex >= 0 && (i % 2)) c->set_screenspace_map_id(texs[tex]);
    c->set_active(true);
  }
  for (uint32_t i = 0; i < h.nl; i++) {
    gbr_light g;
    if (!rd(f, &g)) return 3;
    light l;
    l.set_pos(float4{g.pos[0], g.pos[1], g.pos[2], g.pos[3]});
    l.set_col(float4{g.col[0], g.col[1], g.col[2], g.col[3]});
    l.set_shadow_casting(g.shadow);
    l.set_brightness(g.brightness);
    l.set_radius(g.radius);
    l.set_diffuse(g.diffuse);
    l.set_godray_intensity(g.godray_intensity);
    l.set_is_static(g.is_static != 0);
    light::add_light(&l);
  }
  fclose(f);
  ctx.load_active();
  ctx.set_clear_colour(float4{h.clear[0], h.clear[1], h.clear[2], h.clear[3]});
  ctx.set_use_linear_rendering(h.use_linear);
  if (ctx.build(true) != GBR_OK) {
    fprintf(stderr, "build: %s\n", gbr_last_error_string());
    return 4;
  }
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 3 || argc > 5) {
    fprintf(stderr, "usage: %s scene.bin out.bin [aa|mb|ssr|blend other.bin]\n", argv[0]);
    return 2;
  }
  const std::string mode = argc >= 4 ? argv[3] : "";
  object_context ctx;
  Header h;
  if (int e = load(argv[1], ctx, h)) return e;
  const float* cam = h.cam;
  const int32_t W = h.W, H = h.H;
  const float hfov = h.hfov;
  // "blend": a second context, drawn first from its own camera, blended into this one
  object_context other;
  Header oh;
  if (mode == "blend") {
    if (argc != 5) return 2;
    if (int e = load(argv[4], other, oh)) return e;
    ctx.set_blend_render_context(other);
  }
  light_gpu lights = light::build();
  engine window;
  window.load(W, H);
  window.set_fov(hfov);
  window.set_camera_pos(float4{cam[0], cam[1], cam[2], cam[3]});
  window.set_camera_rot(float4{cam[4], cam[5], cam[6], cam[7]});
  window.set_light_data(lights);
  if (mode == "blend") {
    window.set_camera_pos(float4{oh.cam[0], oh.cam[1], oh.cam[2], oh.cam[3]});
    window.set_camera_rot(float4{oh.cam[4], oh.cam[5], oh.cam[6], oh.cam[7]});
    if (window.set_object_data(*other.fetch()) != GBR_OK || window.draw_bulk_objs_n(*other.fetch()) != GBR_OK) {
      fprintf(stderr, "blend context: %s\n", gbr_last_error_string());
      return 5;
    }
    window.set_camera_pos(float4{cam[0], cam[1], cam[2], cam[3]});
    window.set_camera_rot(float4{cam[4], cam[5], cam[6], cam[7]});
  }
  if (mode == "mb") {  // the previous frame
    window.set_camera_pos(float4{cam[0] + 6.f, cam[1] - 4.f, cam[2] + 15.f, cam[3]});
    window.set_camera_rot(float4{cam[4] + 0.012f, cam[5] - 0.02f, cam[6] + 0.005f, cam[7]});
    if (window.set_object_data(*ctx.fetch()) != GBR_OK || window.draw_bulk_objs_n(*ctx.fetch()) != GBR_OK) {
      fprintf(stderr, "frame 1: %s\n", gbr_last_error_string());
      return 5;
    }
    ctx.fetch()->swap_buffers();
    window.set_camera_pos(float4{cam[0], cam[1], cam[2], cam[3]});
    window.set_camera_rot(float4{cam[4], cam[5], cam[6], cam[7]});
  }
  if (window.set_object_data(*ctx.fetch()) != GBR_OK ||
      window.generate_realtime_shadowing(*ctx.fetch()) != GBR_OK ||
      window.draw_bulk_objs_n(*ctx.fetch()) != GBR_OK || window.draw_godrays(*ctx.fetch()) != GBR_OK) {
    fprintf(stderr, "frame: %s\n", gbr_last_error_string());
    return 5;
  }
  if ((mode == "aa" && window.do_pseudo_aa() != GBR_OK) ||
      (mode == "mb" && window.do_motion_blur(*ctx.fetch(), 0.75f, 0.6f) != GBR_OK) ||
      (mode == "ssr" && window.draw_screenspace_reflections(*ctx.fetch()) != GBR_OK)) {
    fprintf(stderr, "post: %s\n", gbr_last_error_string());
    return 5;
  }
  FILE* o = fopen(argv[2], "wb");
  if (!o) return 6;
  std::vector<uint8_t> plane;
  for (int which = 0; which < 3; which++) {
    if (ctx.fetch()->read_plane(which, plane) != GBR_OK) {
      fprintf(stderr, "read: %s\n", gbr_last_error_string());
      return 7;
    }
    fwrite(plane.data(), 1, plane.size(), o);
  }
  fclose(o);
  printf("ok %d x %d, %u triangles, %u objects, %zu lights\n", W, H, ctx.fetch()->tri_num, ctx.fetch()->obj_num,
         lights.lights.size());
  return 0;
}
