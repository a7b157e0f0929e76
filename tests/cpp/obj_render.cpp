// obj_render.cpp — test driver for include/gbr_obj.hpp: loads an OBJ scene
// through objects_container::set_file + object_context::load_active, renders
// the reference's frame through the engine-shaped API and writes depth, id,
// RGBA8, the loaded triangles and the decoded textures.
//
// params file (little endian): f32 cam[8], i32 width, i32 height, f32 hfov,
// u32 use_linear, f32 clear[4], f32 scale, u32 n_lights, n_lights 64-byte lights.
// out file: depth, id, rgba planes (W*H*4 bytes each), u32 ntris, ntris
// triangles, u32 ntex, per texture i32 edge + edge*edge*4 bytes.  With
// --load-only (no GPU needed) the planes are left out.
#include <cstdio>
#include <cstring>
#include <vector>

#include "gbr_obj.hpp"

using namespace openclrenderer;

// the loaded triangles (object ids as build() assigns them) and textures
static void write_scene(FILE* o, object_context& ctx, objects_container* c) {
  uint32_t nt = 0;
  for (const object& ob : c->objs) nt += (uint32_t)ob.tri_list.size();
  fwrite(&nt, 4, 1, o);
  uint32_t oid = 0;
  for (const object& ob : c->objs) {
    for (gbr_triangle t : ob.tri_list) {
      t.vertices[0].object_id = oid;
      fwrite(&t, sizeof t, 1, o);
    }
    oid++;
  }
  const uint32_t ntex = (uint32_t)ctx.tex_ctx.textures.size();
  fwrite(&ntex, 4, 1, o);
  for (const auto& t : ctx.tex_ctx.textures) {
    fwrite(&t->size, 4, 1, o);
    fwrite(t->rgba.data(), 1, t->rgba.size(), o);
  }
}

int main(int argc, char** argv) {
  const bool load_only = argc == 5 && std::strcmp(argv[4], "--load-only") == 0;
  if (argc != 4 && !load_only) {
    fprintf(stderr, "usage: %s scene.obj params.bin out.bin [--load-only]\n", argv[0]);
    return 2;
  }
  FILE* f = fopen(argv[2], "rb");
  if (!f) return 2;
  float cam[8], hfov, clear[4], scale;
  int32_t W, H;
  uint32_t use_linear, nl;
  if (fread(cam, 4, 8, f) != 8 || fread(&W, 4, 1, f) != 1 || fread(&H, 4, 1, f) != 1 || fread(&hfov, 4, 1, f) != 1 ||
      fread(&use_linear, 4, 1, f) != 1 || fread(clear, 4, 4, f) != 4 || fread(&scale, 4, 1, f) != 1 ||
      fread(&nl, 4, 1, f) != 1)
    return 3;
  std::vector<gbr_light> ls(nl);
  if (nl && fread(ls.data(), sizeof(gbr_light), nl, f) != nl) return 3;
  fclose(f);

  object_context ctx;
  install_obj_loader(ctx);
  objects_container* c = ctx.make_new();
  c->set_file(argv[1]);
  c->request_scale(scale);
  c->set_active(true);
  if (ctx.load_active() != GBR_OK) {
    fprintf(stderr, "load: %s\n", ctx.load_error.c_str());
    return 4;
  }
  c->set_two_sided(true);
  if (load_only) {
    FILE* o = fopen(argv[3], "wb");
    if (!o) return 7;
    write_scene(o, ctx, c);
    fclose(o);
    return 0;
  }
  ctx.set_clear_colour(float4{clear[0], clear[1], clear[2], clear[3]});
  ctx.set_use_linear_rendering(use_linear);
  if (ctx.build(true) != GBR_OK) {
    fprintf(stderr, "build: %s\n", gbr_last_error_string());
    return 5;
  }
  for (const gbr_light& g : ls) {
    light l;
    l.set_pos(float4{g.pos[0], g.pos[1], g.pos[2], 0});
    l.set_col(float4{g.col[0], g.col[1], g.col[2], 0});
    l.set_shadow_casting(g.shadow);
    l.set_brightness(g.brightness);
    l.set_radius(g.radius);
    light::add_light(&l);
  }
  light_gpu lights = light::build();
  engine window;
  window.load(W, H);
  window.set_fov(hfov);
  window.set_camera_pos(float4{cam[0], cam[1], cam[2], cam[3]});
  window.set_camera_rot(float4{cam[4], cam[5], cam[6], cam[7]});
  window.set_light_data(lights);
  if (window.set_object_data(*ctx.fetch()) != GBR_OK || window.generate_realtime_shadowing(*ctx.fetch()) != GBR_OK ||
      window.draw_bulk_objs_n(*ctx.fetch()) != GBR_OK) {
    fprintf(stderr, "frame: %s\n", gbr_last_error_string());
    return 6;
  }
  FILE* o = fopen(argv[3], "wb");
  if (!o) return 7;
  std::vector<uint8_t> plane;
  for (int which = 0; which < 3; which++) {
    if (ctx.fetch()->read_plane(which, plane) != GBR_OK) return 8;
    fwrite(plane.data(), 1, plane.size(), o);
  }
  write_scene(o, ctx, c);
  fclose(o);
  printf("ok %zu objects, %zu textures\n", c->objs.size(), ctx.tex_ctx.textures.size());
  return 0;
}
