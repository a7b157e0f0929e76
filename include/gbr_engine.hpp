// gbr_engine.hpp — C++ host API of the triangle path in the shape of
// OpenCLRenderer's own classes, over the C ABI of gbr.h.
//
// The reference drives the path through object_context / objects_container /
// texture_context / light / engine (main.cpp:60-262).  These classes keep those
// names, the call sequence and the argument meaning, so a caller of the
// reference changes includes and little else:
//
//   object_context ctx;                        object_context.hpp:187
//   objects_container* c = ctx.make_new();     object_context.cpp (make_new)
//   c->add_object(tris, tex); c->set_pos(p);   objects_container.hpp:64-115
//   c->set_active(true); ctx.build(true);      object_context.cpp:646-797
//   light l; l.set_pos(...); light::add_light(&l);
//   light_gpu lights = light::build();         light.cpp:145-276
//   engine w; w.load(1920, 1080);              engine.cpp:290
//   w.set_object_data(*ctx.fetch()); w.set_light_data(lights);
//   w.generate_realtime_shadowing(*ctx.fetch());   engine.cpp:1601
//   w.draw_bulk_objs_n(*ctx.fetch());              engine.cpp:1794 (render_tris)
//
// Differences, all on the host side: geometry comes as triangle arrays or, with
// gbr_obj.hpp, as OBJ files through set_file + load_active; textures as RGBA8
// pixel arrays or image files; object rotation as a quaternion; errors as
// gbr_status (never exit); and the screen is a device framebuffer
// (gbr_framebuffer) instead of a GL surface.  Header-only; link with libgbr.so.
#ifndef GBR_ENGINE_HPP
#define GBR_ENGINE_HPP

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <string>
#include <vector>

#include "gbr.h"

namespace openclrenderer {

struct float4 {
  float x = 0, y = 0, z = 0, w = 0;
};

// feature_flag bits of obj_g_descriptor (cl2.cl:90-97)
enum : int32_t {
  FLAG_SS_REFLECTIVE = 1,
  FLAG_TWO_SIDED = 2,
  FLAG_OUTLINE = 4,
  FLAG_IS_STATIC = 8,
  FLAG_NO_DYN_SHADOWS = 16
};

// ---- textures (texture_context.hpp:39-71) ---------------------------------------
struct texture {
  int id = -1;                 // position in the gpu texture order
  int size = 0;                // square edge, power of two 16..2048
  std::vector<uint8_t> rgba;   // size*size*4
  std::string location;        // texture::set_location: the file (or cache name) it came from
  bool is_unique = false;      // texture::set_unique: never returned by make_new_cached
  void set_location(const std::string& loc) { location = loc; }
  void set_unique() { is_unique = true; }
  // texture::set_create_colour: a uniform square texture
  void set_create_colour(uint8_t r, uint8_t g, uint8_t b, uint8_t a, int edge) {
    size = edge;
    rgba.assign((size_t)edge * edge * 4, 0);
    for (size_t i = 0; i < (size_t)edge * edge; i++) {
      rgba[i * 4] = r; rgba[i * 4 + 1] = g; rgba[i * 4 + 2] = b; rgba[i * 4 + 3] = a;
    }
  }
  // the decoded pixels of an image (what texture::load_from_file would produce)
  void set_pixels(int edge, const uint8_t* px) {
    size = edge;
    rgba.assign(px, px + (size_t)edge * edge * 4);
  }
};

struct texture_context {
  std::vector<std::unique_ptr<texture>> textures;
  texture* make_new() {
    textures.emplace_back(new texture());
    textures.back()->id = (int)textures.size() - 1;
    return textures.back().get();
  }
  // texture_context::make_new_cached (texture_context.cpp:27-49): the first
  // texture of the context at location loc that is not unique, else a new one
  // at loc (*fresh tells which).
  texture* make_new_cached(const std::string& loc, bool* fresh = nullptr) {
    for (const auto& t : textures)
      if (!t->is_unique && t->location == loc) {
        if (fresh) *fresh = false;
        return t.get();
      }
    texture* t = make_new();
    t->location = loc;
    if (fresh) *fresh = true;
    return t;
  }
  void destroy(texture* t) {
    textures.erase(std::remove_if(textures.begin(), textures.end(),
                                  [&](const std::unique_ptr<texture>& u) { return u.get() == t; }),
                   textures.end());
    for (size_t i = 0; i < textures.size(); i++) textures[i]->id = (int)i;
  }
  // texture_context::get_gpu_position_id
  int get_gpu_position_id(const texture* t) const { return t ? t->id : -1; }
};

// ---- objects (object.hpp) and containers (objects_container.hpp:20-115) --------
struct object {
  std::vector<gbr_triangle> tri_list;
  texture* tex = nullptr;
  float4 pos;
  float4 rot_quat{0, 0, 0, 1};
  float dynamic_scale = 1.f;
  float specular = 0.9f, spec_mult = 1.f, diffuse = 1.f;  // object.cpp:72-74
  int32_t feature_flag = 0;
  texture* normal_map = nullptr;  // descriptor rid (obj.rid / normal_map, obj_load.cpp:544-556)
  texture* bump = nullptr;        // obj.bid: the material's map_Bump (obj_load.cpp:520-532)
  uint32_t has_bump = 0;          // descriptor has_bump
  std::string object_name;        // the OBJ group of its usemtl section (obj_load.cpp:414-415, 538)
  texture* ss_map = nullptr;      // descriptor ssid: the screen-space reflection map (object.cpp:106-109)
};

struct objects_container {
  std::vector<object> objs;
  bool isactive = false;
  bool isloaded = false;
  std::string file;             // set_file: loaded by object_context::load_active
  float requested_scale = 1.f;  // applied to positions at load (obj_load.cpp:437)
  float current_scale = 1.f;    // the scale the loaded positions carry (obj_load.cpp:563-564)
  bool textures_are_unique = false;  // set_unique_textures: loads skip the texture cache
  std::string normal_map_file;  // set_normal: every loaded object's normal map (obj_load.cpp:544-556)
  float4 pos;
  float4 rot_quat{0, 0, 0, 1};
  float dynamic_scale = 1.f;

  void add_object(const std::vector<gbr_triangle>& tris, texture* tex) {
    object o;
    o.tri_list = tris;
    o.tex = tex;
    o.pos = pos;
    o.rot_quat = rot_quat;
    o.dynamic_scale = dynamic_scale;
    objs.push_back(o);
  }
  // objects_container::set_load_cube_blank: an axis-aligned box of the given
  // half extents around the origin, 12 two-sided triangles
  void set_load_cube_blank(float4 dim, texture* tex) {
    const float sx = dim.x, sy = dim.y, sz = dim.z;
    const float c[8][3] = {{-sx, -sy, -sz}, {sx, -sy, -sz}, {sx, sy, -sz}, {-sx, sy, -sz},
                           {-sx, -sy, sz},  {sx, -sy, sz},  {sx, sy, sz},  {-sx, sy, sz}};
    const int f[12][3] = {{0, 1, 2}, {0, 2, 3}, {4, 6, 5}, {4, 7, 6}, {0, 4, 5}, {0, 5, 1},
                          {3, 2, 6}, {3, 6, 7}, {0, 3, 7}, {0, 7, 4}, {1, 5, 6}, {1, 6, 2}};
    std::vector<gbr_triangle> tris(12);
    for (int t = 0; t < 12; t++) {
      std::memset(&tris[t], 0, sizeof(gbr_triangle));
      for (int k = 0; k < 3; k++) {
        gbr_vertex& v = tris[t].vertices[k];
        for (int a = 0; a < 3; a++) v.pos[a] = c[f[t][k]][a];
        v.vt[0] = (float)(k & 1);
        v.vt[1] = (float)(k >> 1);
      }
    }
    add_object(tris, tex);
    set_two_sided(true);
  }
  void set_file(const std::string& f) { file = f; isloaded = false; }
  void request_scale(float s) { requested_scale = s; }
  void set_unique_textures(bool u) { textures_are_unique = u; }  // objects_container.cpp:342-345
  void set_normal(const std::string& f) { normal_map_file = f; }  // objects_container.cpp:538-541
  void set_pos(float4 p) { pos = p; for (auto& o : objs) o.pos = p; }
  void offset_pos(float4 d) { set_pos(float4{pos.x + d.x, pos.y + d.y, pos.z + d.z, pos.w}); }
  void set_rot_quat(float4 q) { rot_quat = q; for (auto& o : objs) o.rot_quat = q; }
  void set_dynamic_scale(float s) { dynamic_scale = s; for (auto& o : objs) o.dynamic_scale = s; }
  void set_active(bool a) { isactive = a; }
  void set_specular(float s) { for (auto& o : objs) o.specular = s; }  // 1 - roughness
  void set_spec_mult(float s) { for (auto& o : objs) o.spec_mult = s; }
  void set_diffuse(float d) { for (auto& o : objs) o.diffuse = d; }
  void set_children_texture_id(texture* t) { for (auto& o : objs) o.tex = t; }
  void set_normal_map(texture* t) { for (auto& o : objs) o.normal_map = t; }
  // objects_container::set_screenspace_map_id / set_ss_reflective (objects_container.cpp:28-35, 105-112)
  void set_screenspace_map_id(texture* t) { for (auto& o : objs) o.ss_map = t; }
  void set_ss_reflective(bool on) { set_flag(FLAG_SS_REFLECTIVE, on); }
  void set_outline(bool on) { set_flag(FLAG_OUTLINE, on); }
  void set_flag(int32_t bit, bool on) {
    for (auto& o : objs) o.feature_flag = on ? (o.feature_flag | bit) : (o.feature_flag & ~bit);
  }
  void set_two_sided(bool on) { set_flag(FLAG_TWO_SIDED, on); }
  void set_is_static(bool on) { set_flag(FLAG_IS_STATIC, on); }
  void set_does_not_receive_dynamic_shadows(bool on) { set_flag(FLAG_NO_DYN_SHADOWS, on); }
};

// ---- per-context GPU data (object_context.hpp:82-165) ---------------------------
struct object_context_data {
  gbr_scene* scene = nullptr;
  gbr_framebuffer* fb = nullptr;
  int s_w = 0, s_h = 0;
  float clear_col[4] = {0, 0, 0, 1};
  uint32_t use_linear_rendering = 1;
  uint32_t tri_num = 0, obj_num = 0;
  gbr_status status = GBR_OK;  // the last call's status
  uint32_t frame_id = 0;       // increases monotonically, once per draw_bulk_objs_n
  const object_context_data* blend_render_context = nullptr;  // kernel3's integrated blend source
  float4 c_pos_old, c_rot_old;  // the camera of the previous frame (swap_buffers)

  // object_context_data::swap_buffers (object_context.cpp:17-25): end of a
  // frame; the engine's camera becomes the previous camera
  void swap_buffers();

  // object_context_data::ensure_screen_buffers
  gbr_status ensure_screen_buffers(int w, int h) {
    if (fb && w == s_w && h == s_h) return GBR_OK;
    if (fb) gbr_framebuffer_destroy(fb);
    fb = nullptr;
    s_w = s_h = 0;
    gbr_status st = gbr_framebuffer_create(w, h, 1, &fb);
    if (st == GBR_OK) { s_w = w; s_h = h; }
    return st;
  }
  // copy one framebuffer plane (0 depth, 1 id, 2 rgba, 3 normals) to the host
  gbr_status read_plane(int which, std::vector<uint8_t>& out) const {
    out.resize((size_t)s_w * s_h * 4);
    return fb ? gbr_framebuffer_read(fb, which, out.data(), out.size()) : GBR_INVALID_ARG;
  }
};

struct object_context {
  texture_context tex_ctx;
  std::vector<std::unique_ptr<objects_container>> containers;
  object_context_data gpu_dat;

  object_context() = default;
  object_context(const object_context&) = delete;
  object_context& operator=(const object_context&) = delete;
  ~object_context() {
    if (gpu_dat.fb) gbr_framebuffer_destroy(gpu_dat.fb);
    if (gpu_dat.scene) gbr_scene_destroy(gpu_dat.scene);
  }

  objects_container* make_new() {
    containers.emplace_back(new objects_container());
    return containers.back().get();
  }
  void destroy(objects_container* c) {
    containers.erase(std::remove_if(containers.begin(), containers.end(),
                                     [&](const std::unique_ptr<objects_container>& u) { return u.get() == c; }),
                     containers.end());
  }
  // Loader of objects_container::set_file (gbr_obj.hpp installs obj_load):
  // (container, textures, file, scale, error) -> ok
  std::function<bool(objects_container*, texture_context&, const std::string&, float, std::string*)> file_loader;
  std::string load_error;

  // object_context::load_active: load the files of active containers that
  // have not been loaded (the reference's obj_load / load funcs)
  gbr_status load_active() {
    for (auto& c : containers) {
      if (!c->isactive || c->isloaded || c->file.empty()) continue;
      if (!file_loader || !file_loader(c.get(), tex_ctx, c->file, c->requested_scale, &load_error))
        return gpu_dat.status = GBR_INVALID_ARG;
      c->isloaded = true;
      c->set_pos(c->pos);
      c->set_rot_quat(c->rot_quat);
      c->set_dynamic_scale(c->dynamic_scale);
    }
    return GBR_OK;
  }
  void set_clear_colour(float4 c) {
    gpu_dat.clear_col[0] = c.x; gpu_dat.clear_col[1] = c.y; gpu_dat.clear_col[2] = c.z; gpu_dat.clear_col[3] = c.w;
  }
  void set_use_linear_rendering(uint32_t on) { gpu_dat.use_linear_rendering = on; }

  // Descriptors of every object of the active containers, in container then
  // object order (generate_gpu_object_descriptor, object_context.cpp:228-339).
  std::vector<gbr_obj_g_descriptor> descriptors() const {
    std::vector<gbr_obj_g_descriptor> d;
    for (const auto& c : containers) {
      if (!c->isactive) continue;
      for (const object& o : c->objs) {
        gbr_obj_g_descriptor g;
        std::memset(&g, 0, sizeof g);
        const float wp[4] = {o.pos.x, o.pos.y, o.pos.z, o.pos.w};
        const float q[4] = {o.rot_quat.x, o.rot_quat.y, o.rot_quat.z, o.rot_quat.w};
        std::memcpy(g.world_pos, wp, 16);
        std::memcpy(g.world_rot_quat, q, 16);
        std::memcpy(g.old_world_pos_1, wp, 16);
        std::memcpy(g.old_world_pos_2, wp, 16);
        std::memcpy(g.old_world_rot_quat_1, q, 16);
        std::memcpy(g.old_world_rot_quat_2, q, 16);
        g.scale = o.dynamic_scale;
        g.tid = (uint32_t)tex_ctx.get_gpu_position_id(o.tex);
        g.rid = o.normal_map ? (uint32_t)tex_ctx.get_gpu_position_id(o.normal_map) : 0xFFFFFFFFu;
        g.ssid = o.ss_map ? (uint32_t)tex_ctx.get_gpu_position_id(o.ss_map) : 0xFFFFFFFFu;
        g.has_bump = o.has_bump;
        g.specular = o.specular;
        g.spec_mult = o.spec_mult;
        g.diffuse = o.diffuse;
        g.feature_flag = o.feature_flag;
        d.push_back(g);
      }
    }
    return d;
  }

  // object_context::build: upload triangles (object_id = descriptor index,
  // object_context.cpp:424), descriptors and the texture atlas.
  gbr_status build(bool force = false) {
    (void)force;
    gbr_status st = GBR_OK;
    if (!gpu_dat.scene) st = gbr_scene_create(&gpu_dat.scene);
    if (st != GBR_OK) return gpu_dat.status = st;
    std::vector<gbr_triangle> tris;
    uint32_t o_id = 0;
    for (const auto& c : containers) {
      if (!c->isactive) continue;
      for (const object& o : c->objs) {
        for (gbr_triangle t : o.tri_list) {
          t.vertices[0].object_id = o_id;
          tris.push_back(t);
        }
        o_id++;
      }
    }
    const auto descs = descriptors();
    std::vector<int32_t> sizes;
    std::vector<const uint8_t*> px;
    for (const auto& t : tex_ctx.textures) {
      sizes.push_back(t->size);
      px.push_back(t->rgba.data());
    }
    st = gbr_scene_set_triangles(gpu_dat.scene, tris.data(), (uint32_t)tris.size());
    if (st == GBR_OK) st = gbr_scene_set_descriptors(gpu_dat.scene, descs.data(), (uint32_t)descs.size());
    if (st == GBR_OK) st = gbr_scene_set_textures(gpu_dat.scene, (uint32_t)sizes.size(), sizes.data(), px.data());
    gpu_dat.tri_num = (uint32_t)tris.size();
    gpu_dat.obj_num = (uint32_t)descs.size();
    return gpu_dat.status = st;
  }
  // object_context::flush_locations -> object::g_flush (object.cpp:652-860):
  // position, rotation, scale, texture id and feature flags of every object;
  // the motion-blur pose history kept in the descriptors stays
  gbr_status flush_locations() {
    const auto descs = descriptors();
    std::vector<gbr_object_flush> f(descs.size());
    for (size_t i = 0; i < descs.size(); i++) {
      f[i].index = (uint32_t)i;
      f[i].tid = descs[i].tid;
      f[i].scale = descs[i].scale;
      f[i].feature_flag = descs[i].feature_flag;
      std::memcpy(f[i].world_pos, descs[i].world_pos, 16);
      std::memcpy(f[i].world_rot_quat, descs[i].world_rot_quat, 16);
    }
    return gpu_dat.status = gbr_scene_flush_objects(gpu_dat.scene, f.data(), (uint32_t)f.size());
  }
  object_context_data* fetch() { return &gpu_dat; }
  // object_context::set_blend_render_context (object_context.cpp:891-894):
  // this context's frames blend in the other's last frame where it is nearer
  void set_blend_render_context(object_context& other) { gpu_dat.blend_render_context = &other.gpu_dat; }
};

// ---- lights (light.hpp:11-68) ----------------------------------------------------
struct light_gpu {
  std::vector<gbr_light> lights;  // the active lights, in list order
};

struct light {
  float4 pos, col;
  uint32_t shadow = 0;
  float brightness = 1.f, radius = 20000.f, diffuse = 1.f, godray_intensity = 0.f;
  int32_t is_static = 0;
  bool active = true;

  void set_pos(float4 p) { pos = p; }
  void set_col(float4 c) { col = c; }
  void set_shadow_casting(uint32_t s) { shadow = s; }
  void set_brightness(float b) { brightness = b; }
  void set_radius(float r) { radius = r; }
  void set_diffuse(float d) { diffuse = d; }
  void set_godray_intensity(float g) { godray_intensity = g; }
  void set_is_static(bool s) { is_static = s ? 1 : 0; }
  void set_active(bool a) { active = a; }

  static std::vector<std::unique_ptr<light>>& lightlist() {
    static std::vector<std::unique_ptr<light>> list;
    return list;
  }
  // light::add_light copies the light into the global list
  static light* add_light(const light* l) {
    lightlist().emplace_back(new light(*l));
    return lightlist().back().get();
  }
  static void remove_light(light* l) {
    auto& v = lightlist();
    v.erase(std::remove_if(v.begin(), v.end(), [&](const std::unique_ptr<light>& u) { return u.get() == l; }),
            v.end());
  }
  // light::build: the active lights as the kernels read them
  static light_gpu build() {
    light_gpu g;
    for (const auto& l : lightlist()) {
      if (!l->active) continue;
      gbr_light o;
      std::memset(&o, 0, sizeof o);
      const float p[4] = {l->pos.x, l->pos.y, l->pos.z, l->pos.w};
      const float c[4] = {l->col.x, l->col.y, l->col.z, l->col.w};
      std::memcpy(o.pos, p, 16);
      std::memcpy(o.col, c, 16);
      o.shadow = l->shadow;
      o.brightness = l->brightness;
      o.radius = l->radius;
      o.diffuse = l->diffuse;
      o.godray_intensity = l->godray_intensity;
      o.is_static = l->is_static;
      g.lights.push_back(o);
    }
    return g;
  }
};

// ---- engine (engine.hpp) ----------------------------------------------------------
struct engine {
  int width = 0, height = 0;
  static inline float4 c_pos, c_rot;    // camera position, extrinsic XYZ Euler angles (static, engine.hpp)
  float horizontal_fov_degrees = 120.f;  // engine.hpp:115
  uint32_t view_flags = 0;              // GBR_VIEW_*: kernel3's optional -D switches
  void* stream = nullptr;               // cudaStream_t; null = the default stream
  const light_gpu* lights = nullptr;
  gbr_scene* lights_uploaded_to = nullptr;
  size_t lights_uploaded_n = 0;
  std::vector<gbr_light> lights_uploaded;
  object_context_data* last_dat = nullptr;  // the context of the last draw_bulk_objs_n (do_pseudo_aa's buffers)

  // engine::load: the screen size (the reference also builds the OpenCL
  // program with it compiled in; here it is a per-view parameter)
  void load(int w, int h) { width = w; height = h; }
  void set_camera_pos(float4 p) { c_pos = p; }
  void set_camera_rot(float4 r) { c_rot = r; }
  void set_fov(float hfov_deg) { horizontal_fov_degrees = hfov_deg; }
  void set_view_flags(uint32_t flags) { view_flags = flags; }
  void set_light_data(const light_gpu& l) { lights = &l; lights_uploaded_to = nullptr; }
  gbr_status set_object_data(object_context_data& dat) { return dat.ensure_screen_buffers(width, height); }

  gbr_camera camera() const {
    gbr_camera c;
    const float p[4] = {c_pos.x, c_pos.y, c_pos.z, c_pos.w};
    const float r[4] = {c_rot.x, c_rot.y, c_rot.z, c_rot.w};
    std::memcpy(c.pos, p, 16);
    std::memcpy(c.rot, r, 16);
    return c;
  }
  gbr_view view(const object_context_data& dat) const {
    gbr_view v;
    std::memset(&v, 0, sizeof v);
    v.width = width;
    v.height = height;
    v.hfov_deg = horizontal_fov_degrees;
    std::memcpy(v.clear_col, dat.clear_col, 16);
    v.use_linear = dat.use_linear_rendering;
    v.flags = view_flags;
    return v;
  }
  gbr_status sync_lights(object_context_data& dat) {
    if (!lights || !dat.scene) return GBR_OK;
    const bool same = lights_uploaded_to == dat.scene && lights_uploaded.size() == lights->lights.size() &&
                      std::memcmp(lights_uploaded.data(), lights->lights.data(),
                                  lights->lights.size() * sizeof(gbr_light)) == 0;
    if (same) return GBR_OK;
    gbr_status st = gbr_scene_set_lights(dat.scene, lights->lights.data(), (uint32_t)lights->lights.size());
    if (st == GBR_OK) {
      lights_uploaded_to = dat.scene;
      lights_uploaded = lights->lights;
    }
    return st;
  }
  // engine::generate_realtime_shadowing (engine.cpp:1601-1790)
  gbr_status generate_realtime_shadowing(object_context_data& dat) {
    gbr_status st = sync_lights(dat);
    if (st == GBR_OK) st = gbr_shadow_pass(dat.scene, stream);
    return dat.status = st;
  }
  // engine::draw_bulk_objs_n -> render_tris (engine.cpp:1794-2034)
  gbr_status draw_bulk_objs_n(object_context_data& dat) {
    gbr_status st = sync_lights(dat);
    if (st == GBR_OK) st = dat.ensure_screen_buffers(width, height);
    gbr_outputs o;
    if (st == GBR_OK) st = gbr_framebuffer_outputs(dat.fb, &o, nullptr, nullptr);
    const gbr_camera c = camera();
    const gbr_view v = view(dat);
    const object_context_data* b = dat.blend_render_context;
    gbr_outputs bo;
    if (st == GBR_OK && b && b->fb) {
      // render_tris binds the other context's depth and screen (engine.cpp:1943-1988)
      if (b->s_w != width || b->s_h != height) st = GBR_INVALID_ARG;
      if (st == GBR_OK) st = gbr_framebuffer_outputs(b->fb, &bo, nullptr, nullptr);
      if (st == GBR_OK) st = gbr_render_view_blend(dat.scene, &c, &v, &o, &bo, stream);
    } else if (st == GBR_OK) {
      st = gbr_render_view(dat.scene, &c, &v, &o, stream);
    }
    if (st == GBR_OK) {
      dat.frame_id++;
      last_dat = &dat;
    }
    return dat.status = st;
  }
  // engine::do_pseudo_aa (engine.cpp:1513-1516): over the last frame drawn, in place
  gbr_status do_pseudo_aa() {
    if (!last_dat) return GBR_INVALID_ARG;
    object_context_data& dat = *last_dat;
    gbr_outputs o;
    gbr_status st = gbr_framebuffer_outputs(dat.fb, &o, nullptr, nullptr);
    const gbr_view v = view(dat);
    if (st == GBR_OK) st = gbr_post_pseudo_aa(dat.scene, &v, o.depth, o.id, o.normals, o.rgba, o.rgba, stream);
    return dat.status = st;
  }
  // engine::do_motion_blur (engine.cpp:1518-1536): in place, with the
  // context's frame id and previous camera
  gbr_status do_motion_blur(object_context_data& dat, float strength, float camera_contribution) {
    gbr_outputs o;
    gbr_status st = gbr_framebuffer_outputs(dat.fb, &o, nullptr, nullptr);
    const gbr_camera c = camera();
    gbr_camera old;
    const float p[4] = {dat.c_pos_old.x, dat.c_pos_old.y, dat.c_pos_old.z, dat.c_pos_old.w};
    const float r[4] = {dat.c_rot_old.x, dat.c_rot_old.y, dat.c_rot_old.z, dat.c_rot_old.w};
    std::memcpy(old.pos, p, 16);
    std::memcpy(old.rot, r, 16);
    const gbr_view v = view(dat);
    if (st == GBR_OK)
      st = gbr_post_motion_blur(dat.scene, &c, &old, &v, dat.frame_id, strength, camera_contribution, o.depth, o.id,
                                o.rgba, o.rgba, stream);
    return dat.status = st;
  }
  // engine::draw_screenspace_reflections (engine.cpp:1483-1511): in place over
  // the context's last frame (the reference's tex argument is unused by the kernel)
  gbr_status draw_screenspace_reflections(object_context_data& dat) {
    gbr_outputs o;
    gbr_status st = gbr_framebuffer_outputs(dat.fb, &o, nullptr, nullptr);
    const gbr_camera c = camera();
    const gbr_view v = view(dat);
    if (st == GBR_OK) st = gbr_post_reflections(dat.scene, &c, &v, o.depth, o.id, o.rgba, o.rgba, stream);
    return dat.status = st;
  }
  // engine::draw_godrays (engine.cpp:1463-1482): light shafts added to the
  // RGBA8 screen of the last draw_bulk_objs_n, in place; nothing to do when no
  // light has godray_intensity > 0 (the reference's any_godray check)
  gbr_status draw_godrays(object_context_data& dat) {
    bool any = false;
    if (lights)
      for (const gbr_light& l : lights->lights) any = any || l.godray_intensity > 0;
    if (!any) return GBR_OK;
    gbr_status st = sync_lights(dat);
    if (st == GBR_OK) st = dat.ensure_screen_buffers(width, height);
    gbr_outputs o;
    if (st == GBR_OK) st = gbr_framebuffer_outputs(dat.fb, &o, nullptr, nullptr);
    const gbr_camera c = camera();
    const gbr_view v = view(dat);
    if (st == GBR_OK) st = gbr_post_godrays(dat.scene, &c, &v, o.depth, o.rgba, o.rgba, stream);
    return dat.status = st;
  }
  // engine::generate_depth_buffer (engine.cpp:1540): depth only
  gbr_status generate_depth_buffer(object_context_data& dat) {
    gbr_status st = dat.ensure_screen_buffers(width, height);
    gbr_outputs o;
    if (st == GBR_OK) st = gbr_framebuffer_outputs(dat.fb, &o, nullptr, nullptr);
    o.rgba = nullptr;
    o.normals = nullptr;
    const gbr_camera c = camera();
    const gbr_view v = view(dat);
    if (st == GBR_OK) st = gbr_render_view(dat.scene, &c, &v, &o, stream);
    return dat.status = st;
  }
};

inline void object_context_data::swap_buffers() {
  c_pos_old = engine::c_pos;
  c_rot_old = engine::c_rot;
}

}  // namespace openclrenderer

#endif  // GBR_ENGINE_HPP
