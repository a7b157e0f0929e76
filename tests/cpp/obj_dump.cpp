// obj_dump.cpp — test driver for include/gbr_obj.hpp: loads one OBJ file with
// obj_load and writes what it produced in the format of the reference
// loader's harness (oracle/clref/obj_harness.cpp), plus the decoded texels:
//   <out>.json  objects (triangle count, texture ids, group name), textures
//               (location, square edge)
//   <out>.bin   every object's triangles in order, per vertex pos[4],
//               normal[4], vt[2] as float32 (40 bytes)
//   <out>.tex   every texture's RGBA8 texels in order
// usage: obj_dump file.obj scale unique(0|1) normal_map|- out
#include <cstdio>
#include <cstdlib>
#include <string>

#include "gbr_obj.hpp"

using namespace openclrenderer;

static std::string jstr(const std::string& s) {
  std::string o = "\"";
  for (char ch : s) {
    if (ch == '"' || ch == '\\') o += '\\';
    if ((unsigned char)ch < 0x20) {
      char b[8];
      snprintf(b, sizeof b, "\\u%04x", (unsigned char)ch);
      o += b;
    } else {
      o += ch;
    }
  }
  return o + "\"";
}

int main(int argc, char** argv) {
  if (argc != 6) {
    fprintf(stderr, "usage: %s file.obj scale unique normal_map|- out\n", argv[0]);
    return 2;
  }
  texture_context tex_ctx;
  objects_container c;
  c.request_scale((float)atof(argv[2]));
  c.set_unique_textures(atoi(argv[3]) != 0);
  if (std::string(argv[4]) != "-") c.set_normal(argv[4]);
  std::string err;
  const bool ok = obj_load(&c, tex_ctx, argv[1], c.requested_scale, &err);
  if (!ok) fprintf(stderr, "obj_load: %s\n", err.c_str());
  const std::string out = argv[5];
  FILE* j = fopen((out + ".json").c_str(), "w");
  FILE* b = fopen((out + ".bin").c_str(), "wb");
  FILE* t = fopen((out + ".tex").c_str(), "wb");
  if (!j || !b || !t) return 3;
  fprintf(j, "{\"loaded\": %d, \"current_scale\": %.9g, \"requested_scale\": %.9g,\n \"objects\": [", (int)ok,
          c.current_scale, c.requested_scale);
  for (size_t i = 0; i < c.objs.size(); i++) {
    const object& o = c.objs[i];
    fprintf(j, "%s\n  {\"ntris\": %d, \"tid\": %d, \"has_bump\": %u, \"bid\": %d, \"rid\": %d, \"name\": %s}",
            i ? "," : "", (int)o.tri_list.size(), tex_ctx.get_gpu_position_id(o.tex), o.has_bump,
            o.bump ? o.bump->id : -1, o.normal_map ? o.normal_map->id : -1, jstr(o.object_name).c_str());
    for (const gbr_triangle& tr : o.tri_list)
      for (const gbr_vertex& v : tr.vertices) {
        fwrite(v.pos, 4, 4, b);
        fwrite(v.normal, 4, 4, b);
        fwrite(v.vt, 4, 2, b);
      }
  }
  fprintf(j, "],\n \"textures\": [");
  for (size_t i = 0; i < tex_ctx.textures.size(); i++) {
    const texture& x = *tex_ctx.textures[i];
    fprintf(j, "%s\n  {\"id\": %d, \"location\": %s, \"edge\": %d}", i ? "," : "", x.id, jstr(x.location).c_str(),
            x.size);
    fwrite(x.rgba.data(), 1, x.rgba.size(), t);
  }
  fprintf(j, "]}\n");
  fclose(j);
  fclose(b);
  fclose(t);
  return ok ? 0 : 4;
}
