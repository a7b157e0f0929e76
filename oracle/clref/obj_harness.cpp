// obj_harness.cpp — TEST INFRASTRUCTURE ONLY: runs the reference's obj_load
// (compiled from obj_load.cpp through obj_shim.hpp) on one OBJ file and writes
// what it produced, in the format tests/cpp/obj_dump.cpp writes for
// include/gbr_obj.hpp:
//   <out>.json  objects (triangle count, texture ids, group name) and textures
//               (location; the colour of a blank texture)
//   <out>.bin   every object's triangles in order, per vertex pos[4],
//               normal[4], vt[2] as float32 (40 bytes)
// usage: obj_load_ref file.obj scale unique(0|1) normal_map|- out
#include "obj_shim.hpp"

#include CLREF_OBJ_LOAD

#include <cstdio>

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
  object_context ctx;
  objects_container c;
  c.parent = &ctx;
  c.file = argv[1];
  c.requested_scale = (float)atof(argv[2]);
  c.textures_are_unique = atoi(argv[3]) != 0;
  if (std::string(argv[4]) != "-") c.normal_map = argv[4];
  obj_load(&c);
  const std::string out = argv[5];
  FILE* j = fopen((out + ".json").c_str(), "w");
  FILE* b = fopen((out + ".bin").c_str(), "wb");
  if (!j || !b) return 3;
  fprintf(j, "{\"loaded\": %d, \"current_scale\": %.9g, \"requested_scale\": %.9g,\n \"objects\": [", (int)c.isloaded,
          c.current_scale, c.requested_scale);
  for (size_t i = 0; i < c.objs.size(); i++) {
    const object& o = c.objs[i];
    fprintf(j, "%s\n  {\"ntris\": %d, \"tid\": %d, \"has_bump\": %u, \"bid\": %d, \"rid\": %d, \"name\": %s}",
            i ? "," : "", o.tri_num, (int)o.tid, o.has_bump, o.has_bump ? (int)o.bid : -1, (int)o.rid,
            jstr(o.object_name).c_str());
    for (const triangle& t : o.tri_list)
      for (const vertex& v : t.vertices) {
        const cl_float4 p = v.get_pos(), n = v.get_normal();
        const cl_float2 vt = v.get_vt();
        fwrite(p.s, 4, 4, b);
        fwrite(n.s, 4, 4, b);
        fwrite(vt.s, 4, 2, b);
      }
  }
  fprintf(j, "],\n \"textures\": [");
  for (size_t i = 0; i < ctx.tex_ctx.all_textures.size(); i++) {
    const texture& t = *ctx.tex_ctx.all_textures[i];
    fprintf(j, "%s\n  {\"id\": %d, \"location\": %s", i ? "," : "", t.id, jstr(t.texture_location).c_str());
    if (t.blank)
      fprintf(j, ", \"colour\": [%d, %d, %d, %d], \"size\": [%d, %d]", t.colour[0], t.colour[1], t.colour[2],
              t.colour[3], t.w, t.h);
    fprintf(j, "}");
  }
  fprintf(j, "]}\n");
  fclose(j);
  fclose(b);
  return 0;
}
