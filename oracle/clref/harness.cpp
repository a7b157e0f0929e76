// harness.cpp — TEST INFRASTRUCTURE ONLY: runs the reference's own cl2.cl
// kernels (compiled as C++ through shim.hpp) with the reference's launch
// semantics, as the pin of the oracle restatement.
//
//   render_tris (engine.cpp:1794-2034):  prearrange over triangles, kernel1 and
//     kernel2 over the exact fragment count, kernel3 over pixels
//   generate_realtime_shadowing (engine.cpp:1601-1790): prearrange_realtime_
//     shadowing + kernel1_realtime_shadowing per shadow light
//   update_gpu_tex + generate_mips + generate_mip_mips (texture.cpp:323-460)
//
// prearrange runs its work items in order, so fragment records are ordered by
// (triangle, clip output); kernel2's write_imageui keeps the minimum fragment
// index, i.e. the minimum (triangle, clip output) among fragments passing the
// depth test, which is mapped to the canonical id 2*triangle + clip output.
// Built by build_ref.py into oracle/_ref/libclref.so (not committed).
#include <sys/mman.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

#include "shim.hpp"

namespace clref {
thread_local size_t gbr_ref_gid[2];
int gbr_ref_W = 0, gbr_ref_H = 0;
float gbr_ref_FOV = 0.f;
#include CLREF_KERNELS
}  // namespace clref

using namespace clref;

namespace {

template <class F>
void par_for(int64_t n, int nthreads, F&& f) {
  if (nthreads <= 1 || n < 1024) {
    for (int64_t i = 0; i < n; i++) f(i);
    return;
  }
  std::atomic<int64_t> next{0};
  auto worker = [&]() {
    for (;;) {
      int64_t b = next.fetch_add(4096);
      if (b >= n) break;
      int64_t e = b + 4096 < n ? b + 4096 : n;
      for (int64_t i = b; i < e; i++) f(i);
    }
  };
  std::vector<std::thread> ts;
  for (int t = 0; t < nthreads - 1; t++) ts.emplace_back(worker);
  worker();
  for (auto& t : ts) t.join();
}

// Large lazily-committed buffer for the fragment list (the reference writes it
// without a bound check).
struct Lazy {
  void* p = nullptr;
  size_t bytes = 0;
  explicit Lazy(size_t b) : bytes(b) {
    p = mmap(nullptr, b, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS | MAP_NORESERVE, -1, 0);
    if (p == MAP_FAILED) p = nullptr;
  }
  ~Lazy() {
    if (p) munmap(p, bytes);
  }
};

// The reference's own per-frame buffers, kept for a post pass.
struct Frame {
  Lazy frags{(size_t)1 << 36};
  std::vector<float4> cut;
  std::vector<uint> b_before;   // first cutdown slot of each triangle
  std::vector<uint> raw_ids;    // kernel2's id image: fragment indices
  std::vector<ushort2> nrm;
  uint nfrag = 0;
};

}  // namespace

extern "C" {

// One view: prearrange -> kernel1 -> kernel2 -> kernel3.  cam = pos[4], rot[4].
// Outputs: depth u32, canonical id u32, rgba u8 (quantised as the product does),
// normals ushort2 (may be null).  Returns the fragment count, or -1.
int64_t ref_render_frame(const void* tris_in, uint32_t ntris, const void* descs, const void* lights,
                         uint32_t nlights, const uint8_t* atlas, const uint32_t* nums, const uint32_t* sizes,
                         uint32_t mipmap_start, const uint32_t* shadow_dyn, const uint32_t* shadow_static,
                         const float* cam, int W, int H, float fov, uint32_t use_linear, const float* clear,
                         uint32_t* depth, uint32_t* ids, uint8_t* rgba, uint16_t* normals, int nthreads, int ordered,
                         Frame* keep, const uint32_t* blend_depth = nullptr, const uint8_t* blend_rgba = nullptr) {
  gbr_ref_W = W;
  gbr_ref_H = H;
  gbr_ref_FOV = fov;
  auto* tris = (struct triangle*)const_cast<void*>(tris_in);
  auto* gobj = (struct obj_g_descriptor*)const_cast<void*>(descs);
  const size_t P = (size_t)W * H;
  Frame local_frame;
  Frame& F = keep ? *keep : local_frame;
  if (!F.frags.p) return -1;
  uint* frags = (uint*)F.frags.p;
  std::vector<float4>& cut = F.cut;
  cut.assign((size_t)ntris * 6 + 6, float4(0.f));
  std::vector<uint>& b_before = F.b_before;
  b_before.assign(ntris, 0);
  uint tri_num = ntris, maxlen = 0xFFFFFFFFu, frag_count = 0, cut_count = 0;
  float4 c_pos(cam[0], cam[1], cam[2], cam[3]), c_rot(cam[4], cam[5], cam[6], cam[7]);
  if (ordered) {
    for (uint32_t id = 0; id < ntris; id++) {
      gbr_ref_gid[0] = id;
      b_before[id] = id == 0 ? 0 : cut_count;
      prearrange(tris, &tri_num, c_pos, c_rot, frags, &maxlen, &frag_count, &cut_count, cut.data(), gobj);
    }
  } else {
    // timing mode: work items in parallel with the reference's atomics (item 0,
    // which resets the counters, first)
    if (ntris) {
      gbr_ref_gid[0] = 0;
      prearrange(tris, &tri_num, c_pos, c_rot, frags, &maxlen, &frag_count, &cut_count, cut.data(), gobj);
    }
    par_for((int64_t)ntris - 1, nthreads, [&](int64_t i) {
      gbr_ref_gid[0] = (size_t)i + 1;
      prearrange(tris, &tri_num, c_pos, c_rot, frags, &maxlen, &frag_count, &cut_count, cut.data(), gobj);
    });
  }
  const uint nfrag = frag_count;
  F.nfrag = nfrag;
  for (size_t p = 0; p < P; p++) depth[p] = 0xFFFFFFFFu;
  image2d_t idimg{ids, W, H, 0};
  for (size_t p = 0; p < P; p++) ids[p] = 0xFFFFFFFFu;
  uint f_len = nfrag;
  par_for(nfrag, nthreads, [&](int64_t i) {
    gbr_ref_gid[0] = (size_t)i;
    kernel1(tris, frags, depth, &f_len, cut.data(), idimg);
  });
  par_for(nfrag, nthreads, [&](int64_t i) {
    gbr_ref_gid[0] = (size_t)i;
    kernel2(tris, frags, depth, idimg, &f_len, cut.data());
  });
  std::vector<float> screen(P * 4, 0.f);
  std::vector<uint> to_clear(P);
  std::vector<ushort2>& nrm = F.nrm;
  nrm.assign(P, ushort2{0, 0});
  image2d_t scr{screen.data(), W, H, 2}, backup{nullptr, W, H, 2};
  image2d_t blend{const_cast<uint8_t*>(blend_rgba), W, H, 1};
  const int use_blend = blend_depth && blend_rgba ? 1 : 0;
  uint lnum = nlights;
  float4 clear_col(clear[0], clear[1], clear[2], clear[3]);
  par_for((int64_t)P, nthreads, [&](int64_t p) {
    const int x = (int)(p % W), y = (int)(p / W);
    if (depth[p] != 0xFFFFFFFFu && ids[p] == 0xFFFFFFFFu) {
      // depth without any fragment passing kernel2's test: the reference would
      // read a stale id; the canonical rule shades it as background (kernel3's
      // background path, blend included)
      float4 c = clear_col;
      if (use_blend && blend_depth[p] < depth[p]) {
        const float4 o(blend_rgba[p * 4] / 255.0f, blend_rgba[p * 4 + 1] / 255.0f, blend_rgba[p * 4 + 2] / 255.0f,
                       blend_rgba[p * 4 + 3] / 255.0f);
        for (int k = 0; k < 3; k++) c.s[k] = fmaf(o.s[k], o.s[3], c.s[k] * (1.0f - o.s[3]));
        c.s[3] = c.s[2];
      }
      memcpy(&screen[p * 4], c.s, 16);
      return;
    }
    gbr_ref_gid[0] = (size_t)x;
    gbr_ref_gid[1] = (size_t)y;
    kernel3(tris, c_pos, c_rot, depth, idimg, (uchar4*)atlas, scr, backup, const_cast<uint*>(nums),
            const_cast<uint*>(sizes), gobj, &lnum, (struct light*)const_cast<void*>(lights),
            const_cast<uint*>(shadow_dyn), const_cast<uint*>(shadow_static), to_clear.data(), frags, cut.data(),
            clear_col, 0, nrm.data(), use_blend, const_cast<uint*>(blend_depth), blend, mipmap_start, use_linear);
  });
  if (keep) F.raw_ids.assign(ids, ids + P);
  for (size_t p = 0; p < P; p++) {
    for (int k = 0; k < 4; k++) rgba[p * 4 + k] = (uint8_t)gbr::quant8(screen[p * 4 + k]);
    bool drawn = depth[p] != 0xFFFFFFFFu && ids[p] != 0xFFFFFFFFu;
    if (!drawn) nrm[p] = ushort2{0, 0};
    if (normals) {
      normals[p * 2] = nrm[p].x;
      normals[p * 2 + 1] = nrm[p].y;
    }
    if (ordered && ids[p] != 0xFFFFFFFFu) {
      uint f = ids[p];
      uint tri = frags[(size_t)f * 5 + 0];
      uint ctri = frags[(size_t)f * 5 + 2];
      ids[p] = 2 * tri + (ctri - b_before[tri]);
    }
  }
  return (int64_t)nfrag;
}

int64_t ref_render(const void* tris_in, uint32_t ntris, const void* descs, const void* lights, uint32_t nlights,
                   const uint8_t* atlas, const uint32_t* nums, const uint32_t* sizes, uint32_t mipmap_start,
                   const uint32_t* shadow_dyn, const uint32_t* shadow_static, const float* cam, int W, int H,
                   float fov, uint32_t use_linear, const float* clear, uint32_t* depth, uint32_t* ids,
                   uint8_t* rgba, uint16_t* normals, int nthreads, int ordered, const uint32_t* blend_depth,
                   const uint8_t* blend_rgba) {
  return ref_render_frame(tris_in, ntris, descs, lights, nlights, atlas, nums, sizes, mipmap_start, shadow_dyn,
                          shadow_static, cam, W, H, fov, use_linear, clear, depth, ids, rgba, normals, nthreads,
                          ordered, nullptr, blend_depth, blend_rgba);
}

// A post pass over one rendered frame, with the reference's own fragment
// records, cutdown triangles and kernel2 id image (engine.cpp:1463-1531):
//   kind 0 do_pseudo_aa, 1 do_motion_blur, 2 screenspace_reflections.
// in_screen is the frame's RGBA8 (as the product keeps it); the output image
// starts as a copy of it, so pixels the pass leaves unwritten keep the input.
// Pixels with depth but no id (kernel2's test failed everywhere) would read a
// stale id in the reference; they are left unwritten.  descs is updated by
// do_motion_blur's pose-history writes.  params: frame_id, strength,
// camera_contribution; cam_old = pos[4], rot[4] of the previous frame.
// Outputs: rgba (the frame), rgba_post.
int64_t ref_post(int kind, const void* tris_in, uint32_t ntris, void* descs, const void* lights, uint32_t nlights,
                 const uint8_t* atlas, const uint32_t* nums, const uint32_t* sizes, uint32_t mipmap_start,
                 const uint32_t* shadow_dyn, const uint32_t* shadow_static, const float* cam, const float* cam_old,
                 int W, int H, float fov, uint32_t use_linear, const float* clear, uint32_t frame_id, float strength,
                 float camera_contribution, uint32_t* depth, uint32_t* ids, uint8_t* rgba, uint16_t* normals,
                 uint8_t* rgba_post) {
  Frame F;
  const int64_t nf = ref_render_frame(tris_in, ntris, descs, lights, nlights, atlas, nums, sizes, mipmap_start,
                                      shadow_dyn, shadow_static, cam, W, H, fov, use_linear, clear, depth, ids, rgba,
                                      normals, 1, 1, &F);
  if (nf < 0) return nf;
  auto* tris = (struct triangle*)const_cast<void*>(tris_in);
  auto* gobj = (struct obj_g_descriptor*)descs;
  const size_t P = (size_t)W * H;
  // the id image the post kernels read: fragment indices; pixels without one
  // point at fragment 0 (read by do_pseudo_aa, its value unused)
  std::vector<uint> raw(F.raw_ids);
  for (size_t p = 0; p < P; p++)
    if (raw[p] == 0xFFFFFFFFu) raw[p] = 0;
  uint zero_frag[5] = {0, 0, 0, 0, 0};
  uint* frags = F.nfrag ? (uint*)F.frags.p : zero_frag;
  image2d_t idimg{raw.data(), W, H, 0};
  image2d_t in{rgba, W, H, 1};
  std::vector<float> out(P * 4), front(P * 4);
  for (size_t i = 0; i < P * 4; i++) out[i] = front[i] = rgba[i] / 255.0f;
  image2d_t o{out.data(), W, H, 2}, fr{front.data(), W, H, 2};
  float4 c_pos(cam[0], cam[1], cam[2], cam[3]), c_rot(cam[4], cam[5], cam[6], cam[7]);
  float4 c_pos_old(cam_old[0], cam_old[1], cam_old[2], cam_old[3]);
  float4 c_rot_old(cam_old[4], cam_old[5], cam_old[6], cam_old[7]);
  // one thread: do_motion_blur's pose-history writes from every pixel of an
  // object store the same values
  for (size_t p = 0; p < P; p++) {
    if (depth[p] != 0xFFFFFFFFu && F.raw_ids[p] == 0xFFFFFFFFu) continue;
    gbr_ref_gid[0] = p % W;
    gbr_ref_gid[1] = p / W;
    if (kind == 0)
      do_pseudo_aa(idimg, frags, in, o, fr, F.cut.data(), depth, F.nrm.data());
    else if (kind == 1)
      do_motion_blur(idimg, frags, in, o, F.cut.data(), depth, gobj, frame_id, c_pos, c_rot, c_pos_old, c_rot_old,
                     strength, camera_contribution);
    else
      screenspace_reflections(0, tris, idimg, frags, in, o, F.cut.data(), depth, gobj, frame_id, c_pos, c_rot,
                              c_pos_old, c_rot_old, (uchar4*)atlas, const_cast<uint*>(nums),
                              const_cast<uint*>(sizes), mipmap_start);
  }
  for (size_t i = 0; i < P * 4; i++) rgba_post[i] = (uint8_t)gbr::quant8(out[i]);
  if (kind == 0)
    for (size_t i = 0; i < P * 4; i++)
      if (out[i] != front[i]) return -2;  // the two screens must agree
  return nf;
}

// Cubemaps of every shadow light (dynamic: lights with shadow == 1; static:
// shadow && is_static), 6 * 1024^2 u32 each.
void ref_shadow(const void* tris_in, uint32_t ntris, const void* descs, const void* lights_in, uint32_t nlights,
                uint32_t* dyn, uint32_t* stat, int nthreads, int ordered) {
  auto* tris = (struct triangle*)const_cast<void*>(tris_in);
  auto* gobj = (struct obj_g_descriptor*)const_cast<void*>(descs);
  auto* lights = (const struct light*)lights_in;
  const size_t face = (size_t)1024 * 1024;
  Lazy fragbuf((size_t)1 << 36);
  uint* frags = (uint*)fragbuf.p;
  std::vector<float4> cut((size_t)ntris * 36 + 36);
  uint nn = 0, kk = 0;
  auto one = [&](const struct light& L, int only_static, uint* out) {
    for (size_t i = 0; i < 6 * face; i++) out[i] = 0xFFFFFFFFu;
    uint tri_num = ntris, maxlen = 0xFFFFFFFFu, frag_count = 0, cut_count = 0;
    float4 lpos = L.pos, no_rot(0.f);
    if (ordered) {
      for (uint32_t id = 0; id < ntris; id++) {
        gbr_ref_gid[0] = id;
        prearrange_realtime_shadowing(tris, &tri_num, lpos, no_rot, frags, &maxlen, &frag_count, &cut_count,
                                      cut.data(), gobj, only_static);
      }
    } else if (ntris) {
      gbr_ref_gid[0] = 0;
      prearrange_realtime_shadowing(tris, &tri_num, lpos, no_rot, frags, &maxlen, &frag_count, &cut_count,
                                    cut.data(), gobj, only_static);
      par_for((int64_t)ntris - 1, nthreads, [&](int64_t i) {
        gbr_ref_gid[0] = (size_t)i + 1;
        prearrange_realtime_shadowing(tris, &tri_num, lpos, no_rot, frags, &maxlen, &frag_count, &cut_count,
                                      cut.data(), gobj, only_static);
      });
    }
    uint f_len = frag_count;
    par_for(frag_count, nthreads, [&](int64_t i) {
      gbr_ref_gid[0] = (size_t)i;
      kernel1_realtime_shadowing(tris, frags, out, &f_len, cut.data());
    });
  };
  for (uint32_t i = 0; i < nlights; i++) {
    if (lights[i].shadow == 1) one(lights[i], 0, dyn + (size_t)(nn++) * 6 * face);
    if (lights[i].shadow && lights[i].is_static && stat) one(lights[i], 1, stat + (size_t)(kk++) * 6 * face);
  }
}

// screenspace_godrays (cl2.cl:1792-1917) over a rendered view: depth u32 and
// RGBA8 in, RGBA8 out (quantised as the product does).  cam = pos[4], rot[4].
void ref_godrays(const uint32_t* depth, const uint8_t* rgba_in, int W, int H, float fov, const void* lights_in,
                 uint32_t nlights, const float* cam, uint8_t* rgba_out, int nthreads) {
  gbr_ref_W = W;
  gbr_ref_H = H;
  gbr_ref_FOV = fov;
  const size_t P = (size_t)W * H;
  std::vector<float> out(P * 4, 0.f);
  image2d_t in{const_cast<uint8_t*>(rgba_in), W, H, 1}, o{out.data(), W, H, 2};
  uint lnum = nlights;
  float4 c_pos(cam[0], cam[1], cam[2], cam[3]), c_rot(cam[4], cam[5], cam[6], cam[7]);
  par_for((int64_t)P, nthreads, [&](int64_t p) {
    gbr_ref_gid[0] = (size_t)(p % W);
    gbr_ref_gid[1] = (size_t)(p / W);
    screenspace_godrays(const_cast<uint*>(depth), in, o, &lnum, (struct light*)const_cast<void*>(lights_in), c_pos,
                        c_rot);
  });
  for (size_t i = 0; i < P * 4; i++) rgba_out[i] = (uint8_t)gbr::quant8(out[i]);
}

// update_gpu_tex (flip 1) + generate_mips + generate_mip_mips for every
// texture, into an atlas already laid out by the page packing (nums, sizes).
void ref_textures(uint32_t n, const int32_t* tsizes, const uint8_t* const* rgba, uint8_t* atlas, uint32_t* nums,
                  uint32_t* sizes, uint32_t mipmap_start) {
  uchar4* arr = (uchar4*)atlas;
  for (uint32_t t = 0; t < n; t++) {
    const int s = tsizes[t];
    image2d_t tex{const_cast<uint8_t*>(rgba[t]), s, s, 1};
    for (int y = 0; y < s; y++)
      for (int x = 0; x < s; x++) {
        gbr_ref_gid[0] = x;
        gbr_ref_gid[1] = y;
        update_gpu_tex(tex, t, mipmap_start, nums, sizes, arr, 1);
      }
    for (int y = 0; y < s; y++)
      for (int x = 0; x < s; x++) {
        gbr_ref_gid[0] = x;
        gbr_ref_gid[1] = y;
        generate_mips(t, mipmap_start, nums, sizes, arr, arr);
      }
    for (uint32_t level = 0; level < 3; level++)
      for (int y = 0; y < s; y++)
        for (int x = 0; x < s; x++) {
          gbr_ref_gid[0] = x;
          gbr_ref_gid[1] = y;
          generate_mip_mips(t, level, mipmap_start, nums, sizes, arr, arr);
        }
  }
}

}  // extern "C"
