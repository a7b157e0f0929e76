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

}  // namespace

extern "C" {

// One view: prearrange -> kernel1 -> kernel2 -> kernel3.  cam = pos[4], rot[4].
// Outputs: depth u32, canonical id u32, rgba u8 (quantised as the product does),
// normals ushort2 (may be null).  Returns the fragment count, or -1.
int64_t ref_render(const void* tris_in, uint32_t ntris, const void* descs, const void* lights, uint32_t nlights,
                   const uint8_t* atlas, const uint32_t* nums, const uint32_t* sizes, uint32_t mipmap_start,
                   const uint32_t* shadow_dyn, const uint32_t* shadow_static, const float* cam, int W, int H,
                   float fov, uint32_t use_linear, const float* clear, uint32_t* depth, uint32_t* ids,
                   uint8_t* rgba, uint16_t* normals, int nthreads, int ordered) {
  gbr_ref_W = W;
  gbr_ref_H = H;
  gbr_ref_FOV = fov;
  auto* tris = (struct triangle*)const_cast<void*>(tris_in);
  auto* gobj = (struct obj_g_descriptor*)const_cast<void*>(descs);
  const size_t P = (size_t)W * H;
  Lazy fragbuf((size_t)1 << 36);
  if (!fragbuf.p) return -1;
  uint* frags = (uint*)fragbuf.p;
  std::vector<float4> cut((size_t)ntris * 6 + 6);
  std::vector<uint> b_before(ntris);
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
  std::vector<ushort2> nrm(P);
  image2d_t scr{screen.data(), W, H, 2}, backup{nullptr, W, H, 2}, blend{nullptr, W, H, 2};
  uint lnum = nlights;
  float4 clear_col(clear[0], clear[1], clear[2], clear[3]);
  par_for((int64_t)P, nthreads, [&](int64_t p) {
    const int x = (int)(p % W), y = (int)(p / W);
    if (depth[p] != 0xFFFFFFFFu && ids[p] == 0xFFFFFFFFu) {
      // depth without any fragment passing kernel2's test: the reference would
      // read a stale id; the canonical rule shades it as background
      memcpy(&screen[p * 4], clear_col.s, 16);
      return;
    }
    gbr_ref_gid[0] = (size_t)x;
    gbr_ref_gid[1] = (size_t)y;
    kernel3(tris, c_pos, c_rot, depth, idimg, (uchar4*)atlas, scr, backup, const_cast<uint*>(nums),
            const_cast<uint*>(sizes), gobj, &lnum, (struct light*)const_cast<void*>(lights),
            const_cast<uint*>(shadow_dyn), const_cast<uint*>(shadow_static), to_clear.data(), frags, cut.data(),
            clear_col, 0, nrm.data(), 0, nullptr, blend, mipmap_start, use_linear);
  });
  for (size_t p = 0; p < P; p++) {
    for (int k = 0; k < 4; k++) rgba[p * 4 + k] = (uint8_t)gbr::quant8(screen[p * 4 + k]);
    if (normals) {
      bool drawn = depth[p] != 0xFFFFFFFFu && ids[p] != 0xFFFFFFFFu;
      normals[p * 2] = drawn ? nrm[p].x : 0;
      normals[p * 2 + 1] = drawn ? nrm[p].y : 0;
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
