// gbr_oracle.cpp — TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of OpenCLRenderer's cl2.cl triangle path, used as the parity
// checker of the CUDA pipeline.  Only tests/, __graft_entry__.smoke() and the
// CPU-baseline leg of bench.py may load it; the product never does.
//
// It follows the reference kernels step by step, on the reference's own work
// decomposition:
//   prearrange                   cl2.cl:4271-4409  (1 work item per triangle)
//   kernel1                      cl2.cl:4985-5127  (1 work item per 500-pixel fragment,
//                                                   literal float walk state machine)
//   kernel2 (canonical id)       cl2.cl:5390-5546  (same walk; id = min triangle key
//                                                   among fragments passing the +-20 test)
//   kernel3                      cl2.cl:5792-6408  (1 work item per pixel)
//   prearrange_realtime_shadowing cl2.cl:4419-4636
//   kernel1_realtime_shadowing   cl2.cl:5129-5246
//   update_gpu_tex / generate_mips / generate_mip_mips  cl2.cl:923-953, 1070-1189
//   texture page packing         texture_context.cpp:94-261
// with every implementation-defined builtin pinned by gbr_math.h.  Work items
// run on std::threads; atomics are std::atomic.
//
// Parity pin: the restatement is checked against the reference's own cl2.cl
// kernels compiled as C++ (oracle/clref), through golden fixtures.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "../include/gbr.h"
#include "../openclrenderer_gb300/csrc/gbr_math.h"

using namespace gbr;

namespace {

// ---- threading ------------------------------------------------------------
template <class F>
void parallel_for(int64_t n, int nthreads, F&& f) {
  if (n <= 0) return;
  if (nthreads <= 1 || n < 256) {
    for (int64_t i = 0; i < n; i++) f(i);
    return;
  }
  std::atomic<int64_t> next{0};
  const int64_t chunk = std::max<int64_t>(64, n / (int64_t)(nthreads * 16));
  auto worker = [&]() {
    for (;;) {
      int64_t b = next.fetch_add(chunk);
      if (b >= n) break;
      int64_t e = std::min(n, b + chunk);
      for (int64_t i = b; i < e; i++) f(i);
    }
  };
  std::vector<std::thread> ts;
  for (int t = 0; t < nthreads - 1; t++) ts.emplace_back(worker);
  worker();
  for (auto& t : ts) t.join();
}

inline void atomic_min_u32(std::atomic<uint32_t>* a, uint32_t v) {
  uint32_t cur = a->load(std::memory_order_relaxed);
  while (v < cur && !a->compare_exchange_weak(cur, v, std::memory_order_relaxed)) {
  }
}

inline f3 v3(const float* p) { return mk3(p[0], p[1], p[2]); }
inline f4 v4(const float* p) {
  f4 r; r.x = p[0]; r.y = p[1]; r.z = p[2]; r.w = p[3];
  return r;
}

// Host-side cosines/sines of Euler angles (the pinned native_cos/native_sin).
void euler_cs(f3 ang, f3* c, f3* s) {
  *c = mk3((float)cos((double)ang.x), (float)cos((double)ang.y), (float)cos((double)ang.z));
  *s = mk3((float)sin((double)ang.x), (float)sin((double)ang.y), (float)sin((double)ang.z));
}

// ---- prearrange ------------------------------------------------------------
struct Cut {
  f3 p[3];
};
struct Frag {
  uint32_t tri, a, ctri;
  float rconst;
  uint32_t o_id;
};

struct Setup {
  // per triangle: number of clip outputs (the reference reserves this many
  // cutdown slots, culled or not) and, per output, its fragment count (-1 culled)
  std::vector<int> num;
  std::vector<int> nfrag;  // 2 per triangle
  std::vector<float> rconst;
  std::vector<Cut> cut;    // 2 per triangle
  std::vector<uint32_t> ctri_base;
  std::vector<Frag> frags;
};

// full_rotate_quat (cl2.cl:700-729) + the per-output culls of prearrange.
// Returns the clip outputs of triangle T for a camera (cpos, c, s).
int project_tri(const gbr_triangle& T, const gbr_obj_g_descriptor& G, f3 cpos, f3 c, f3 s,
                float fov, float w, float h, f3 out[2][3]) {
  f4 q = v4(G.world_rot_quat);
  f3 wp = v3(G.world_pos);
  f3 pr[3];
  for (int k = 0; k < 3; k++) {
    f3 v = mul3s(v3(T.vertices[k].pos), G.scale);
    f3 inter = rot_quat(v, q);
    pr[k] = rot_cs(add3(inter, wp), cpos, c, s);
  }
  f3 tris[2][3];
  int n = clip_tri(pr, tris);
  for (int i = 0; i < n; i++)
    for (int k = 0; k < 3; k++) out[i][k] = depth_project1(tris[i][k], w, h, fov);
  return n;
}

// Per clip output: -1 when culled, else the fragment count ceil(area/chunk).
int cull_and_count(const f3 p[3], bool two_sided, float w, float h, int chunk, float* rc) {
  int valid = two_sided || backface_front(p[0], p[1], p[2]);
  int cond = (p[0].x < 0 && p[1].x < 0 && p[2].x < 0) ||
             (p[0].x >= w && p[1].x >= w && p[2].x >= w) ||
             (p[0].y < 0 && p[1].y < 0 && p[2].y < 0) ||
             (p[0].y >= h && p[1].y >= h && p[2].y >= h);
  if (!valid || cond) return -1;
  f3 xpv = mk3(roundf(p[0].x), roundf(p[1].x), roundf(p[2].x));
  f3 ypv = mk3(roundf(p[0].y), roundf(p[1].y), roundf(p[2].y));
  *rc = rconstant(xpv, ypv);
  float mm[4];
  bbox4(p[0], p[1], p[2], w, h, mm);
  float area = (mm[1] - mm[0]) * (mm[3] - mm[2]);
  return (int)ceilf(fdiv(area, (float)chunk));
}

void prearrange(const gbr_triangle* tris, uint32_t n, const gbr_obj_g_descriptor* descs,
                f3 cpos, f3 crot, float fov, float w, float h, int nthreads, Setup* S) {
  f3 c, s;
  euler_cs(crot, &c, &s);
  S->num.assign(n, 0);
  S->nfrag.assign((size_t)n * 2, -1);
  S->rconst.assign((size_t)n * 2, 0.0f);
  S->cut.resize((size_t)n * 2);
  parallel_for(n, nthreads, [&](int64_t id) {
    const gbr_triangle& T = tris[id];
    const gbr_obj_g_descriptor& G = descs[T.vertices[0].object_id];
    if (fast_length3(sub3(v3(G.world_pos), cpos)) > kDepthFar) return;
    f3 out[2][3];
    int num = project_tri(T, G, cpos, c, s, fov, w, h, out);
    S->num[id] = num;
    bool two = (G.feature_flag & kFlagTwoSided) > 0;
    for (int i = 0; i < num; i++) {
      Cut& ct = S->cut[id * 2 + i];
      ct.p[0] = out[i][0]; ct.p[1] = out[i][1]; ct.p[2] = out[i][2];
      float rc = 0;
      S->nfrag[id * 2 + i] = cull_and_count(ct.p, two, w, h, kOpSize, &rc);
      S->rconst[id * 2 + i] = rc;
    }
  });
  // The reference appends with atomics in arbitrary order; a serial prefix
  // sum gives the same set of records in triangle order.
  S->ctri_base.assign(n, 0);
  uint64_t ctri = 0, nf = 0;
  std::vector<uint64_t> fbase((size_t)n * 2, 0);
  for (uint32_t id = 0; id < n; id++) {
    S->ctri_base[id] = (uint32_t)ctri;
    ctri += S->num[id];
    for (int i = 0; i < 2; i++) {
      fbase[id * 2 + i] = nf;
      if (S->nfrag[id * 2 + i] > 0) nf += S->nfrag[id * 2 + i];
    }
  }
  S->frags.resize(nf);
  parallel_for(n, nthreads, [&](int64_t id) {
    const gbr_triangle& T = tris[id];
    for (int i = 0; i < 2; i++) {
      int tn = S->nfrag[id * 2 + i];
      for (int a = 0; a < tn; a++) {
        Frag& f = S->frags[fbase[id * 2 + i] + a];
        f.tri = (uint32_t)id;
        f.a = (uint32_t)a;
        f.ctri = (uint32_t)(id * 2 + i);  // index into S->cut
        f.rconst = S->rconst[id * 2 + i];
        f.o_id = T.vertices[0].object_id;
      }
    }
  });
}

// ---- the literal fragment walk of kernel1 / kernel2 -------------------------
// Visits pixels exactly as cl2.cl:5046-5126 (and 5455-5545, 5188-5245).
template <class V>
void walk(const f3 tp[3], float ew, float eh, int chunk, uint32_t distance, bool k2_guards,
          V&& visit) {
  float mm[4];
  bbox4(tp[0], tp[1], tp[2], ew, eh, mm);
  int width = (int)(mm[1] - mm[0]);
  if (width <= 0) return;
  int pixel_along = chunk * (int)distance;
  int pcount = -1;
  float x = ((float)((pixel_along + 0) % width) + mm[0]) - 1.0f;
  float y = floorf(fdiv((float)(pixel_along + pcount), (float)width)) + mm[2];
  float iwidth = fdiv(1.0f, (float)width);
  float rwm = (float)((pixel_along + pcount) % width);
  while (pcount < chunk) {
    pcount++;
    x += 1.0f;
    rwm += 1.0f;
    if (rwm >= (float)width) rwm = 0.0f;
    float ty = y;
    y = floorf(fma_((float)(pixel_along + pcount), iwidth, mm[2]));
    x = y != ty ? rwm + mm[0] : x;
    if (y >= mm[3]) break;
    bool oob = x >= mm[1];
    if (k2_guards) oob = oob || x < mm[0] || y < mm[2];
    if (oob) continue;
    visit(x, y);
  }
}

// point_in_tri, written out as cl2.cl:4798-4807.
bool point_in_tri(float px, float py, float p0x, float p0y, float p1x, float p1y, float p2x,
                  float p2y) {
  float A = 0.5f * ((((-p1y) * p2x + p0y * ((-p1x) + p2x)) + p0x * (p1y - p2y)) + p1x * p2y);
  float sign = A < 0 ? -1.0f : 1.0f;
  float s = (((p0y * p2x - p0x * p2y) + (p2y - p0y) * px) + (p0x - p2x) * py) * sign;
  float t = (((p0x * p1y - p0y * p1x) + (p0y - p1y) * px) + (p1x - p0x) * py) * sign;
  return s > -0.0001f && t > -0.0001f && (s + t) < (2.0001f * A) * sign;
}

struct FragGeom {
  f3 xpv, ypv;
  float A, B, C;
};
FragGeom frag_geom(const f3 tp[3], float rconst) {
  FragGeom g;
  g.xpv = mk3(roundf(tp[0].x), roundf(tp[1].x), roundf(tp[2].x));
  g.ypv = mk3(roundf(tp[0].y), roundf(tp[1].y), roundf(tp[2].y));
  f3 depths = mk3(rcp(fdiv(tp[0].z, kDepthFar)), rcp(fdiv(tp[1].z, kDepthFar)),
                  rcp(fdiv(tp[2].z, kDepthFar)));
  plane_const(depths, g.xpv, g.ypv, rconst, &g.A, &g.B, &g.C);
  return g;
}

void kernel1(const Setup& S, float ew, float eh, std::atomic<uint32_t>* depth, int W,
             int nthreads) {
  parallel_for((int64_t)S.frags.size(), nthreads, [&](int64_t id) {
    const Frag& f = S.frags[id];
    const Cut& ct = S.cut[f.ctri];
    FragGeom g = frag_geom(ct.p, f.rconst);
    walk(ct.p, ew, eh, kOpSize, f.a, false, [&](float x, float y) {
      if (point_in_tri(x, y, g.xpv.x, g.ypv.x, g.xpv.y, g.ypv.y, g.xpv.z, g.ypv.z)) {
        uint32_t d = depth_at(g.A, g.B, g.C, x, y);
        atomic_min_u32(&depth[(int)(y * (float)W) + (int)x], d);
      }
    });
  });
}

void kernel2(const Setup& S, float ew, float eh, const uint32_t* depth,
             std::atomic<uint32_t>* ids, int W, int nthreads) {
  parallel_for((int64_t)S.frags.size(), nthreads, [&](int64_t id) {
    const Frag& f = S.frags[id];
    const Cut& ct = S.cut[f.ctri];
    FragGeom g = frag_geom(ct.p, f.rconst);
    uint32_t key = f.ctri;  // 2*triangle + clip_sub: the canonical id
    walk(ct.p, ew, eh, kOpSize, f.a, true, [&](float x, float y) {
      if (point_in_tri(x, y, g.xpv.x, g.ypv.x, g.xpv.y, g.ypv.y, g.xpv.z, g.ypv.z)) {
        uint32_t my = depth_at(g.A, g.B, g.C, x, y);
        size_t p = (size_t)((int)y * W + (int)x);
        uint32_t val = depth[p];
        int c2 = my > val - kBufError && my < val + kBufError;
        if (c2) atomic_min_u32(&ids[p], key);
      }
    });
  });
}

// ---- kernel3 ---------------------------------------------------------------
struct Atlas {
  const uint8_t* data;
  const uint32_t* nums;
  const uint32_t* sizes;
  uint32_t mipmap_start;
};

f4 read_tex_pre(f2 coords, int which, int slice, float width, const Atlas& at) {
  const float imax = 1.0f / 2048.0f;
  float ihnum = width * imax;
  float tnumy = floorf((float)which * ihnum);
  float tnumx = (float)which - fdiv(tnumy, ihnum);
  coords.x = clampf_(coords.x, 0.001f, width - 0.001f);
  coords.y = clampf_(coords.y, 0.001f, width - 0.001f);
  int cx = f2i_sat(fma_(tnumx, width, coords.x));
  int cy = f2i_sat(fma_(tnumy, width, coords.y));
  const uint8_t* t = at.data + ((size_t)slice * kTexPage * kTexPage + (size_t)cy * kTexPage + cx) * 4;
  f4 r; r.x = t[0]; r.y = t[1]; r.z = t[2]; r.w = t[3];
  return r;
}

f4 bilinear_pre(f2 m, int which, int slice, float width, const Atlas& at) {
  f2 pos = mk2(floorf(m.x), floorf(m.y));
  f4 c0 = read_tex_pre(pos, which, slice, width, at);
  f4 c1 = read_tex_pre(mk2(pos.x + 1, pos.y), which, slice, width, at);
  f4 c2 = read_tex_pre(mk2(pos.x, pos.y + 1), which, slice, width, at);
  f4 c3 = read_tex_pre(mk2(pos.x + 1, pos.y + 1), which, slice, width, at);
  f2 u = mk2(m.x - pos.x, m.y - pos.y);
  f2 b = mk2(1.0f - u.x, 1.0f - u.y);
  f4 r;
  r.x = fma_(c0.x, b.x, c1.x * u.x) * b.y + fma_(c2.x, b.x, c3.x * u.x) * u.y;
  r.y = fma_(c0.y, b.x, c1.y * u.x) * b.y + fma_(c2.y, b.x, c3.y * u.x) * u.y;
  r.z = fma_(c0.z, b.x, c1.z * u.x) * b.y + fma_(c2.z, b.x, c3.z * u.x) * u.y;
  r.w = fma_(c0.w, b.x, c1.w * u.x) * b.y + fma_(c2.w, b.x, c3.w * u.x) * u.y;
  return r;
}

f4 texture_filter_diff(f2 vt, f2 vtdiff, int tid2, const Atlas& at) {
  uint32_t nv = at.nums[tid2];
  int slice = (int)(nv >> 16);
  int tsize = (int)at.sizes[slice];
  f2 vtm = texture_mod(vt);
  float wx = vtdiff.x * (float)tsize, wy = vtdiff.y * (float)tsize;
  float worst = fsqrt(wx * wx + wy * wy);
  float wif = log2_approx(worst);
  wif = fmax_(wif, 0.0f);
  float mip_lower = floorf(wif);
  mip_lower = clampf_(mip_lower, 0.0f, (float)kMipLevels);
  float fmd = wif - mip_lower;
  int tid_lower = mip_lower == 0.0f
                      ? tid2
                      : (int)(((mip_lower - 1.0f) + (float)at.mipmap_start) + (float)(tid2 * kMipLevels));
  int tid_higher = (int)((clampf_(mip_lower, 0.0f, kMipLevels - 1.0f) + (float)at.mipmap_start) +
                         (float)(tid2 * kMipLevels));
  uint32_t lnv = at.nums[tid_lower], hnv = at.nums[tid_higher];
  int sl = (int)(lnv >> 16), sh = (int)(hnv >> 16);
  int wl = (int)(lnv & 0xFFFF), wh = (int)(hnv & 0xFFFF);
  float szl = (float)at.sizes[sl], szh = (float)at.sizes[sh];
  f4 c1 = bilinear_pre(mk2(vtm.x * szl, vtm.y * szl), wl, sl, szl, at);
  f4 c2 = bilinear_pre(mk2(vtm.x * szh, vtm.y * szh), wh, sh, szh, at);
  const float i255 = 1.0f / 255.0f;
  f4 r;
  r.x = (c1.x + (c2.x - c1.x) * fmd) * i255;
  r.y = (c1.y + (c2.y - c1.y) * fmd) * i255;
  r.z = (c1.z + (c2.z - c1.z) * fmd) * i255;
  r.w = (c1.w + (c2.w - c1.w) * fmd) * i255;
  return r;
}

struct ShadeView {
  int W, H;
  float fov;
  f3 cpos, crot_c, crot_s;
  f3 crot;  // the Euler angles themselves (the FP64 shading takes exact cos / sin)
  uint32_t flags = 0;  // gbr_view.flags: kernel3's optional switches
  f3 face_c[6], face_s[6];
  uint32_t use_linear;
  f4 clear;
  // CAN_INTEGRATED_BLEND: the blend context's depth and RGBA8, or null
  const uint32_t* blend_depth = nullptr;
  const uint8_t* blend_rgba = nullptr;
};

// alpha_blend (cl2.cl:1721-1728) of the blend context's texel p over c, when
// that context is nearer than depth d (cl2.cl:5839-5851, 6339-6351).
bool blend_over(const ShadeView& v, size_t p, uint32_t d, float c[3]) {
  if (!v.blend_depth || !(v.blend_depth[p] < d)) return false;
  float o[4];
  for (int k = 0; k < 4; k++) o[k] = fdiv((float)v.blend_rgba[4 * p + k], 255.0f);
  for (int k = 0; k < 3; k++) c[k] = fma_(o[k], o[3], c[k] * (1.0f - o[3]));
  return true;
}

f2 get_vtdiff(const f3 tp[3], float x, float y, const ShadeView& v,
              const gbr_obj_g_descriptor& G, f2 vt, f3 p1, f3 p2, f3 p3, f2 vt1, f2 vt2, f2 vt3,
              float rconst) {
  f3 xpv = mk3(roundf(tp[0].x), roundf(tp[1].x), roundf(tp[2].x));
  f3 ypv = mk3(roundf(tp[0].y), roundf(tp[1].y), roundf(tp[2].y));
  f3 depths = mk3(rcp(tp[0].z), rcp(tp[1].z), rcp(tp[2].z));
  float DA, DB, DC;
  plane_const(depths, xpv, ypv, rconst, &DA, &DB, &DC);
  float dmx = fma_(DA, x + 1.0f, fma_(DB, y, DC));
  float dmy = fma_(DA, x, fma_(DB, y + 1.0f, DC));
  float hw = (float)v.W / 2.0f, hh = (float)v.H / 2.0f;
  f3 lmx = mk3(fdiv((x + 1.0f) - hw, v.fov), fdiv(y - hh, v.fov), 1.0f);
  f3 lmy = mk3(fdiv(x - hw, v.fov), fdiv((y + 1.0f) - hh, v.fov), 1.0f);
  lmx = mk3(fdiv(lmx.x, dmx), fdiv(lmx.y, dmx), fdiv(lmx.z, dmx));
  lmy = mk3(fdiv(lmy.x, dmy), fdiv(lmy.y, dmy), fdiv(lmy.z, dmy));
  f3 zero = mk3(0, 0, 0);
  f3 wp = v3(G.world_pos);
  f4 q = v4(G.world_rot_quat);
  f3 gmx = back_rot_quat(sub3(add3(back_rot_cs(lmx, zero, v.crot_c, v.crot_s), v.cpos), wp), q);
  f3 gmy = back_rot_quat(sub3(add3(back_rot_cs(lmy, zero, v.crot_c, v.crot_s), v.cpos), wp), q);
  float lx1, lx2, lx3, ly1, ly2, ly3;
  barycentric(gmx, p1, p2, p3, &lx1, &lx2, &lx3);
  barycentric(gmy, p1, p2, p3, &ly1, &ly2, &ly3);
  f2 vtx = mk2(fma_(vt1.x, lx1, fma_(vt2.x, lx2, vt3.x * lx3)),
               fma_(vt1.y, lx1, fma_(vt2.y, lx2, vt3.y * lx3)));
  f2 vty = mk2(fma_(vt1.x, ly1, fma_(vt2.x, ly2, vt3.x * ly3)),
               fma_(vt1.y, ly1, fma_(vt2.y, ly2, vt3.y * ly3)));
  f2 vdx = mk2(fabsf(vtx.x - vt.x), fabsf(vtx.y - vt.y));
  f2 vdy = mk2(fabsf(vty.x - vt.x), fabsf(vty.y - vt.y));
  const float mip_bias = 1.0f / kMipBias;
  return mk2((vdx.x + vdy.x) * mip_bias, (vdx.y + vdy.y) * mip_bias);
}

float depth_to_dist(uint32_t d) { return fdiv((float)d, kMulInt) * kDepthFar; }

float generate_ssao(int x, int y, const uint32_t* depth, const ShadeView& v) {
  uint32_t seed1 = wang_hash((uint32_t)x + (uint32_t)v.W * (uint32_t)v.H * (uint32_t)y);
  uint32_t seed2 = rand_xorshift(seed1);
  float foffset = fdiv((float)seed2, kMulInt);
  float dep = depth_to_dist(depth[(size_t)y * v.W + x]);
  float rad = kSsaoRad;
  rad += fdiv(foffset, 2.0f);
  float world_rad = fdiv(rad * v.fov, dep);
  const int samples = 2;
  float acc = 0.0f;
  for (int yy = -samples; yy <= samples; yy++) {
    for (int xx = -samples; xx <= samples; xx++) {
      float ox = roundf((float)xx * world_rad), oy = roundf((float)yy * world_rad);
      float wx = (float)x + ox, wy = (float)y + oy;
      wx = clampf_(wx, 1.0f, (float)v.W - 2.0f);
      wy = clampf_(wy, 1.0f, (float)v.H - 2.0f);
      // views 1 or 2 pixels wide (high): [1, n - 2] is empty and the
      // reference reads outside its buffer; pinned to the view's edge (0)
      const int ix = std::max((int)wx, 0), iy = std::max((int)wy, 0);
      float d2 = depth_to_dist(depth[(size_t)iy * v.W + ix]);
      for (float z = -samples; z <= samples; z += 1.0f)
        if (d2 > dep + z) acc += 1.0f;
    }
  }
  acc = fdiv(acc, 125.0f);
  return 1.0f - fdiv(1.0f - acc, kSsaoDiv);
}

// generate_outline (cl2.cl:2315-2362)
float generate_outline(int x, int y, const uint32_t* depth_buffer, const ShadeView& v) {
  float depth = depth_to_dist(depth_buffer[(size_t)y * v.W + x]);
  float furthest = depth;
  const int rad = 1;
  for (int xx = -rad; xx <= rad; xx++) {
    int px = x + xx, py = y;
    if (px < 0 || px >= v.W || py < 0 || py >= v.H) continue;
    float new_depth = depth_to_dist(depth_buffer[(size_t)py * v.W + px]);
    if (new_depth > furthest) furthest = new_depth;
  }
  for (int yy = -rad; yy <= rad; yy++) {
    int px = x, py = y + yy;
    if (px < 0 || px >= v.W || py < 0 || py >= v.H) continue;
    uint32_t d = depth_buffer[(size_t)py * v.W + px];
    float new_depth = depth_to_dist(d);
    if (fabsf(new_depth - depth) > fabsf(furthest - depth) && new_depth > kDepthCutoff && d != 0) furthest = new_depth;
  }
  float diff = fabsf(furthest - depth);
  return fmin_(fdiv(diff, 100.f), 1.f);
}

float bilinear_interpolate(float cx, float cy, const float val[4]) {
  float mx = cx - 0.5f, my = cy - 0.5f;
  float ux = mx - floorf(mx), uy = my - floorf(my);
  float bx = 1.0f - ux, by = 1.0f - uy;
  return (val[0] * bx + val[1] * ux) * by + (val[2] * bx + val[3] * ux) * uy;
}

float hard_occlusion(f3 lpos, f3 normal, f3 ptl, const uint32_t* buf, int face, f3 gpos,
                     int shnum, const ShadeView& v) {
  ptl = fast_normalize3(ptl);
  f3 local = rot_cs(gpos, lpos, v.face_c[face], v.face_s[face]);
  f3 post = depth_project1(local, (float)kLightBufferDim, (float)kLightBufferDim, kLFov);
  float dpth = post.z;
  const uint32_t* map = buf + (size_t)(face + shnum * 6) * kLightBufferDim * kLightBufferDim;
  float px = clampf_(post.x, 3.0f, kLightBufferDim - 4.0f);
  float py = clampf_(post.y, 3.0f, kLightBufferDim - 4.0f);
  int ix = f2i_sat(px), iy = f2i_sat(py);
  float acos_res = rational_acos(clampf_(dot3(normal, ptl), 0.05f, 0.95f));
  float bias = kShadowBias * gbr_tanf(acos_res);
  bias = clampf_(bias, 0.1f * kShadowBias, kShadowBias);
  float cond[16];
  for (int yy = -1; yy <= 2; yy++)
    for (int xx = -1; xx <= 2; xx++) {
      float ldp = depth_to_dist(map[(iy + yy) * kLightBufferDim + ix + xx]);
      cond[(yy + 1) * 4 + xx + 1] = dpth > ldp + bias ? 1.0f : 0.0f;
    }
  float shadow = 0.0f;
  for (int yy = -1; yy <= 1; yy++)
    for (int xx = -1; xx <= 1; xx++) {
      float val[4] = {cond[(yy + 1) * 4 + xx + 1], cond[(yy + 1) * 4 + xx + 2],
                      cond[(yy + 2) * 4 + xx + 1], cond[(yy + 2) * 4 + xx + 2]};
      shadow += bilinear_interpolate((px + 0.5f) + (float)xx, (py + 0.5f) + (float)yy, val);
    }
  return fdiv(shadow, 9.0f);
}

struct ShadeIn {
  const gbr_triangle* tris;
  const gbr_obj_g_descriptor* descs;
  const gbr_light* lights;
  uint32_t nlights;
  Atlas atlas;
  const uint32_t* shadow_dyn;
  const uint32_t* shadow_static;
};

f4 vertex_col(uint32_t c) {
  f4 r;
  r.x = fdiv((float)(c >> 24), 255.f);
  r.y = fdiv((float)((c >> 16) & 0xFF), 255.f);
  r.z = fdiv((float)((c >> 8) & 0xFF), 255.f);
  r.w = fdiv((float)(c & 0xFF), 255.f);
  return r;
}

void kernel3_pixel(int x, int y, const ShadeView& v, const ShadeIn& in, const Setup& S,
                   const uint32_t* depth, const uint32_t* ids, uint8_t* rgba, uint16_t* normals) {
  size_t p = (size_t)y * v.W + x;
  uint32_t d = depth[p];
  uint32_t key = ids[p];
  auto put = [&](float r, float g, float b, float a) {
    rgba[p * 4 + 0] = (uint8_t)quant8(r);
    rgba[p * 4 + 1] = (uint8_t)quant8(g);
    rgba[p * 4 + 2] = (uint8_t)quant8(b);
    rgba[p * 4 + 3] = (uint8_t)quant8(a);
  };
  if (d == kDepthClear || key == kNoId) {
    float c[3] = {v.clear.x, v.clear.y, v.clear.z};
    if (blend_over(v, p, d, c))
      put(c[0], c[1], c[2], c[2]);  // the reference's .xyzz: alpha = blue
    else
      put(v.clear.x, v.clear.y, v.clear.z, v.clear.w);
    if (normals) { normals[p * 2] = 0; normals[p * 2 + 1] = 0; }
    return;
  }
  uint32_t tri = key >> 1;
  const Cut& ct = S.cut[key];
  float rconst = S.rconst[key];
  const gbr_triangle& T = in.tris[tri];
  uint32_t o_id = T.vertices[0].object_id;
  const gbr_obj_g_descriptor& G = in.descs[o_id];
  f3 p1 = mul3s(v3(T.vertices[0].pos), G.scale);
  f3 p2 = mul3s(v3(T.vertices[1].pos), G.scale);
  f3 p3 = mul3s(v3(T.vertices[2].pos), G.scale);
  f2 vt1 = mk2(T.vertices[0].vt[0], T.vertices[0].vt[1]);
  f2 vt2 = mk2(T.vertices[1].vt[0], T.vertices[1].vt[1]);
  f2 vt3 = mk2(T.vertices[2].vt[0], T.vertices[2].vt[1]);
  f3 n1 = v3(T.vertices[0].normal), n2 = v3(T.vertices[1].normal), n3 = v3(T.vertices[2].normal);
  float ldepth = depth_to_dist(d);
  f3 local = mk3(fdiv(((float)x - (float)v.W / 2.0f) * ldepth, v.fov),
                 fdiv(((float)y - (float)v.H / 2.0f) * ldepth, v.fov), ldepth);
  f3 zero = mk3(0, 0, 0);
  f3 gpos = add3(back_rot_cs(local, zero, v.crot_c, v.crot_s), v.cpos);
  f4 q = v4(G.world_rot_quat);
  f3 olocal = back_rot_quat(sub3(gpos, v3(G.world_pos)), q);
  float l1, l2, l3;
  barycentric(olocal, p1, p2, p3, &l1, &l2, &l3);
  f2 vt = mk2(fma_(vt1.x, l1, fma_(vt2.x, l2, vt3.x * l3)),
              fma_(vt1.y, l1, fma_(vt2.y, l2, vt3.y * l3)));
  f3 normal = mk3(fma_(n1.x, l1, fma_(n2.x, l2, n3.x * l3)), fma_(n1.y, l1, fma_(n2.y, l2, n3.y * l3)),
                  fma_(n1.z, l1, fma_(n2.z, l2, n3.z * l3)));
  const f3 model_normal = normal;
  normal = rot_quat(normal, q);
  f4 col;
  bool has_col = T.vertices[0].vertex_col != 0;
  // kernel3 computes vtdiff for every pixel; the texture and the normal map read it
  const bool normal_mapped = (v.flags & GBR_VIEW_NORMAL_MAPPING) && G.rid != 0xFFFFFFFFu;
  f2 vtdiff = mk2(0.0f, 0.0f);
  if (!has_col || normal_mapped)
    vtdiff = get_vtdiff(ct.p, (float)x, (float)y, v, G, vt, p1, p2, p3, vt1, vt2, vt3, rconst);
  if (has_col) {
    f4 c0 = vertex_col(T.vertices[0].vertex_col), c1 = vertex_col(T.vertices[1].vertex_col),
       c2 = vertex_col(T.vertices[2].vertex_col);
    col.x = fma_(c0.x, l1, fma_(c1.x, l2, c2.x * l3));
    col.y = fma_(c0.y, l1, fma_(c1.y, l2, c2.y * l3));
    col.z = fma_(c0.z, l1, fma_(c1.z, l2, c2.z * l3));
    col.w = fma_(c0.w, l1, fma_(c1.w, l2, c2.w * l3));
  } else {
    col = texture_filter_diff(vt, vtdiff, (int)G.tid, in.atlas);
  }
  if (v.use_linear) {
    col.x = gamma_fwd(col.x);
    col.y = gamma_fwd(col.y);
    col.z = gamma_fwd(col.z);
  }
  uint32_t seed1 = wang_hash((uint32_t)x + (uint32_t)y * (uint32_t)v.W * (uint32_t)v.H);
  uint32_t seed2 = rand_xorshift(seed1);
  uint32_t seed3 = rand_xorshift(seed2);
  uint32_t seed4 = rand_xorshift(seed3);
  f3 rseed = mk3((fdiv((float)seed2, kMulInt) - 0.5f) * 2.0f, (fdiv((float)seed3, kMulInt) - 0.5f) * 2.0f,
                 (fdiv((float)seed4, kMulInt) - 0.5f) * 2.0f);
  if (normal_mapped) {
    // ENABLE_NORMAL_MAPPING (cl2.cl:5987-6027)
    f4 t4 = texture_filter_diff(vt, vtdiff, (int)G.rid, in.atlas);
    f3 t_normal = mk3(2.f * t4.x - 1.f, 2.f * t4.y - 1.f, 2.f * t4.z - 1.f);
    t_normal = fast_normalize3(t_normal);  // normalize, pinned as fast_normalize
    f3 deltaPos1 = sub3(p2, p1), deltaPos2 = sub3(p3, p1);
    f2 deltaUV1 = mk2(vt2.x - vt1.x, vt2.y - vt1.y), deltaUV2 = mk2(vt3.x - vt1.x, vt3.y - vt1.y);
    float r = fdiv(1.0f, deltaUV1.x * deltaUV2.y - deltaUV1.y * deltaUV2.x);
    f3 tangent = mul3s(sub3(mul3s(deltaPos1, deltaUV2.y), mul3s(deltaPos2, deltaUV1.y)), r);
    f3 bitangent = mul3s(sub3(mul3s(deltaPos2, deltaUV1.x), mul3s(deltaPos1, deltaUV2.x)), r);
    tangent = fast_normalize3(tangent);
    bitangent = fast_normalize3(bitangent);
    tangent = fast_normalize3(sub3(tangent, mul3s(model_normal, dot3(model_normal, tangent))));
    if (dot3(cross3(model_normal, tangent), bitangent) < 0.0f) tangent = mul3s(tangent, -1.0f);
    f3 model_space = mk3(tangent.x * t_normal.x + bitangent.x * t_normal.y + model_normal.x * t_normal.z,
                         tangent.y * t_normal.x + bitangent.y * t_normal.y + model_normal.y * t_normal.z,
                         tangent.z * t_normal.x + bitangent.z * t_normal.y + model_normal.z * t_normal.z);
    normal = rot_quat(model_space, q);
  }
  f3 l2p = fast_normalize3(sub3(v.cpos, gpos));
  int ff = G.feature_flag;
  bool two = (ff & kFlagTwoSided) > 0;
  bool recv_dyn = !((ff & kFlagNoDynShadows) > 0);
  int is_front = backface_front(ct.p[0], ct.p[1], ct.p[2]);
  if (!is_front && two) normal = neg3(normal);
  float ssao = generate_ssao(x, y, depth, v);
  normal = fast_normalize3(normal);
  f3 lnormal = fast_normalize3(add3(normal, mk3(fdiv(rseed.x, 100.f), fdiv(rseed.y, 100.f), fdiv(rseed.z, 100.f))));
  float ambient = v.use_linear ? gamma_fwd(kAmbient) : kAmbient;
  f3 diffuse_sum = mk3(0, 0, 0), specular_sum = mk3(0, 0, 0);
  int shnum = 0, static_num = 0;
  for (uint32_t i = 0; i < in.nlights; i++) {
    const gbr_light& L = in.lights[i];
    f3 lpos = v3(L.pos);
    f3 ptl = sub3(lpos, gpos);
    float occlusion = 1.0f;
    if (L.shadow && L.is_static) {
      int face = ret_cubeface(gpos, lpos);
      occlusion = 1.0f - hard_occlusion(lpos, normal, ptl, in.shadow_static, face, gpos, static_num, v);
      static_num++;
    }
    float distance = fast_length3(ptl);
    float tt = fdiv(distance, L.radius) + 1.0f;
    float illum = fdiv(L.brightness, tt * tt);
    const float cutoff = 0.1f;
    illum -= cutoff;
    illum *= fdiv(1.0f, 1.0f - cutoff);
    if (illum <= 0) continue;
    f3 lcol = v3(L.col);
    if (v.use_linear) lcol = mk3(gamma_fwd(lcol.x), gamma_fwd(lcol.y), gamma_fwd(lcol.z));
    if (L.shadow && recv_dyn) {
      int face = ret_cubeface(gpos, lpos);
      float dyn = 1.0f - hard_occlusion(lpos, normal, ptl, in.shadow_dyn, face, gpos, shnum, v);
      occlusion = fmin_(occlusion, dyn);
      shnum++;
    }
    ptl = fast_normalize3(ptl);
    float light = dot3(ptl, lnormal);
    light *= occlusion;
    light = fmax_(light, 0.0f);
    float diffuse = (1.0f - ambient) * light;
    float dscale = (((diffuse + ambient) * L.diffuse) * G.diffuse) * illum;
    diffuse_sum = add3(diffuse_sum, mul3s(lcol, dscale));
    f3 H = fast_normalize3(add3(l2p, ptl));
    f3 N = normal;
    const float kS = 0.4f;
    float ndh = fmax_(0.0f, dot3(N, H));
    float ndv = fmax_(0.0f, dot3(N, l2p));
    float vdh = fmax_(0.0f, dot3(l2p, H));
    float ndl = fmax_(0.0f, dot3(N, ptl));
    const float F0 = 0.4f;
    float fresnel = F0 + (1.0f - F0) * powf(1.0f - vdh, 5.0f);
    float rough = clampf_(1.0f - G.specular, 0.001f, 10.0f);
    float alpha = rational_acos(ndh);
    float microfacet = 0.8346f * expf(fdiv((-alpha) * alpha, rough * rough));
    float sv = fdiv(2.0f * ndh, vdh);
    float c1 = sv * ndv, c2 = sv * ndl;
    float geometric = min3f(1.0f, c1, c2);
    float spec = fdiv((fresnel * microfacet) * geometric, kPi * ndv);
    float sscale = (spec * kS) * illum;
    f3 sp = mul3s(mul3s(lcol, sscale), G.spec_mult);
    specular_sum = add3(specular_sum, sp);
    specular_sum = mk3(fmax_(specular_sum.x, 0.0f), fmax_(specular_sum.y, 0.0f), fmax_(specular_sum.z, 0.0f));
    specular_sum = mul3s(specular_sum, occlusion);
  }
  specular_sum = mul3s(specular_sum, ssao);
  diffuse_sum = mul3s(diffuse_sum, ssao);
  const float rsc = 0.7f;
  f3 colclamp = add3(add3(mk3(col.x, col.y, col.z), mk3(0, 0, 0)), mul3s(specular_sum, rsc));
  f3 sp2 = mul3s(specular_sum, 1.0f - rsc);
  f3 fin = mk3(fma_(colclamp.x, diffuse_sum.x, sp2.x), fma_(colclamp.y, diffuse_sum.y, sp2.y),
               fma_(colclamp.z, diffuse_sum.z, sp2.z));
  {
    float c[3] = {fin.x, fin.y, fin.z};
    if (blend_over(v, p, d, c)) fin = mk3(c[0], c[1], c[2]);
  }
  if (v.use_linear) fin = mk3(gamma_inv(fin.x), gamma_inv(fin.y), gamma_inv(fin.z));
  if ((v.flags & GBR_VIEW_OUTLINE) && (ff & kFlagOutline) > 0) {
    // CAN_OUTLINE (cl2.cl:6368-6373)
    float outline = generate_outline(x, y, depth, v);
    fin = mk3(fin.x + outline, fin.y + outline, fin.z + outline);
  }
  put(fin.x, fin.y, fin.z, col.w);
  if (normals) {
    float nx = normal.x, ny = normal.y, nz = normal.z;
    float len_sq = nx * nx + ny * ny;
    if (len_sq < 0.0001f) nx = 0.01f;
    float l = fsqrt(nx * nx + ny * ny);
    float sq = fsqrt(fmax_(nz * 0.5f + 0.5f, 0.0f));
    float rx = fdiv(nx, l) * sq, ry = fdiv(ny, l) * sq;
    float ex = fdiv(rx + 1.0f, 2.0f) * 65536.0f - 1.0f;
    float ey = fdiv(ry + 1.0f, 2.0f) * 65536.0f - 1.0f;
    normals[p * 2] = (uint16_t)std::min<uint32_t>(f2u_sat(ex), 65535u);
    normals[p * 2 + 1] = (uint16_t)std::min<uint32_t>(f2u_sat(ey), 65535u);
  }
}

// ---- FP64 shading reference ------------------------------------------------
// kernel3 (cl2.cl:5792-6408) evaluated in double precision with exact library
// functions (sqrt, exp, pow, tan, division) where the float pipeline uses the
// vendor's native_* approximations or float rounding.  The reference's own
// formula approximations stay (rational_acos unless exact_acos, the sRGB
// polynomials, log2_approx), so the difference to this is the floating-point
// error of a float implementation.  Inputs: the same depth, canonical id,
// clipped triangles, atlas and cubemaps as the float path.
struct D3 { double x, y, z; };
struct D4 { double x, y, z, w; };
inline D3 d3(double x, double y, double z) { return D3{x, y, z}; }
inline D3 d3f(f3 a) { return D3{a.x, a.y, a.z}; }
inline D3 d3p(const float* p) { return D3{p[0], p[1], p[2]}; }
inline D3 operator+(D3 a, D3 b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline D3 operator-(D3 a, D3 b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline D3 operator*(D3 a, double s) { return d3(a.x * s, a.y * s, a.z * s); }
inline double dotd(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 crossd(D3 a, D3 b) { return d3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline D3 normd(D3 a) { return a * (1.0 / std::sqrt(dotd(a, a))); }
inline double clampd(double x, double lo, double hi) { return std::fmin(std::fmax(x, lo), hi); }

struct CamD { D3 c, s; };
inline CamD camd(f3 ang) {
  return CamD{d3(std::cos((double)ang.x), std::cos((double)ang.y), std::cos((double)ang.z)),
              d3(std::sin((double)ang.x), std::sin((double)ang.y), std::sin((double)ang.z))};
}
// rot / back_rot (cl2.cl:220-348) in double
inline D3 rotd(D3 p, D3 cpos, const CamD& k) {
  D3 r = p - cpos, c = k.c, s = k.s;
  double a = s.z * r.y + c.z * r.x, b = c.y * r.z + s.y * a, d = c.z * r.y - s.z * r.x;
  return d3(c.y * a - s.y * r.z, s.x * b + c.x * d, c.x * b - s.x * d);
}
inline D3 back_rotd(D3 p, D3 cpos, const CamD& k) {
  D3 r = p - cpos, c = k.c, s = k.s;
  return d3(c.z * (c.y * r.x + s.x * s.y * r.y + c.x * s.y * r.z) + s.z * (s.x * r.z - c.x * r.y),
            s.z * c.y * r.x + (c.x * c.z + s.x * s.y * s.z) * r.y + (-s.x * c.z + c.x * s.y * s.z) * r.z,
            -s.y * r.x + c.y * (s.x * r.y + c.x * r.z));
}
inline D4 qnormd(D4 q) {
  double l = std::sqrt(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
  return D4{q.x / l, q.y / l, q.z / l, q.w / l};
}
inline D3 rot_quatd(D3 p, D4 q) {  // q normalised
  D3 qv = d3(q.x, q.y, q.z);
  D3 t = crossd(qv, p) * 2.0;
  return p + t * q.w + crossd(qv, t);
}
inline D4 qinvd(D4 q) { return qnormd(D4{-q.x, -q.y, -q.z, q.w}); }
inline void baryd(D3 p, D3 a, D3 b, D3 c, double* u, double* v, double* w) {
  D3 v0 = b - a, v1 = c - a, v2 = p - a;
  double d00 = dotd(v0, v0), d01 = dotd(v0, v1), d11 = dotd(v1, v1), d20 = dotd(v2, v0), d21 = dotd(v2, v1);
  double den = d00 * d11 - d01 * d01;
  *v = (d11 * d20 - d01 * d21) / den;
  *w = (d00 * d21 - d01 * d20) / den;
  *u = 1.0 - *v - *w;
}
inline double gamma_fwd_d(double c) { return 0.012522878 * c + 0.682171111 * c * c + 0.305306011 * c * c * c; }
inline double gamma_inv_d(double c) {
  double s1 = std::sqrt(c), s2 = std::sqrt(s1), s3 = std::sqrt(s2);
  return 0.585122381 * s1 + 0.783140355 * s2 - 0.368262736 * s3;
}
inline double rational_acos_d(double x, bool exact) {
  if (exact) return std::acos(x);
  const double a = -0.939115566365855, b = 0.9217841528914573, c = -1.2845906244690837, d = 0.295624144969963174;
  return 3.14159265358979323846 / 2.0 + (a * x + b * x * x * x) / (1.0 + c * x * x + d * x * x * x * x);
}
// log2_approx (cl2.cl:1498-1505): exponent plus a quadratic in the mantissa
inline double log2_approx_d(double v) {
  int e = 0;
  double f = std::frexp(v, &e);  // v = f * 2^e, f in [0.5, 1)
  double m = 2.0 * f;            // mantissa in [1, 2)
  return (double)(e - 2) + ((-0.3358287811 * m + 2.0) * m - 0.65871759316667);
}
inline double depth_to_dist_d(uint32_t d) { return (double)d / 4294967296.0 * 350000.0; }

D4 read_tex_d(double cx, double cy, int which, int slice, double width, const Atlas& at) {
  const int hnum = kTexPage / (int)width;
  const int tny = which / hnum, tnx = which - tny * hnum;
  cx = clampd(cx, 0.001, width - 0.001);
  cy = clampd(cy, 0.001, width - 0.001);
  int ix = (int)(tnx * width + cx), iy = (int)(tny * width + cy);
  const uint8_t* t = at.data + ((size_t)slice * kTexPage * kTexPage + (size_t)iy * kTexPage + ix) * 4;
  return D4{(double)t[0], (double)t[1], (double)t[2], (double)t[3]};
}
D4 bilinear_d(double mx, double my, int which, int slice, double width, const Atlas& at) {
  double px = std::floor(mx), py = std::floor(my);
  D4 c0 = read_tex_d(px, py, which, slice, width, at), c1 = read_tex_d(px + 1, py, which, slice, width, at);
  D4 c2 = read_tex_d(px, py + 1, which, slice, width, at), c3 = read_tex_d(px + 1, py + 1, which, slice, width, at);
  double ux = mx - px, uy = my - py, bx = 1 - ux, by = 1 - uy;
  auto mix = [&](double a, double b, double c, double d) { return (a * bx + b * ux) * by + (c * bx + d * ux) * uy; };
  return D4{mix(c0.x, c1.x, c2.x, c3.x), mix(c0.y, c1.y, c2.y, c3.y), mix(c0.z, c1.z, c2.z, c3.z),
            mix(c0.w, c1.w, c2.w, c3.w)};
}
inline double tex_mod_d(double v) {
  v = v >= 1.0 ? 1.0 - (v - std::floor(v)) : v;
  v = v < 0.0 ? (1.0 + std::fabs(v)) - std::fabs(std::floor(v)) : v;
  return v;
}
D4 texture_filter_d(double vtx, double vty, double dx, double dy, int tid2, const Atlas& at) {
  uint32_t nv = at.nums[tid2];
  int slice = (int)(nv >> 16);
  double tsize = (double)at.sizes[slice];
  double mx = tex_mod_d(vtx), my = tex_mod_d(vty);
  double wx = dx * tsize, wy = dy * tsize;
  double worst = std::sqrt(wx * wx + wy * wy);
  double wif = std::fmax(log2_approx_d(worst), 0.0);
  double lower = clampd(std::floor(wif), 0.0, (double)kMipLevels);
  double fmd = wif - lower;
  int tl = lower == 0.0 ? tid2 : (int)((lower - 1.0) + at.mipmap_start + tid2 * kMipLevels);
  int th = (int)(clampd(lower, 0.0, kMipLevels - 1.0) + at.mipmap_start + tid2 * kMipLevels);
  uint32_t lnv = at.nums[tl], hnv = at.nums[th];
  int sl = (int)(lnv >> 16), sh = (int)(hnv >> 16);
  double szl = at.sizes[sl], szh = at.sizes[sh];
  D4 c1 = bilinear_d(mx * szl, my * szl, (int)(lnv & 0xFFFF), sl, szl, at);
  D4 c2 = bilinear_d(mx * szh, my * szh, (int)(hnv & 0xFFFF), sh, szh, at);
  return D4{(c1.x + (c2.x - c1.x) * fmd) / 255.0, (c1.y + (c2.y - c1.y) * fmd) / 255.0,
            (c1.z + (c2.z - c1.z) * fmd) / 255.0, (c1.w + (c2.w - c1.w) * fmd) / 255.0};
}
inline int ret_cubeface_d(D3 p, D3 l) {
  D3 r = p - l;
  double ax = std::fabs(r.x), ay = std::fabs(r.y), az = std::fabs(r.z);
  if (ax >= ay && ax >= az) return r.x < 0.0 ? 4 : 5;
  if (ay > ax && ay >= az) return r.y < 0.0 ? 1 : 3;
  if (az > ax && az > ay && r.z < 0.0) return 2;
  return 0;
}
double hard_occlusion_d(D3 lpos, D3 normal, D3 ptl, const uint32_t* buf, int face, D3 gpos, int shnum,
                        const CamD* faces, bool exact_acos) {
  ptl = normd(ptl);
  D3 local = rotd(gpos, lpos, faces[face]);
  const double L = kLightBufferDim;
  double k = 512.0 / local.z;
  double px = local.x * k + L / 2, py = local.y * k + L / 2, dpth = local.z;
  const uint32_t* map = buf + (size_t)(face + shnum * 6) * kLightBufferDim * kLightBufferDim;
  px = clampd(px, 3.0, L - 4.0);
  py = clampd(py, 3.0, L - 4.0);
  int ix = (int)px, iy = (int)py;
  double ac = rational_acos_d(clampd(dotd(normal, ptl), 0.05, 0.95), exact_acos);
  double bias = clampd(50.0 * std::tan(ac), 5.0, 50.0);
  double cond[16];
  for (int yy = -1; yy <= 2; yy++)
    for (int xx = -1; xx <= 2; xx++)
      cond[(yy + 1) * 4 + xx + 1] =
          dpth > depth_to_dist_d(map[(iy + yy) * kLightBufferDim + ix + xx]) + bias ? 1.0 : 0.0;
  double sh = 0.0;
  for (int yy = -1; yy <= 1; yy++)
    for (int xx = -1; xx <= 1; xx++) {
      double cx = px + 0.5 + xx, cy = py + 0.5 + yy;
      double mx = cx - 0.5, my = cy - 0.5, ux = mx - std::floor(mx), uy = my - std::floor(my);
      int b = (yy + 1) * 4 + xx + 1;
      sh += (cond[b] * (1 - ux) + cond[b + 1] * ux) * (1 - uy) + (cond[b + 4] * (1 - ux) + cond[b + 5] * ux) * uy;
    }
  return sh / 9.0;
}

void kernel3_pixel_fp64(int x, int y, const ShadeView& v, const ShadeIn& in, const Setup& S,
                        const uint32_t* depth, const uint32_t* ids, bool exact_acos, double* out) {
  const size_t p = (size_t)y * v.W + x;
  const uint32_t d = depth[p], key = ids[p];
  double* o = out + p * 4;
  auto blend_d = [&](double c[3]) {
    if (!v.blend_depth || !(v.blend_depth[p] < d)) return false;
    double b[4];
    for (int k = 0; k < 4; k++) b[k] = v.blend_rgba[4 * p + k] / 255.0;
    for (int k = 0; k < 3; k++) c[k] = b[k] * b[3] + c[k] * (1.0 - b[3]);
    return true;
  };
  if (d == kDepthClear || key == kNoId) {
    double c[3] = {v.clear.x, v.clear.y, v.clear.z};
    const bool bl = blend_d(c);
    o[0] = clampd(c[0], 0, 1); o[1] = clampd(c[1], 0, 1);
    o[2] = clampd(c[2], 0, 1); o[3] = clampd(bl ? c[2] : v.clear.w, 0, 1);
    return;
  }
  const uint32_t tri = key >> 1;
  const Cut& ct = S.cut[key];
  const gbr_triangle& T = in.tris[tri];
  const gbr_obj_g_descriptor& G = in.descs[T.vertices[0].object_id];
  const CamD cam = camd(v.crot);
  CamD faces[6];
  for (int f = 0; f < 6; f++) faces[f] = camd(face_angles(f));
  const double fov = v.fov, W = v.W, H = v.H;
  const D3 cpos = d3f(v.cpos), wpos = d3p(G.world_pos);
  const D4 q = qnormd(D4{G.world_rot_quat[0], G.world_rot_quat[1], G.world_rot_quat[2], G.world_rot_quat[3]});
  const D4 qi = qinvd(D4{G.world_rot_quat[0], G.world_rot_quat[1], G.world_rot_quat[2], G.world_rot_quat[3]});
  const D3 p1 = d3p(T.vertices[0].pos) * G.scale, p2 = d3p(T.vertices[1].pos) * G.scale,
           p3 = d3p(T.vertices[2].pos) * G.scale;
  const double ld = depth_to_dist_d(d);
  const D3 gpos = back_rotd(d3((x - W / 2) * ld / fov, (y - H / 2) * ld / fov, ld), d3(0, 0, 0), cam) + cpos;
  double l1, l2, l3;
  baryd(rot_quatd(gpos - wpos, qi), p1, p2, p3, &l1, &l2, &l3);
  auto interp2 = [&](int c, double a, double b, double cc) {
    return T.vertices[0].vt[c] * a + T.vertices[1].vt[c] * b + T.vertices[2].vt[c] * cc;
  };
  const double vtx = interp2(0, l1, l2, l3), vty = interp2(1, l1, l2, l3);
  D3 normal = d3p(T.vertices[0].normal) * l1 + d3p(T.vertices[1].normal) * l2 + d3p(T.vertices[2].normal) * l3;
  normal = rot_quatd(normal, q);
  D4 col;
  if (T.vertices[0].vertex_col != 0) {
    D4 acc{0, 0, 0, 0};
    const double w3[3] = {l1, l2, l3};
    for (int k = 0; k < 3; k++) {
      uint32_t c = T.vertices[k].vertex_col;
      acc.x += (c >> 24) / 255.0 * w3[k];
      acc.y += ((c >> 16) & 0xFF) / 255.0 * w3[k];
      acc.z += ((c >> 8) & 0xFF) / 255.0 * w3[k];
      acc.w += (c & 0xFF) / 255.0 * w3[k];
    }
    col = acc;
  } else {
    // get_vtdiff (cl2.cl:5691-5760) in double
    double xp[3], yp[3], dp[3];
    for (int k = 0; k < 3; k++) {
      xp[k] = std::round((double)ct.p[k].x);
      yp[k] = std::round((double)ct.p[k].y);
      dp[k] = 1.0 / (double)ct.p[k].z;
    }
    const double rc = 1.0 / ((xp[1] * yp[2] + xp[0] * (yp[1] - yp[2]) - xp[2] * yp[1]) + (xp[2] - xp[1]) * yp[0]);
    const double A = ((dp[1] * yp[2] + dp[0] * (yp[1] - yp[2]) - dp[2] * yp[1]) + (dp[2] - dp[1]) * yp[0]) * rc;
    const double B = -((dp[1] * xp[2] + dp[0] * (xp[1] - xp[2]) - dp[2] * xp[1]) + (dp[2] - dp[1]) * xp[0]) * rc;
    const double C = dp[0] - A * xp[0] - B * yp[0];
    const double dmx = A * (x + 1) + B * y + C, dmy = A * x + B * (y + 1) + C;
    const D3 lmx = d3((x + 1 - W / 2) / fov / dmx, (y - H / 2) / fov / dmx, 1.0 / dmx);
    const D3 lmy = d3((x - W / 2) / fov / dmy, (y + 1 - H / 2) / fov / dmy, 1.0 / dmy);
    double a1, a2, a3, b1, b2, b3;
    baryd(rot_quatd(back_rotd(lmx, d3(0, 0, 0), cam) + cpos - wpos, qi), p1, p2, p3, &a1, &a2, &a3);
    baryd(rot_quatd(back_rotd(lmy, d3(0, 0, 0), cam) + cpos - wpos, qi), p1, p2, p3, &b1, &b2, &b3);
    const double mb = 1.0 / 1.1;
    const double dx = (std::fabs(interp2(0, a1, a2, a3) - vtx) + std::fabs(interp2(0, b1, b2, b3) - vtx)) * mb;
    const double dy = (std::fabs(interp2(1, a1, a2, a3) - vty) + std::fabs(interp2(1, b1, b2, b3) - vty)) * mb;
    col = texture_filter_d(vtx, vty, dx, dy, (int)G.tid, in.atlas);
  }
  if (v.use_linear) {
    col.x = gamma_fwd_d(col.x);
    col.y = gamma_fwd_d(col.y);
    col.z = gamma_fwd_d(col.z);
  }
  const uint32_t s1 = wang_hash((uint32_t)x + (uint32_t)y * (uint32_t)v.W * (uint32_t)v.H);
  const uint32_t s2 = rand_xorshift(s1), s3 = rand_xorshift(s2), s4 = rand_xorshift(s3);
  const D3 rseed = d3((s2 / 4294967296.0 - 0.5) * 2, (s3 / 4294967296.0 - 0.5) * 2, (s4 / 4294967296.0 - 0.5) * 2);
  const D3 l2p = normd(cpos - gpos);
  const int ff = G.feature_flag;
  const bool two = (ff & kFlagTwoSided) > 0, recv_dyn = !((ff & kFlagNoDynShadows) > 0);
  if (!backface_front(ct.p[0], ct.p[1], ct.p[2]) && two) normal = normal * -1.0;
  // SSAO (cl2.cl:2194-2260)
  double ssao;
  {
    const uint32_t ss2 = rand_xorshift(wang_hash((uint32_t)x + (uint32_t)v.W * (uint32_t)v.H * (uint32_t)y));
    const double dep = depth_to_dist_d(d);
    const double wr = (2.0 + (ss2 / 4294967296.0) / 2.0) * fov / dep;
    double acc = 0;
    for (int yy = -2; yy <= 2; yy++)
      for (int xx = -2; xx <= 2; xx++) {
        int wx = std::max((int)clampd(x + std::round(xx * wr), 1.0, W - 2.0), 0);
        int wy = std::max((int)clampd(y + std::round(yy * wr), 1.0, H - 2.0), 0);
        double d2 = depth_to_dist_d(depth[(size_t)wy * v.W + wx]);
        for (int z = -2; z <= 2; z++) acc += d2 > dep + z ? 1.0 : 0.0;
      }
    ssao = 1.0 - (1.0 - acc / 125.0) / 2.5;
  }
  normal = normd(normal);
  const D3 lnormal = normd(normal + rseed * 0.01);
  const double ambient = v.use_linear ? gamma_fwd_d(0.2) : 0.2;
  const double rough = clampd(1.0 - G.specular, 0.001, 10.0);
  D3 dsum = d3(0, 0, 0), ssum = d3(0, 0, 0);
  int shnum = 0, static_num = 0;
  for (uint32_t i = 0; i < in.nlights; i++) {
    const gbr_light& L = in.lights[i];
    const D3 lpos = d3p(L.pos);
    D3 ptl = lpos - gpos;
    double occ = 1.0;
    if (L.shadow && L.is_static) {
      occ = 1.0 - hard_occlusion_d(lpos, normal, ptl, in.shadow_static, ret_cubeface_d(gpos, lpos), gpos,
                                   static_num, faces, exact_acos);
      static_num++;
    }
    const double dist = std::sqrt(dotd(ptl, ptl));
    const double tt = dist / L.radius + 1.0;
    double illum = (L.brightness / (tt * tt) - 0.1) / 0.9;
    if (illum <= 0) continue;
    D3 lcol = d3p(L.col);
    if (v.use_linear) lcol = d3(gamma_fwd_d(lcol.x), gamma_fwd_d(lcol.y), gamma_fwd_d(lcol.z));
    if (L.shadow && recv_dyn) {
      double dyn = 1.0 - hard_occlusion_d(lpos, normal, ptl, in.shadow_dyn, ret_cubeface_d(gpos, lpos), gpos,
                                          shnum, faces, exact_acos);
      occ = std::fmin(occ, dyn);
      shnum++;
    }
    ptl = normd(ptl);
    const double light = std::fmax(dotd(ptl, lnormal) * occ, 0.0);
    const double dscale = (((1.0 - ambient) * light + ambient) * L.diffuse) * G.diffuse * illum;
    dsum = dsum + lcol * dscale;
    const D3 Hv = normd(l2p + ptl);
    const double ndh = std::fmax(0.0, dotd(normal, Hv)), ndv = std::fmax(0.0, dotd(normal, l2p));
    const double vdh = std::fmax(0.0, dotd(l2p, Hv)), ndl = std::fmax(0.0, dotd(normal, ptl));
    const double fresnel = 0.4 + 0.6 * std::pow(1.0 - vdh, 5.0);
    const double alpha = rational_acos_d(ndh, exact_acos);
    const double micro = 0.8346 * std::exp(-alpha * alpha / (rough * rough));
    const double sv = 2.0 * ndh / vdh;
    const double geom = std::fmin(std::fmin(1.0, sv * ndv), sv * ndl);
    const double spec = fresnel * micro * geom / (3.14159265358979323846 * ndv);
    ssum = ssum + lcol * (spec * 0.4 * illum * G.spec_mult);
    ssum = d3(std::fmax(ssum.x, 0.0), std::fmax(ssum.y, 0.0), std::fmax(ssum.z, 0.0)) * occ;
  }
  ssum = ssum * ssao;
  dsum = dsum * ssao;
  D3 fin = d3((col.x + ssum.x * 0.7) * dsum.x + ssum.x * 0.3, (col.y + ssum.y * 0.7) * dsum.y + ssum.y * 0.3,
              (col.z + ssum.z * 0.7) * dsum.z + ssum.z * 0.3);
  {
    double c[3] = {fin.x, fin.y, fin.z};
    if (blend_d(c)) fin = d3(c[0], c[1], c[2]);
  }
  if (v.use_linear) fin = d3(gamma_inv_d(fin.x), gamma_inv_d(fin.y), gamma_inv_d(fin.z));
  o[0] = clampd(fin.x, 0, 1);
  o[1] = clampd(fin.y, 0, 1);
  o[2] = clampd(fin.z, 0, 1);
  o[3] = clampd(col.w, 0, 1);
}

// ---- shadow cubemaps ---------------------------------------------------------
struct ShadowFrag {
  uint32_t face, a, ctri;
  float rconst;
};

void shadow_light(const gbr_triangle* tris, uint32_t n, const gbr_obj_g_descriptor* descs,
                  f3 lpos, int only_static, uint32_t* out, int nthreads) {
  f3 fc[6], fs[6];
  for (int f = 0; f < 6; f++) euler_cs(face_angles(f), &fc[f], &fs[f]);
  const float L = (float)kLightBufferDim;
  // per triangle and face: up to 2 clip outputs
  std::vector<Cut> cut((size_t)n * 12);
  std::vector<float> nfr((size_t)n * 12, -1.0f);
  std::vector<float> rcs((size_t)n * 12, 0.0f);
  parallel_for(n, nthreads, [&](int64_t id) {
    const gbr_triangle& T = tris[id];
    const gbr_obj_g_descriptor& G = descs[T.vertices[0].object_id];
    int ff = G.feature_flag;
    if (!only_static && (ff & kFlagIsStatic) > 0) return;
    if (only_static && !((ff & kFlagIsStatic) > 0)) return;
    f3 wp = v3(G.world_pos);
    if (fast_length3(sub3(wp, lpos)) > kDepthFar) return;
    f4 q = v4(G.world_rot_quat);
    int skip[6] = {0, 0, 0, 0, 0, 0};
    for (int k = 0; k < 3; k++) {
      f3 r = add3(rot_quat(mul3s(v3(T.vertices[k].pos), G.scale), q), wp);
      skip[ret_cubeface(r, lpos)] = 1;
    }
    bool two = (ff & kFlagTwoSided) > 0;
    for (int f = 0; f < 6; f++) {
      if (!skip[f]) continue;
      f3 out2[2][3];
      int num = project_tri(T, G, lpos, fc[f], fs[f], kLFov, L, L, out2);
      for (int i = 0; i < num; i++) {
        size_t s = (size_t)id * 12 + f * 2 + i;
        cut[s].p[0] = out2[i][0]; cut[s].p[1] = out2[i][1]; cut[s].p[2] = out2[i][2];
        float rc = 0;
        int tn = cull_and_count(cut[s].p, two, L, L, kOpSizeLight, &rc);
        nfr[s] = (float)tn;
        rcs[s] = rc;
      }
    }
  });
  std::vector<ShadowFrag> frags;
  for (size_t s = 0; s < (size_t)n * 12; s++) {
    float tn = nfr[s];
    for (uint32_t a = 0; (float)a < tn; a++)
      frags.push_back(ShadowFrag{(uint32_t)((s % 12) / 2), a, (uint32_t)s, rcs[s]});
  }
  std::atomic<uint32_t>* dep = reinterpret_cast<std::atomic<uint32_t>*>(out);
  parallel_for((int64_t)frags.size(), nthreads, [&](int64_t id) {
    const ShadowFrag& f = frags[id];
    const Cut& ct = cut[f.ctri];
    FragGeom g = frag_geom(ct.p, f.rconst);
    walk(ct.p, L, L, kOpSizeLight, f.a, false, [&](float x, float y) {
      if (point_in_tri(x, y, g.xpv.x, g.ypv.x, g.xpv.y, g.ypv.y, g.xpv.z, g.ypv.z)) {
        uint32_t d = depth_at(g.A, g.B, g.C, x, y);
        atomic_min_u32(&dep[(size_t)((int)(y * L) + (int)x) + (size_t)f.face * kLightBufferDim * kLightBufferDim], d);
      }
    });
  });
}

}  // namespace

// ---- screenspace_godrays (cl2.cl:1792-1917, engine.cpp:1463-1482) ----------
// The sampler of the reference's screen image: unnormalised coordinates,
// clamp to edge, bilinear (OpenCL 1.2 section 8.2), float weights.
f4 sample_bilinear(const uint8_t* img, int W, int H, float x, float y) {
  const float u = x - 0.5f, v = y - 0.5f;
  const float fu = floorf(u), fv = floorf(v);
  const float a = u - fu, b = v - fv;
  auto cl = [](int i, int n) { return std::min(std::max(i, 0), n - 1); };
  const int x0 = cl((int)fu, W), x1 = cl((int)fu + 1, W), y0 = cl((int)fv, H), y1 = cl((int)fv + 1, H);
  auto texel = [&](int xx, int yy, int c) { return fdiv((float)img[((size_t)yy * W + xx) * 4 + c], 255.0f); };
  float o[4];
  for (int c = 0; c < 4; c++) {
    const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    o[c] = w00 * texel(x0, y0, c) + w10 * texel(x1, y0, c);
    o[c] = o[c] + w01 * texel(x0, y1, c);
    o[c] = o[c] + w11 * texel(x1, y1, c);
  }
  return v4(o);
}

// One pixel: every light with godray_intensity > 0 marches up to 80 steps of
// 400/80 pixels from the pixel towards the light's screen position (mirrored
// through the pixel when the light is behind the camera), adding the light's
// colour where the depth buffer holds something more than 5 units nearer than
// the pixel; the march stops at the first step off screen.
void godrays_pixel(int x, int y, const uint32_t* depth, const uint8_t* in, int W, int H, float fov,
                   const gbr_light* lights, uint32_t nl, f3 cpos, f3 cc, f3 cs, uint8_t* out) {
  f4 acc = sample_bilinear(in, W, H, (float)x - 0.25f, (float)y - 0.25f);
  const float here = depth_to_dist(depth[(size_t)y * W + x]);
  for (uint32_t l = 0; l < nl; l++) {
    const gbr_light& L = lights[l];
    if (L.godray_intensity <= 0) continue;
    const f3 sl = depth_project1(rot_cs(v3(L.pos), cpos, cc, cs), (float)W, (float)H, fov);
    f3 cur = mk3((float)x, (float)y, here);
    const f3 to = sl.z < 0 ? add3(sub3(cur, sl), cur) : sl;
    const float dx = std::fabs(cur.x - to.x), dy = std::fabs(cur.y - to.y);
    const float steps = dx > dy ? dx : dy;
    f3 d = sub3(to, cur);
    d = mk3(fdiv(d.x, steps) * 5.0f, fdiv(d.y, steps) * 5.0f, fdiv(d.z, steps) * 5.0f);
    float decay = 1.0f, sx = 0, sy = 0, sz = 0;
    for (int j = 0; (float)j < steps && j < 80; j++) {
      if (cur.x < 0 || cur.y < 0 || cur.x >= (float)(W - 1) || cur.y >= (float)(H - 1)) break;
      const uint32_t cd = depth[(size_t)f2i_sat(cur.y) * W + f2i_sat(cur.x)];  // (NaN -> 0, as the GPU converts)
      float r = 0, g = 0, b = 0;
      if (cd != kDepthClear && depth_to_dist(cd) < here - 5.0f) {
        decay = decay * 0.9f;
        r = L.col[0] * L.godray_intensity;
        g = L.col[1] * L.godray_intensity;
        b = L.col[2] * L.godray_intensity;
      }
      sx += (r * decay) * 0.01f;
      sy += (g * decay) * 0.01f;
      sz += (b * decay) * 0.01f;
      decay = decay * 0.97f;
      cur = add3(cur, d);
    }
    acc.x += sx;
    acc.y += sy;
    acc.z += sz;
  }
  const size_t p = ((size_t)y * W + x) * 4;
  out[p + 0] = (uint8_t)quant8(acc.x * 0.99f);
  out[p + 1] = (uint8_t)quant8(acc.y * 0.99f);
  out[p + 2] = (uint8_t)quant8(acc.z * 0.99f);
  out[p + 3] = (uint8_t)quant8(1.0f * 0.99f);
}

// ---- do_pseudo_aa (cl2.cl:6437-6657, engine.cpp:1513-1516) -----------------
// An edge pixel -- exactly one of its horizontal and one of its vertical
// neighbours, and at least one diagonal, differ from it by more than 100 depth
// units (test 0) or 20 degrees of normal (test 1) -- becomes 0.65 x the mean
// of its similar neighbours + 0.35 x the mean of the differing ones; the first
// test that finds an edge decides.  Every other pixel keeps its colour.
bool pseudo_aa_pixel(int x, int y, int W, int H, const uint32_t* depth, const uint16_t* nrm,
                     const uint8_t* in, float out[3]) {
  if (x < 1 || y < 1 || x >= W - 1 || y >= H - 1) return false;
  const size_t p = (size_t)y * W + x;
  if (depth[p] == kDepthClear) return false;
  const float here = depth_to_dist(depth[p]);
  const f3 n0 = fast_normalize3(decode_normal(nrm[2 * p], nrm[2 * p + 1]));
  int horiz[2] = {0, 0}, vert[2] = {0, 0}, diag[2] = {0, 0};
  float same[2][3] = {}, other[2][3] = {}, nsame[2] = {0, 0}, nother[2] = {0, 0};
  for (int dy = -1; dy <= 1; dy++)
    for (int dx = -1; dx <= 1; dx++) {
      if (dx == 0 && dy == 0) continue;
      const size_t q = (size_t)(y + dy) * W + (x + dx);
      const float d = depth_to_dist(depth[q]);
      const f3 n = decode_normal(nrm[2 * q], nrm[2 * q + 1]);
      float c[3];
      for (int k = 0; k < 3; k++) c[k] = (float)in[4 * q + k] / 255.0f;
      const bool edge[2] = {std::fabs(d - here) > 100.0f, dot3(n0, n) < kAACos};
      for (int t = 0; t < 2; t++) {
        if (edge[t]) {
          if (dx == dy || dx == -dy) diag[t]++;
          else if (dx != 0) horiz[t]++;
          else vert[t]++;
          for (int k = 0; k < 3; k++) other[t][k] += c[k];
          nother[t] += 1.0f;
        } else {
          for (int k = 0; k < 3; k++) same[t][k] += c[k];
          nsame[t] += 1.0f;
        }
      }
    }
  for (int t = 0; t < 2; t++) {
    if (horiz[t] == 1 && vert[t] == 1 && diag[t] >= 1) {
      for (int k = 0; k < 3; k++) out[k] = (same[t][k] / nsame[t]) * 0.65f + (other[t][k] / nother[t]) * 0.35f;
      return true;
    }
  }
  return false;
}

// ---- do_motion_blur (cl2.cl:6714-6860, engine.cpp:1518-1536) ----------------
// The pixel's surface point is carried back through its object's pose of the
// previous frame (descriptor history slot 1 on even frames, 2 on odd) and
// projected with this frame's camera and with last frame's; the blend of the
// two screen-space motions (camera_contribution), scaled by strength and
// capped at 50 px, is averaged over n bilinear taps centred on the pixel.
struct MotionArgs {
  f3 cpos, cc, cs, opos, oc, os;
  float fov, strength, cam_w;
  uint32_t frame_id;
};
bool motion_blur_pixel(int x, int y, int W, int H, const gbr_triangle* tris, const gbr_obj_g_descriptor* descs,
                       const uint32_t* depth, const uint32_t* ids, const uint8_t* in, const MotionArgs& a,
                       float out[4], uint32_t* obj) {
  const size_t p = (size_t)y * W + x;
  if (depth[p] == kDepthClear || ids[p] == kNoId) return false;
  const uint32_t o = tris[ids[p] >> 1].vertices[0].object_id;
  *obj = o;
  const gbr_obj_g_descriptor& G = descs[o];
  const float dist = depth_to_dist(depth[p]);
  const f3 local = mk3(fdiv(((float)x - (float)W / 2.0f) * dist, a.fov), fdiv(((float)y - (float)H / 2.0f) * dist, a.fov),
                       dist);
  const f3 world = add3(back_rot_cs(local, mk3(0, 0, 0), a.cc, a.cs), a.cpos);
  const f3 objl = back_rot_quat(sub3(world, v3(G.world_pos)), v4(G.world_rot_quat));
  const bool even = (a.frame_id & 1u) == 0;
  const f3 opos = v3(even ? G.old_world_pos_1 : G.old_world_pos_2);
  const f4 oq = v4(even ? G.old_world_rot_quat_1 : G.old_world_rot_quat_2);
  const f3 last = add3(rot_quat(objl, oq), opos);
  const f3 nocam = depth_project1(rot_cs(last, a.cpos, a.cc, a.cs), (float)W, (float)H, a.fov);
  const f3 prev = depth_project1(rot_cs(last, a.opos, a.oc, a.os), (float)W, (float)H, a.fov);
  if (prev.z < 20.0f) {
    const f4 c = sample_bilinear(in, W, H, (float)x + 0.5f, (float)y + 0.5f);
    out[0] = c.x; out[1] = c.y; out[2] = c.z; out[3] = c.w;
    return true;
  }
  float mx = (float)x - prev.x, my = (float)y - prev.y;
  const float nx = (float)x - nocam.x, ny = (float)y - nocam.y;
  mx = a.cam_w * mx + (1.0f - a.cam_w) * nx;
  my = a.cam_w * my + (1.0f - a.cam_w) * ny;
  mx = mx * a.strength;
  my = my * a.strength;
  int n = f2i_sat(fmax_(std::fabs(mx), std::fabs(my)) + 1.0f);
  if (n > 50) {
    mx = (mx / (float)n) * 50.0f;
    my = (my / (float)n) * 50.0f;
    n = 50;
  }
  float sx = 0.0f, sy = 0.0f;
  if (n != 0) {
    sx = mx / (float)n;
    sy = my / (float)n;
  }
  float cx = (float)x - mx / 2.0f, cy = (float)y - my / 2.0f;
  float acc[4] = {0, 0, 0, 0}, cnt = 0.0f;
  for (int i = 0; i < n; i++, cx += sx, cy += sy) {
    if (cx < 0 || cx >= (float)W || cy < 0 || cy >= (float)H) continue;
    const f4 c = sample_bilinear(in, W, H, cx + 0.5f, cy + 0.5f);
    acc[0] += c.x; acc[1] += c.y; acc[2] += c.z; acc[3] += c.w;
    cnt += 1.0f;
  }
  for (int k = 0; k < 4; k++) out[k] = cnt != 0.0f ? acc[k] / cnt : acc[k];
  return true;
}

// ---- screenspace_reflections (cl2.cl:6862-7355, engine.cpp:1483-1511) -------
// interpolate_single_line_depth (cl2.cl:6862-6873): a point on the screen-space
// segment s -> f at parameter a, depth interpolated in 1/z.
f3 line_depth_point(f3 s, f3 f, float a) {
  s.z = rcp(s.z);
  f.z = rcp(f.z);
  const float b = 1.0f - a;
  const f3 r = mk3(fma_(s.x, b, f.x * a), fma_(s.y, b, f.y * a), fma_(s.z, b, f.z * a));
  return mk3(r.x, r.y, rcp(r.z));
}

// One pixel of a surface whose object has FEATURE_FLAG_SS_REFLECTIVE: the eye
// ray is mirrored in the interpolated normal, marched over the depth buffer in
// screen space from a point 10.5 units along it (200 steps, until it passes
// behind the depth by more than 1), refined in tenths of a step, and the
// colour found there is mixed in by a contact fade (400 units, fading towards
// the screen edge) times the object's screen-space map (ssid) when it has one.
// Returns 0: unchanged, 1: out written.  Background pixels become 0.
int reflection_pixel(int x, int y, const ShadeView& v, const gbr_triangle* tris, const gbr_obj_g_descriptor* descs,
                     const Atlas& at, const uint32_t* depth, const uint32_t* ids, const uint8_t* in, float out[4]) {
  const int W = v.W, H = v.H;
  const size_t p = (size_t)y * W + x;
  if (depth[p] == kDepthClear) {
    out[0] = out[1] = out[2] = out[3] = 0.0f;
    return 1;
  }
  if (ids[p] == kNoId) return 0;
  const uint32_t tri = ids[p] >> 1, sub = ids[p] & 1u;
  const gbr_triangle& T = tris[tri];
  const gbr_obj_g_descriptor& G = descs[T.vertices[0].object_id];
  if (!((G.feature_flag & 1) > 0)) return 0;
  const float dist = depth_to_dist(depth[p]);
  const f3 local = mk3(fdiv(((float)x - (float)W / 2.0f) * dist, v.fov), fdiv(((float)y - (float)H / 2.0f) * dist, v.fov),
                       dist);
  const f3 zero = mk3(0, 0, 0);
  const f3 world = add3(back_rot_cs(local, zero, v.crot_c, v.crot_s), v.cpos);
  const f3 ray = sub3(world, v.cpos);
  f3 pv[3], nv[3];
  f2 tv[3];
  for (int k = 0; k < 3; k++) {
    pv[k] = mul3s(v3(T.vertices[k].pos), G.scale);
    nv[k] = v3(T.vertices[k].normal);
    tv[k] = mk2(T.vertices[k].vt[0], T.vertices[k].vt[1]);
  }
  const f4 q = v4(G.world_rot_quat);
  const f3 objl = back_rot_quat(sub3(world, v3(G.world_pos)), q);
  float l1, l2, l3;
  barycentric(objl, pv[0], pv[1], pv[2], &l1, &l2, &l3);
  f3 normal = mk3(fma_(nv[0].x, l1, fma_(nv[1].x, l2, nv[2].x * l3)), fma_(nv[0].y, l1, fma_(nv[1].y, l2, nv[2].y * l3)),
                  fma_(nv[0].z, l1, fma_(nv[1].z, l2, nv[2].z * l3)));
  normal = fast_normalize3(rot_quat(normal, q));
  const f2 vt = mk2(fma_(tv[0].x, l1, fma_(tv[1].x, l2, tv[2].x * l3)), fma_(tv[0].y, l1, fma_(tv[1].y, l2, tv[2].y * l3)));
  float refl = 1.0f;
  if (G.ssid != 0xFFFFFFFFu) {
    f3 outs[2][3];
    const int n = project_tri(T, G, v.cpos, v.crot_c, v.crot_s, v.fov, (float)W, (float)H, outs);
    if ((int)sub >= n) return 0;
    const f3* tp = outs[sub];
    const float rc = rconstant(mk3(roundf(tp[0].x), roundf(tp[1].x), roundf(tp[2].x)),
                               mk3(roundf(tp[0].y), roundf(tp[1].y), roundf(tp[2].y)));
    const f2 vtdiff = get_vtdiff(tp, (float)x, (float)y, v, G, vt, pv[0], pv[1], pv[2], tv[0], tv[1], tv[2], rc);
    refl = texture_filter_diff(vt, vtdiff, (int)G.ssid, at).x;
    if (refl < 0.1f) return 0;
  }
  // reflect (cl2.cl:169-176) normalises the normal once more
  const f3 nn = fast_normalize3(normal);
  const float k2 = 2.0f * dot3(ray, nn);
  const f3 refd = fast_normalize3(sub3(ray, mul3s(nn, k2)));
  const f3 jit = add3(world, mul3s(refd, 10.5f));
  const f3 sj = depth_project1(rot_cs(jit, v.cpos, v.crot_c, v.crot_s), (float)W, (float)H, v.fov);
  const f3 ss = depth_project1(rot_cs(world, v.cpos, v.crot_c, v.crot_s), (float)W, (float)H, v.fov);
  const float dx = sj.x - ss.x, dy = sj.y - ss.y;
  const float sdist = fsqrt(dx * dx + dy * dy);
  const float back = 1.0f - fdiv(sdist - 3.0f, sdist);
  f3 vprev = mk3(ss.x * back + sj.x * (1.0f - back), ss.y * back + sj.y * (1.0f - back),
                 rcp(ss.z) * back + rcp(sj.z) * (1.0f - back));
  vprev.z = rcp(vprev.z);
  const f3 vstart = sj;
  f3 cur = sj;
  auto off = [&](f3 c) { return c.x < 0 || c.y < 0 || c.x >= (float)W || c.y >= (float)H; };
  auto dist_at = [&](f3 c) { return depth_to_dist(depth[(size_t)f2i_sat(c.y) * W + f2i_sat(c.x)]); };
  if (off(cur)) return 0;
  bool found = false;
  float a = 1.0f;
  for (int i = 0; i < 200; i++) {
    if (off(cur)) return 0;
    if (dist_at(cur) < cur.z - 1.0f) {
      found = true;
      break;
    }
    a += 1.0f;
    cur = line_depth_point(vprev, vstart, a);
  }
  if (!found) return 0;
  // the refinement reads the depth where the march stopped on every try
  const float stop = dist_at(cur);
  float ta = a;
  f3 hit = cur;
  bool ok = false;
  for (int i = 0; i < 10; i++) {
    hit = line_depth_point(vprev, vstart, ta);
    if (stop < hit.z + 1.0f && stop > hit.z - 20.0f) {
      ok = true;
      break;
    }
    ta += 1.0f / 10.0f;
  }
  if (!ok) return 0;
  const f3 te = line_depth_point(vstart, hit, 1.35f);
  float fextra = 0.0f;
  if (te.x < 0) fextra += std::fabs(te.x);
  if (te.y < 0) fextra += std::fabs(te.y);
  if (te.x >= (float)W) fextra += te.x - (float)W;
  if (te.y >= (float)H) fextra += te.y - (float)H;
  fextra = clampf_(fextra / 200.0f, 0.0f, 1.0f);
  f3 gl = mk3(fdiv((hit.x - (float)W / 2.0f) * hit.z, v.fov), fdiv((hit.y - (float)H / 2.0f) * hit.z, v.fov), hit.z);
  gl = add3(back_rot_cs(gl, zero, v.crot_c, v.crot_s), v.cpos);
  const float ray_len = fast_length3(sub3(gl, world));
  float fade = 1.0f - ray_len / 400.0f;
  fade = fade - fextra;
  fade = clampf_(fade, 0.0f, 1.0f) * refl;
  const f4 found_col = sample_bilinear(in, W, H, hit.x, hit.y);
  const float fc[3] = {found_col.x, found_col.y, found_col.z};
  for (int k = 0; k < 3; k++) {
    const float c = (float)in[4 * p + k] / 255.0f;
    out[k] = (c + fc[k] * fade) / (1.0f + fade);
  }
  out[3] = 1.0f;
  return 1;
}

extern "C" {

// engine.cpp:119-133 then the std::to_string / -D FOV_CONST round trip (engine.cpp:474-477).
float oracle_fov_const(float hfov_deg, int width) {
  float fov_radians = (float)((double)((hfov_deg / 360.f) * 2) * 3.14159265358979323846);
  float half = fov_radians / 2;
  float fc = ((float)width / 2) / tanf(half);
  char buf[64];
  snprintf(buf, sizeof buf, "%f", (double)fc);
  return strtof(buf, nullptr);
}

// texture_context.cpp:94-261 page packing; update_gpu_tex with flip
// (cl2.cl:923-953, texture.cpp:323-346); generate_mips + generate_mip_mips
// (cl2.cl:1070-1189, texture.cpp:430-460).  atlas must hold n_pages*2048^2*4
// bytes; returns the page count, or -1 on error / -2 if capacities are short.
int oracle_build_textures(uint32_t n, const int32_t* sizes_in, const uint8_t* const* rgba,
                          uint8_t* atlas, uint32_t atlas_pages, uint32_t* nums, uint32_t nums_cap,
                          uint32_t* page_sizes, uint32_t sizes_cap, uint32_t* mipmap_start) {
  std::map<int, int> size_to_num;
  for (uint32_t i = 0; i < n; i++) {
    size_to_num[sizes_in[i]]++;
    for (int j = 0; j < kMipLevels; j++) size_to_num[sizes_in[i] / (1 << (j + 1))]++;
  }
  struct Page { int size, num; };
  std::vector<Page> pages;
  for (auto& kv : size_to_num) {
    if (kv.first <= 0) return -1;
    int maxp = (kTexPage / kv.first) * (kTexPage / kv.first);
    int rem = kv.second;
    while (rem >= maxp) { pages.push_back({kv.first, maxp}); rem -= maxp; }
    if (rem > 0) pages.push_back({kv.first, rem});
  }
  if (pages.size() > sizes_cap || pages.size() > atlas_pages || n * 5 > nums_cap) return -2;
  std::vector<Page> fp = pages;
  auto take = [&](int size) -> int64_t {
    for (size_t s = 0; s < fp.size(); s++)
      if (fp[s].size == size && fp[s].num > 0) {
        int fn = fp[s].num - 1;
        fp[s].num--;
        return (int64_t)((s << 16) | (uint32_t)fn);
      }
    return -1;
  };
  std::vector<uint32_t> desc;
  for (uint32_t i = 0; i < n; i++) {
    int64_t d = take(sizes_in[i]);
    if (d < 0) return -1;
    desc.push_back((uint32_t)d);
  }
  for (uint32_t i = 0; i < n; i++)
    for (int j = 0; j < kMipLevels; j++) {
      int64_t d = take(sizes_in[i] / (1 << (j + 1)));
      if (d < 0) return -1;
      desc.push_back((uint32_t)d);
    }
  for (size_t i = 0; i < desc.size(); i++) nums[i] = desc[i];
  for (size_t i = 0; i < pages.size(); i++) page_sizes[i] = (uint32_t)pages[i].size;
  *mipmap_start = n;
  memset(atlas, 0, (size_t)pages.size() * kTexPage * kTexPage * 4);

  // write_tex_array (cl2.cl:856-889) and read_tex_array (cl2.cl:785-821)
  auto tex_xy = [&](uint32_t tid, float* tx, float* ty, int* slice, float* width) {
    uint32_t nv = nums[tid];
    *slice = (int)(nv >> 16);
    int which = (int)(nv & 0xFFFF);
    *width = (float)page_sizes[*slice];
    float hnum = floorf(fdiv(2048.0f, *width));
    float tnumy = floorf(fdiv((float)which, hnum));
    float tnumx = fma_(-tnumy, hnum, (float)which);
    *tx = tnumx;
    *ty = tnumy;
  };
  auto write_tex = [&](const uint32_t c[4], float cx, float cy, uint32_t tid) {
    float tnx, tny, w; int slice;
    tex_xy(tid, &tnx, &tny, &slice, &w);
    float tx = tnx * w, ty = tny * w;
    cx = fmodf(cx, w); cy = fmodf(cy, w);
    cx = clampf_(cx, 0.001f, w - 0.001f);
    cy = clampf_(cy, 0.001f, w - 0.001f);
    int ix = (int)(tx + cx), iy = (int)(ty + cy);
    uint8_t* t = atlas + ((size_t)slice * kTexPage * kTexPage + (size_t)iy * kTexPage + ix) * 4;
    for (int k = 0; k < 4; k++) t[k] = (uint8_t)c[k];
  };
  auto read_tex = [&](float cx, float cy, uint32_t tid, float out[4]) {
    float tnx, tny, w; int slice;
    tex_xy(tid, &tnx, &tny, &slice, &w);
    cx = clampf_(cx, 0.001f, w - 0.001f);
    cy = clampf_(cy, 0.001f, w - 0.001f);
    int ix = f2i_sat(fma_(tnx, w, cx)), iy = f2i_sat(fma_(tny, w, cy));
    const uint8_t* t = atlas + ((size_t)slice * kTexPage * kTexPage + (size_t)iy * kTexPage + ix) * 4;
    for (int k = 0; k < 4; k++) out[k] = (float)t[k];
  };
  auto mip = [&](uint32_t src, uint32_t dst, int gw, int gh) {
    float w = (float)page_sizes[nums[src] >> 16];
    float nw = (float)page_sizes[nums[dst] >> 16];
    const float gauss[3][3] = {{1, 2, 1}, {2, 4, 2}, {1, 2, 1}};
    for (int y = 0; y < gh; y++)
      for (int x = 0; x < gw; x++) {
        if ((float)x >= w || (float)y >= w) continue;
        float acc[4] = {0, 0, 0, 0};
        float div = 0.f;
        for (int j = -1; j <= 1; j++)
          for (int i = -1; i <= 1; i++) {
            float c[4];
            read_tex((float)(x * 2 + i), (float)(y * 2 + j), src, c);
            c[3] = fdiv(c[3], 255.f);
            c[0] *= c[3]; c[1] *= c[3]; c[2] *= c[3];
            float g = gauss[j + 1][i + 1];
            for (int k = 0; k < 4; k++) acc[k] += c[k] * g;
            div += g;
          }
        for (int k = 0; k < 4; k++) acc[k] = fdiv(acc[k], div);
        if (acc[3] > 0.00000001f)
          for (int k = 0; k < 3; k++) acc[k] = fdiv(acc[k], acc[3]);
        acc[3] *= 255.f;
        float yx0 = fdiv((float)(x * 2), w) * nw, yx1 = fdiv((float)(y * 2), w) * nw;
        if (yx0 >= nw || yx1 >= nw) continue;
        uint32_t c[4];
        for (int k = 0; k < 4; k++) c[k] = f2u_sat(acc[k]);
        write_tex(c, yx0, yx1, dst);
      }
  };
  for (uint32_t t = 0; t < n; t++) {
    int s = sizes_in[t];
    float w = (float)page_sizes[nums[t] >> 16];
    for (int y = 0; y < s; y++)
      for (int x = 0; x < s; x++) {
        const uint8_t* px = rgba[t] + ((size_t)y * s + x) * 4;
        uint32_t c[4] = {px[0], px[1], px[2], px[3]};
        float fy = (float)y;
        fy = w - fy;  // flip = 1 (texture.cpp:344)
        write_tex(c, (float)x, fy, t);
      }
    uint32_t m0 = t * kMipLevels + *mipmap_start;
    mip(t, m0, s, s);
    for (int l = 0; l < kMipLevels - 1; l++) mip(m0 + l, m0 + l + 1, s, s);
  }
  return (int)pages.size();
}

// Shadow cubemaps of every shadow-casting light (engine.cpp:1601-1790).
// dyn: 6*1024^2 u32 per light with shadow==1; stat: per light with shadow && is_static.
void oracle_shadow(const gbr_triangle* tris, uint32_t n, const gbr_obj_g_descriptor* descs,
                   const gbr_light* lights, uint32_t nl, uint32_t* dyn, uint32_t* stat,
                   int nthreads) {
  const size_t face = (size_t)kLightBufferDim * kLightBufferDim;
  uint32_t nn = 0, kk = 0;
  for (uint32_t i = 0; i < nl; i++) {
    f3 lpos = v3(lights[i].pos);
    if (lights[i].shadow == 1) {
      uint32_t* out = dyn + (size_t)nn * 6 * face;
      std::fill(out, out + 6 * face, kDepthClear);
      shadow_light(tris, n, descs, lpos, 0, out, nthreads);
      nn++;
    }
    if (lights[i].shadow && lights[i].is_static && stat) {
      uint32_t* out = stat + (size_t)kk * 6 * face;
      std::fill(out, out + 6 * face, kDepthClear);
      shadow_light(tris, n, descs, lpos, 1, out, nthreads);
      kk++;
    }
  }
}

// One view: prearrange -> kernel1 -> kernel2 -> kernel3 (render_tris).
// Any output pointer may be NULL except depth and id.
int oracle_render(const gbr_triangle* tris, uint32_t n, const gbr_obj_g_descriptor* descs,
                  const gbr_light* lights, uint32_t nl, const uint8_t* atlas,
                  const uint32_t* nums, const uint32_t* sizes, uint32_t mipmap_start,
                  const uint32_t* shadow_dyn, const uint32_t* shadow_static,
                  const gbr_camera* cam, const gbr_view* view, uint32_t* depth, uint32_t* ids,
                  uint8_t* rgba, uint16_t* normals, int nthreads, uint64_t* nfrags_out,
                  const uint32_t* blend_depth, const uint8_t* blend_rgba) {
  const int W = view->width, H = view->height;
  const float fov = view->fov_const > 0 ? view->fov_const : oracle_fov_const(view->hfov_deg, W);
  f3 cpos = v3(cam->pos), crot = v3(cam->rot);
  Setup S;
  prearrange(tris, n, descs, cpos, crot, fov, (float)W, (float)H, nthreads, &S);
  if (nfrags_out) *nfrags_out = S.frags.size();
  const size_t P = (size_t)W * H;
  std::fill(depth, depth + P, kDepthClear);
  std::fill(ids, ids + P, kNoId);
  kernel1(S, (float)W, (float)H, reinterpret_cast<std::atomic<uint32_t>*>(depth), W, nthreads);
  kernel2(S, (float)W, (float)H, depth, reinterpret_cast<std::atomic<uint32_t>*>(ids), W, nthreads);
  if (!rgba) return 0;
  ShadeView v;
  v.W = W; v.H = H; v.fov = fov; v.cpos = cpos; v.crot = crot; v.flags = view->flags;
  euler_cs(crot, &v.crot_c, &v.crot_s);
  for (int f = 0; f < 6; f++) euler_cs(face_angles(f), &v.face_c[f], &v.face_s[f]);
  v.use_linear = view->use_linear;
  v.clear.x = view->clear_col[0]; v.clear.y = view->clear_col[1];
  v.clear.z = view->clear_col[2]; v.clear.w = view->clear_col[3];
  v.blend_depth = blend_depth;
  v.blend_rgba = blend_rgba;
  ShadeIn in{tris, descs, lights, nl, Atlas{atlas, nums, sizes, mipmap_start}, shadow_dyn, shadow_static};
  parallel_for((int64_t)P, nthreads, [&](int64_t p) {
    kernel3_pixel((int)(p % W), (int)(p / W), v, in, S, depth, ids, rgba, normals);
  });
  return 0;
}

// kernel3 in double precision (see kernel3_pixel_fp64) over the depth / id
// of the float path: rgba64 gets H*W*4 colours in [0, 1] before quantisation.
int oracle_render_fp64(const gbr_triangle* tris, uint32_t n, const gbr_obj_g_descriptor* descs,
                       const gbr_light* lights, uint32_t nl, const uint8_t* atlas, const uint32_t* nums,
                       const uint32_t* sizes, uint32_t mipmap_start, const uint32_t* shadow_dyn,
                       const uint32_t* shadow_static, const gbr_camera* cam, const gbr_view* view,
                       double* rgba64, int exact_acos, int nthreads, const uint32_t* blend_depth,
                       const uint8_t* blend_rgba) {
  const int W = view->width, H = view->height;
  const float fov = view->fov_const > 0 ? view->fov_const : oracle_fov_const(view->hfov_deg, W);
  f3 cpos = v3(cam->pos), crot = v3(cam->rot);
  Setup S;
  prearrange(tris, n, descs, cpos, crot, fov, (float)W, (float)H, nthreads, &S);
  const size_t P = (size_t)W * H;
  std::vector<uint32_t> depth(P, kDepthClear), ids(P, kNoId);
  kernel1(S, (float)W, (float)H, reinterpret_cast<std::atomic<uint32_t>*>(depth.data()), W, nthreads);
  kernel2(S, (float)W, (float)H, depth.data(), reinterpret_cast<std::atomic<uint32_t>*>(ids.data()), W, nthreads);
  ShadeView v;
  v.W = W; v.H = H; v.fov = fov; v.cpos = cpos; v.crot = crot; v.flags = view->flags;
  euler_cs(crot, &v.crot_c, &v.crot_s);
  for (int f = 0; f < 6; f++) euler_cs(face_angles(f), &v.face_c[f], &v.face_s[f]);
  v.use_linear = view->use_linear;
  v.clear.x = view->clear_col[0]; v.clear.y = view->clear_col[1];
  v.clear.z = view->clear_col[2]; v.clear.w = view->clear_col[3];
  v.blend_depth = blend_depth;
  v.blend_rgba = blend_rgba;
  ShadeIn in{tris, descs, lights, nl, Atlas{atlas, nums, sizes, mipmap_start}, shadow_dyn, shadow_static};
  parallel_for((int64_t)P, nthreads, [&](int64_t p) {
    kernel3_pixel_fp64((int)(p % W), (int)(p / W), v, in, S, depth.data(), ids.data(), exact_acos != 0, rgba64);
  });
  return 0;
}

// The literal walk of one fragment, for unit tests: writes visited (x,y) pairs.
int oracle_walk(const float* tp9, float ew, float eh, int chunk, uint32_t distance, int32_t* xy,
                int cap) {
  f3 tp[3] = {mk3(tp9[0], tp9[1], tp9[2]), mk3(tp9[3], tp9[4], tp9[5]), mk3(tp9[6], tp9[7], tp9[8])};
  int n = 0;
  walk(tp, ew, eh, chunk, distance, false, [&](float x, float y) {
    if (n < cap) { xy[2 * n] = (int)x; xy[2 * n + 1] = (int)y; }
    n++;
  });
  return n;
}

// engine::draw_godrays over a rendered view (depth, RGBA8): RGBA8 out.
int oracle_godrays(const uint32_t* depth, const uint8_t* rgba_in, const gbr_light* lights, uint32_t nl,
                   const gbr_camera* cam, const gbr_view* view, uint8_t* rgba_out, int nthreads) {
  const int W = view->width, H = view->height;
  const float fov = view->fov_const > 0 ? view->fov_const : oracle_fov_const(view->hfov_deg, W);
  f3 cc, cs;
  euler_cs(v3(cam->rot), &cc, &cs);
  const f3 cpos = v3(cam->pos);
  parallel_for((int64_t)W * H, nthreads, [&](int64_t p) {
    godrays_pixel((int)(p % W), (int)(p / W), depth, rgba_in, W, H, fov, lights, nl, cpos, cc, cs, rgba_out);
  });
  return 0;
}

// do_pseudo_aa over a rendered view: rgba_out = rgba_in with edge pixels
// replaced.  Pixels with depth but no id are left as they are.
int oracle_pseudo_aa(const uint32_t* depth, const uint32_t* ids, const uint16_t* normals, const uint8_t* rgba_in,
                     int W, int H, uint8_t* rgba_out, int nthreads) {
  parallel_for((int64_t)W * H, nthreads, [&](int64_t p) {
    const int x = (int)(p % W), y = (int)(p / W);
    float c[3];
    const bool edge = ids[p] != kNoId && pseudo_aa_pixel(x, y, W, H, depth, normals, rgba_in, c);
    for (int k = 0; k < 4; k++)
      rgba_out[4 * p + k] = edge ? (uint8_t)quant8(k < 3 ? c[k] : 1.0f) : rgba_in[4 * p + k];
  });
  return 0;
}

// do_motion_blur over a rendered view.  descs is updated with the pose
// history: every object with a pixel on screen gets its current pose in slot
// 2 (even frame_id) or 1 (odd).
int oracle_motion_blur(const gbr_triangle* tris, gbr_obj_g_descriptor* descs, uint32_t ndescs, const uint32_t* depth,
                       const uint32_t* ids, const uint8_t* rgba_in, const gbr_camera* cam, const gbr_camera* cam_old,
                       const gbr_view* view, uint32_t frame_id, float strength, float camera_contribution,
                       uint8_t* rgba_out, int nthreads) {
  const int W = view->width, H = view->height;
  MotionArgs a;
  a.fov = view->fov_const > 0 ? view->fov_const : oracle_fov_const(view->hfov_deg, W);
  a.cpos = v3(cam->pos);
  euler_cs(v3(cam->rot), &a.cc, &a.cs);
  a.opos = v3(cam_old->pos);
  euler_cs(v3(cam_old->rot), &a.oc, &a.os);
  a.strength = strength;
  a.cam_w = camera_contribution;
  a.frame_id = frame_id;
  std::vector<std::atomic<uint8_t>> seen(ndescs);
  for (auto& f : seen) f.store(0);
  parallel_for((int64_t)W * H, nthreads, [&](int64_t p) {
    float c[4];
    uint32_t o = 0;
    const bool hit = motion_blur_pixel((int)(p % W), (int)(p / W), W, H, tris, descs, depth, ids, rgba_in, a, c, &o);
    if (hit) seen[o].store(1);
    for (int k = 0; k < 4; k++) rgba_out[4 * p + k] = hit ? (uint8_t)quant8(c[k]) : rgba_in[4 * p + k];
  });
  for (uint32_t o = 0; o < ndescs; o++) {
    if (!seen[o].load()) continue;
    gbr_obj_g_descriptor& G = descs[o];
    float* pos = (frame_id & 1u) == 0 ? G.old_world_pos_2 : G.old_world_pos_1;
    float* q = (frame_id & 1u) == 0 ? G.old_world_rot_quat_2 : G.old_world_rot_quat_1;
    for (int k = 0; k < 3; k++) pos[k] = G.world_pos[k];
    for (int k = 0; k < 4; k++) q[k] = G.world_rot_quat[k];
  }
  return 0;
}

// screenspace_reflections over a rendered view (cl2.cl:6906-7355).
int oracle_reflections(const gbr_triangle* tris, const gbr_obj_g_descriptor* descs, const uint8_t* atlas,
                       const uint32_t* nums, const uint32_t* sizes, uint32_t mipmap_start, const uint32_t* depth,
                       const uint32_t* ids, const uint8_t* rgba_in, const gbr_camera* cam, const gbr_view* view,
                       uint8_t* rgba_out, int nthreads) {
  ShadeView v;
  v.W = view->width;
  v.H = view->height;
  v.fov = view->fov_const > 0 ? view->fov_const : oracle_fov_const(view->hfov_deg, v.W);
  v.cpos = v3(cam->pos);
  v.crot = v3(cam->rot);
  euler_cs(v.crot, &v.crot_c, &v.crot_s);
  const Atlas at{atlas, nums, sizes, mipmap_start};
  parallel_for((int64_t)v.W * v.H, nthreads, [&](int64_t p) {
    float c[4];
    const int w = reflection_pixel((int)(p % v.W), (int)(p / v.W), v, tris, descs, at, depth, ids, rgba_in, c);
    for (int k = 0; k < 4; k++) rgba_out[4 * p + k] = w ? (uint8_t)quant8(c[k]) : rgba_in[4 * p + k];
  });
  return 0;
}

}  // extern "C"
