// gbr_kernels.cu — sm_103a kernels of the triangle pipeline.
//
// Compiled with --fmad=false: every fused multiply-add below is an explicit
// fmaf() standing for a `mad` of cl2.cl; all other float expressions round
// after each operation, as the determinism contract in gbr_math.h requires.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "gbr_internal.h"

namespace gbr {
namespace {

__device__ __forceinline__ f3 ld3(const float* p) { return mk3(__ldg(p), __ldg(p + 1), __ldg(p + 2)); }
__device__ __forceinline__ f4 ld4(const float* p) {
  float4 v = __ldg(reinterpret_cast<const float4*>(p));
  f4 r; r.x = v.x; r.y = v.y; r.z = v.z; r.w = v.w;
  return r;
}

// Warp-aggregated allocation of n slots from *counter; every lane of the
// warp must call it (n may be 0).  Returns this lane's first slot.
__device__ __forceinline__ uint32_t warp_alloc(uint32_t* counter, uint32_t n) {
  const unsigned full = 0xFFFFFFFFu;
  int lane = threadIdx.x & 31;
  uint32_t incl = n;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t v = __shfl_up_sync(full, incl, o);
    if (lane >= o) incl += v;
  }
  uint32_t total = __shfl_sync(full, incl, 31);
  uint32_t base = 0;
  if (lane == 31 && total) base = atomicAdd(counter, total);
  base = __shfl_sync(full, base, 31);
  return base + incl - n;
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
  return v;
}

// Warp-aggregated "atomicAdd(&counter[key], 1)": lanes with the same key
// share one atomic.  Every lane of the warp must call it; inactive lanes pass
// active = false.  Returns this lane's old value + its rank within its key.
__device__ __forceinline__ uint32_t agg_inc(uint32_t* counter, uint32_t key, bool active) {
  const unsigned act = __ballot_sync(0xFFFFFFFFu, active);
  uint32_t res = 0;
  if (active) {
    const int lane = threadIdx.x & 31;
    const unsigned grp = __match_any_sync(act, key);
    const int leader = __ffs(grp) - 1;
    uint32_t old = 0;
    if (lane == leader) old = atomicAdd(&counter[key], (uint32_t)__popc(grp));
    old = __shfl_sync(grp, old, leader);
    res = old + (uint32_t)__popc(grp & ((1u << lane) - 1u));
  }
  return res;
}

// A visible clipped triangle before it becomes a record.
struct Cand {
  f3 p[3];
  float rc;
  float mm[4];
  uint32_t key;
};

// prearrange's per-output culls (cl2.cl:4352-4377): returns false when the
// output is culled or its bbox is empty (ceil(area/op_size) == 0).
__device__ __forceinline__ bool cull_candidate(Cand& c, bool two_sided, float w, float h) {
  const f3* p = c.p;
  int valid = two_sided || backface_front(p[0], p[1], p[2]);
  int cond = (p[0].x < 0 && p[1].x < 0 && p[2].x < 0) ||
             (p[0].x >= w && p[1].x >= w && p[2].x >= w) ||
             (p[0].y < 0 && p[1].y < 0 && p[2].y < 0) ||
             (p[0].y >= h && p[1].y >= h && p[2].y >= h);
  if (!valid || cond) return false;
  f3 xpv = mk3(roundf(p[0].x), roundf(p[1].x), roundf(p[2].x));
  f3 ypv = mk3(roundf(p[0].y), roundf(p[1].y), roundf(p[2].y));
  c.rc = rconstant(xpv, ypv);
  bbox4(p[0], p[1], p[2], w, h, c.mm);
  return (c.mm[1] - c.mm[0]) * (c.mm[3] - c.mm[2]) > 0.0f;
}

__device__ __forceinline__ void make_rec(const Cand& c, uint32_t surface, RasterRec& R) {
  const f3* p = c.p;
  f3 xpv = mk3(roundf(p[0].x), roundf(p[1].x), roundf(p[2].x));
  f3 ypv = mk3(roundf(p[0].y), roundf(p[1].y), roundf(p[2].y));
  f3 depths = mk3(rcp(fdiv(p[0].z, kDepthFar)), rcp(fdiv(p[1].z, kDepthFar)),
                  rcp(fdiv(p[2].z, kDepthFar)));
  plane_const(depths, xpv, ypv, c.rc, &R.A, &R.B, &R.C);
  EdgeTest e = make_edge(xpv.x, ypv.x, xpv.y, ypv.y, xpv.z, ypv.z);
  R.s0 = e.s0; R.sa = e.sa; R.sb = e.sb; R.sign = e.sign;
  R.t0 = e.t0; R.ta = e.ta; R.tb = e.tb; R.bound = e.bound;
  R.key = c.key;
  R.xr = (uint32_t)c.mm[0] | ((uint32_t)c.mm[1] << 16);
  R.yr = (uint32_t)c.mm[2] | ((uint32_t)c.mm[3] << 16);
  R.surface = surface;
  R.pad = 0;
}

__device__ __forceinline__ void store_rec(RasterRec* dst, const RasterRec& R) {
  float4* d = reinterpret_cast<float4*>(dst);
  d[0] = make_float4(R.A, R.B, R.C, R.bound);
  d[1] = make_float4(R.s0, R.sa, R.sb, R.sign);
  d[2] = make_float4(R.t0, R.ta, R.tb, __uint_as_float(R.key));
  d[3] = make_float4(__uint_as_float(R.xr), __uint_as_float(R.yr), __uint_as_float(R.surface), 0.0f);
}

// Tile footprint of a bbox [minx,maxx) x [miny,maxy).
struct Foot {
  int tx0, tx1, ty0, ty1;  // inclusive fine tiles
  bool coarse;
};
__device__ __forceinline__ int foot_count(const Foot& f) { return (f.tx1 - f.tx0 + 1) * (f.ty1 - f.ty0 + 1); }
// Global tile index (fine or coarse counter array) of the k-th tile of a footprint.
__device__ __forceinline__ uint32_t foot_tile(const Foot& f, int k, const Surface& S) {
  const int w = f.tx1 - f.tx0 + 1;
  const int ty = f.ty0 + k / w, tx = f.tx0 + k % w;
  return f.coarse ? S.ctile_base + ty * S.ctiles_x + tx : S.tile_base + ty * S.tiles_x + tx;
}
// Records touching more than ws.fine_max fine tiles go to the coarse bins
// (tiles of kTile << ws.coarse_shift pixels).
__device__ __forceinline__ Foot footprint(uint32_t xr, uint32_t yr, const Workspace& ws) {
  Foot f;
  int minx = xr & 0xFFFF, maxx = xr >> 16, miny = yr & 0xFFFF, maxy = yr >> 16;
  f.tx0 = minx / kTile; f.tx1 = (maxx - 1) / kTile;
  f.ty0 = miny / kTile; f.ty1 = (maxy - 1) / kTile;
  f.coarse = (f.tx1 - f.tx0 + 1) * (f.ty1 - f.ty0 + 1) > ws.fine_max;
  if (f.coarse) {
    const int sh = ws.coarse_shift;
    f.tx0 >>= sh; f.tx1 >>= sh;
    f.ty0 >>= sh; f.ty1 >>= sh;
  }
  return f;
}

// point_in_tri of a record at pixel (px, py).
__device__ __forceinline__ bool rec_in_tri(const float4 q[4], int px, int py) {
  float fx = (float)px, fy = (float)py;
  float sgn = q[1].w;
  float s = ((q[1].x + q[1].y * fx) + q[1].z * fy) * sgn;
  float t = ((q[2].x + q[2].y * fx) + q[2].z * fy) * sgn;
  return s > -0.0001f && t > -0.0001f && (s + t) < q[0].w;
}

// Is the left-column pixel (minx, py) of a record's bbox skipped by the
// reference walk (py > miny)?
__device__ __forceinline__ bool walk_skips(uint32_t xr, uint32_t yr, int py, int chunk) {
  const int minx = xr & 0xFFFF, miny = yr & 0xFFFF;
  return py > miny && !walk_visits(0, py - miny, (int)(xr >> 16) - minx, (int)(yr >> 16) - miny, (float)miny, chunk);
}

// walk_skips for the rows [y0, y1) of a record's bbox at once: bit py - ty
// set where the left-column pixel is skipped.  The same arithmetic as
// walk_visits (walk_row_late's 1 / w computed once, (r + 1) * w % chunk
// stepped row by row).
__device__ __forceinline__ uint32_t walk_skip_rows(uint32_t xr, uint32_t yr, int y0, int y1, int ty, int chunk) {
  const int minx = xr & 0xFFFF, miny = yr & 0xFFFF;
  const int w = (int)(xr >> 16) - minx, h = (int)(yr >> 16) - miny;
  const float iw = fdiv(1.0f, (float)w), fminy = (float)miny;
  const int first = max(y0, miny + 1) - miny;  // r of the first row with r > 0
  const int last = y1 - miny;                  // one past
  if (first >= last) return 0u;
  auto late = [&](int r) { return floorf(fma_((float)(r * w), iw, fminy)) != fminy + (float)r; };
  const int wm = w % chunk;
  int m = ((first + 1) * w) % chunk;  // (r + 1) * w % chunk
  bool late_r = late(first);
  uint32_t bits = 0;
  for (int r = first; r < last; r++) {
    const int r1 = r + 1;
    const bool late_r1 = r1 < h ? late(r1) : false;
    // walk_visits: not late, or the next row is late and a fragment starts at (r + 1) * w
    const bool visits = !late_r || (r1 < h && m == 0 && late_r1);
    if (!visits) bits |= 1u << (miny + r - ty);
    late_r = late_r1;
    m += wm;
    if (m >= chunk) m -= chunk;
  }
  return bits;
}

// Coverage of a pixel known to lie inside the record's bbox: the reference
// walk's skipped left-column pixels, then point_in_tri.
__device__ __forceinline__ bool covers_in_bbox(const float4 q[4], int px, int py, int chunk) {
  const uint32_t xr = __float_as_uint(q[3].x), yr = __float_as_uint(q[3].y);
  if (px == (int)(xr & 0xFFFF) && walk_skips(xr, yr, py, chunk)) return false;
  return rec_in_tri(q, px, py);
}

// One candidate as a record (and shade record for views); returns its tile footprint.
__device__ __forceinline__ int write_rec(const Cand& c, uint32_t r, uint32_t surface, const Workspace& ws, bool view,
                                         Foot* foot) {
  RasterRec R;
  make_rec(c, surface, R);
  store_rec(ws.rec + r, R);
  if (view) {  // what prep_shade needs (the fill turns it into the shade constants)
    uint32_t tri = c.key >> 1;
    ws.srec[r].a = make_float4(c.p[0].x, c.p[0].y, c.p[0].z, c.rc);
    ws.srec[r].e0 = make_float4(c.p[1].x, c.p[1].y, c.p[1].z, __uint_as_float(tri));
    ws.srec[r].e1 = make_float4(c.p[2].x, c.p[2].y, c.p[2].z, 0.0f);
  }
  *foot = footprint(R.xr, R.yr, ws);
  return foot_count(*foot);
}

// Depth-only passes (cube faces): a candidate whose bbox has at most this
// many pixels is rasterised by its setup thread straight into the face with
// global atomicMin -- the same coverage tests and depths as the tile raster,
// and a minimum does not depend on order -- instead of becoming a record.
constexpr float kDirectArea = 64.0f;

__device__ __forceinline__ bool direct_cand(const Cand& c) {
  return (c.mm[1] - c.mm[0]) * (c.mm[3] - c.mm[2]) <= kDirectArea;
}

// kernel1 of one small candidate into its surface's depth; returns the
// covered pixel count.
__device__ __noinline__ uint32_t direct_raster(const Cand& c, uint32_t surface, const Surface& S) {
  RasterRec R;
  make_rec(c, surface, R);
  const float4 q[4] = {make_float4(R.A, R.B, R.C, R.bound), make_float4(R.s0, R.sa, R.sb, R.sign),
                       make_float4(R.t0, R.ta, R.tb, __uint_as_float(R.key)),
                       make_float4(__uint_as_float(R.xr), __uint_as_float(R.yr), 0.0f, 0.0f)};
  const int x0 = (int)(R.xr & 0xFFFF), x1 = (int)(R.xr >> 16), y0 = (int)(R.yr & 0xFFFF), y1 = (int)(R.yr >> 16);
  uint32_t hits = 0;
  // covers_in_bbox row by row: the walk rule of each row's left-column pixel
  // (walk_visits) with 1 / w and (r + 1) * w % chunk computed incrementally
  const int w = x1 - x0, h = y1 - y0, chunk = S.chunk;
  const float iw = fdiv(1.0f, (float)w), fminy = (float)y0;
  auto late = [&](int r) { return floorf(fma_((float)(r * w), iw, fminy)) != fminy + (float)r; };
  const int wm = w % chunk;
  int m = (2 * w) % chunk;  // (r + 1) * w % chunk for row r = 1
  bool late_r = h > 1 ? late(1) : false;
  for (int y = y0; y < y1; y++) {
    const int r = y - y0;
    bool skip_left = false;
    if (r > 0) {
      const int r1 = r + 1;
      const bool late_r1 = r1 < h ? late(r1) : false;
      skip_left = late_r && !(r1 < h && m == 0 && late_r1);
      late_r = late_r1;
      m += wm;
      if (m >= chunk) m -= chunk;
    }
    for (int x = skip_left ? x0 + 1 : x0; x < x1; x++)
      if (rec_in_tri(q, x, y)) {
        atomicMin(S.depth + (size_t)y * S.width + x, depth_at(R.A, R.B, R.C, (float)x, (float)y));
        hits++;
      }
  }
  return hits;
}

// Append this lane's candidates (n = 0, 1 or 2: c0, then c1) as records and
// count their bins (depth-only passes rasterise small ones directly).  Every
// lane of the warp must call it.  Returns this lane's reference fragment count
// (sum of ceil(area / chunk)).
__device__ unsigned long long emit(const Cand& c0, const Cand& c1, int n, uint32_t surface, const Surface* surfs,
                                   const Workspace& ws, bool view) {
  const bool d0 = !view && n > 0 && direct_cand(c0), d1 = !view && n > 1 && direct_cand(c1);
  const uint32_t nr = (uint32_t)(n > 0 && !d0) + (uint32_t)(n > 1 && !d1);
  const uint32_t base = warp_alloc(&ws.ctr->nrec, nr);
  unsigned long long frags = 0;
  const Surface& S = surfs[surface];
  Foot f0{0, 0, 0, 0, false}, f1{0, 0, 0, 0, false};
  int n0 = 0, n1 = 0;
  uint32_t slot = base, hits = 0;
  if (n > 0) {
    frags += (unsigned long long)ceilf(fdiv((c0.mm[1] - c0.mm[0]) * (c0.mm[3] - c0.mm[2]), (float)S.chunk));
    if (d0) hits += direct_raster(c0, surface, S);
    else if (slot < ws.rec_cap) n0 = write_rec(c0, slot++, surface, ws, view, &f0);
    else atomicOr(&ws.ctr->overflow, 1u);
  }
  if (n > 1) {
    frags += (unsigned long long)ceilf(fdiv((c1.mm[1] - c1.mm[0]) * (c1.mm[3] - c1.mm[2]), (float)S.chunk));
    if (d1) hits += direct_raster(c1, surface, S);
    else if (slot < ws.rec_cap) n1 = write_rec(c1, slot++, surface, ws, view, &f1);
    else atomicOr(&ws.ctr->overflow, 1u);
  }
  if (!view) {
    hits = __reduce_add_sync(0xFFFFFFFFu, hits);
    if ((threadIdx.x & 31) == 0 && hits) atomicAdd(&ws.ctr->samples, (unsigned long long)hits);
  }
  // tile counts, aggregated across the warp (neighbouring triangles usually
  // share tiles): iterate over this lane's (record, tile) pairs in lockstep
  const int total = n0 + n1;
  int maxt = total;
  for (int o = 16; o > 0; o >>= 1) maxt = max(maxt, __shfl_xor_sync(0xFFFFFFFFu, maxt, o));
  for (int it = 0; it < maxt; it++) {
    const bool act = it < total;
    const bool second = it >= n0;
    const Foot& f = second ? f1 : f0;
    const int k = second ? it - n0 : it;
    const bool coarse = act && f.coarse;
    const uint32_t tile = act ? foot_tile(f, k, S) : 0u;
    // fine and coarse counters live in different arrays: aggregate them separately
    agg_inc(ws.fine_count, tile, act && !coarse);
    agg_inc(ws.coarse_count, tile, act && coarse);
  }
  return frags;
}

__device__ __forceinline__ void add_frags(const Workspace& ws, unsigned long long frags) {
  frags = warp_sum_u64(frags);
  if ((threadIdx.x & 31) == 0 && frags) atomicAdd(&ws.ctr->frag_ref, frags);
}

__device__ __forceinline__ void load_tri_pos(const gbr_triangle* T, f3 v[3], uint32_t* o_id) {
  const float* base = reinterpret_cast<const float*>(T);
  float4 a = __ldg(reinterpret_cast<const float4*>(base));       // v0.pos
  float4 b = __ldg(reinterpret_cast<const float4*>(base + 8));   // v0.vt, object_id, col
  float4 c = __ldg(reinterpret_cast<const float4*>(base + 12));  // v1.pos
  float4 d = __ldg(reinterpret_cast<const float4*>(base + 24));  // v2.pos
  v[0] = mk3(a.x, a.y, a.z);
  v[1] = mk3(c.x, c.y, c.z);
  v[2] = mk3(d.x, d.y, d.z);
  *o_id = __float_as_uint(b.z);
}


// World-space vertices of every triangle: rot_quat(v * scale, q) + world_pos,
// the object half of full_rotate_quat (cl2.cl:700-710).  It does not depend on
// the camera, so one pass serves the view and all cube faces until the
// triangles or descriptors change.
// Also the radius of each object's world-space vertices around its
// world_pos (objr, float bits, zeroed before): the bounding sphere of the
// object cull.
__global__ void __launch_bounds__(256) k_world(SceneDev sc, float4* __restrict__ world, uint32_t* __restrict__ objr) {
  const uint32_t tri = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = tri < sc.ntris;
  uint32_t o_id = 0;
  float rmax = 0.0f;
  if (valid) {
    f3 v[3];
    load_tri_pos(sc.tris + tri, v, &o_id);
    const gbr_obj_g_descriptor* G = sc.descs + o_id;
    const f4 qn = fast_normalize4(ld4(G->world_rot_quat));
    const f3 wp = ld3(G->world_pos);
    const float scale = __ldg(&G->scale);
    float4* out = world + (size_t)tri * 3;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      f3 r = add3(rot_quat_n(mul3s(v[k], scale), qn), wp);
      out[k] = make_float4(r.x, r.y, r.z, k == 0 ? __uint_as_float(o_id) : 0.0f);
      const float d = fast_length3(sub3(r, wp));
      rmax = d == d ? fmax_(rmax, d) : __int_as_float(0x7F800000);  // a NaN vertex disables the cull
    }
  }
  // the largest radius per object, aggregated over the warp's lanes of that object
  const unsigned act = __ballot_sync(0xFFFFFFFFu, valid);
  if (valid) {
    const unsigned grp = __match_any_sync(act, o_id);
    const uint32_t m = __reduce_max_sync(grp, __float_as_uint(rmax));  // non-negative floats order as integers
    if ((threadIdx.x & 31) == (uint32_t)(__ffs(grp) - 1)) atomicMax(objr + o_id, m);
  }
}

// Object cull of a view pass: bit o of row v is 0 when every triangle of
// object o is culled by prearrange's own tests in view v, so its setup
// threads stop after reading the object id.  Object o lies within radius
// objr[o] of its world_pos.  It is culled when it is farther than depth_far
// (the reference's object test, exactly), or when its bounding sphere lies
// entirely behind the near clip (z <= 20) or beyond the far clip (z >
// 350000) -- every vertex is then clipped away -- or, lying entirely nearer
// than the far clip, beyond one side plane of the view.  In that last case a
// clipped vertex lies on an edge between a vertex behind the near clip and
// one in front of it, inside the same half-space, so every projected vertex
// is off-screen on that side and the off-screen cull removes the triangle
// (cl2.cl:4352-4377).  (A vertex beyond the far clip is also clipped against
// z = 20, by extrapolation along its edge, which can leave the half-space:
// hence the far-clip condition.)  The margins (a relative 1e-3 of the radius
// and of the distance, plus one unit) are orders of magnitude above the
// float rounding of the per-triangle transform.
__global__ void __launch_bounds__(256) k_object_cull(SceneDev sc, const ViewParams* __restrict__ views,
                                                     const Surface* __restrict__ surfs, const uint32_t* __restrict__ objr,
                                                     uint32_t words, uint32_t* __restrict__ vis) {
  const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t v = blockIdx.y;
  bool keep = false;
  if (o < sc.ndescs) {
    const ViewParams& V = views[v];
    const Surface& S = surfs[V.surface];
    const f3 cpos = mk3(V.cpos[0], V.cpos[1], V.cpos[2]);
    const float4 q2 = __ldg(sc.objq + (size_t)o * kObjQuads + 2);
    const f3 wp = mk3(q2.x, q2.y, q2.z);
    const float dist = fast_length3(sub3(wp, cpos));
    if (!(dist > kDepthFar)) {
      const float r = __uint_as_float(__ldg(objr + o));
      const float m = r * 1.001f + dist * 1e-3f + 1.0f;
      const f3 q = rot_cs(wp, cpos, mk3(V.ccos[0], V.ccos[1], V.ccos[2]), mk3(V.csin[0], V.csin[1], V.csin[2]));
      // side planes through the camera: x * fov = -+ z * W/2, y * fov = -+ z * H/2
      const float hw = (float)S.width * 0.5f, hh = (float)S.height * 0.5f;
      const float nx = rsqrtf(V.fov * V.fov + hw * hw), ny = rsqrtf(V.fov * V.fov + hh * hh);
      const bool side = (q.x * V.fov + q.z * hw) * nx < -m || (q.x * V.fov - q.z * hw) * nx > m ||
                        (q.y * V.fov + q.z * hh) * ny < -m || (q.y * V.fov - q.z * hh) * ny > m;
      const bool out = q.z + m < kDepthCutoff || q.z - m > kDepthFar || (q.z + m < kDepthFar && side);
      keep = !out || !(m < 1e30f);  // an infinite or NaN radius culls nothing
    }
  }
  const unsigned bits = __ballot_sync(0xFFFFFFFFu, keep);
  if ((threadIdx.x & 31) == 0 && (o >> 5) < words) vis[(size_t)v * words + (o >> 5)] = bits;
}

// Per object: the normalised rotation quaternion rot_quat applies, and the
// normalised inverse back_rot_quat applies (conjugate / |q|^2, normalised by
// rot_quat) -- the same arithmetic every pixel of kernel3 would repeat.
__device__ __forceinline__ f4 quat_inverse_n(f4 q) {
  f4 conj; conj.x = -q.x; conj.y = -q.y; conj.z = -q.z; conj.w = q.w;
  float len_sq = dot4(conj, conj);
  f4 n; n.x = fdiv(conj.x, len_sq); n.y = fdiv(conj.y, len_sq);
  n.z = fdiv(conj.z, len_sq); n.w = fdiv(conj.w, len_sq);
  return fast_normalize4(n);
}

// and the material terms kernel3 reads (kObjQuads float4 per object).
__global__ void __launch_bounds__(256) k_objects(SceneDev sc, float4* __restrict__ objq) {
  const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= sc.ndescs) return;
  const gbr_obj_g_descriptor* G = sc.descs + o;
  const f4 q = ld4(G->world_rot_quat);
  const f4 qn = fast_normalize4(q), qi = quat_inverse_n(q);
  float4* d = objq + (size_t)kObjQuads * o;
  d[0] = make_float4(qn.x, qn.y, qn.z, qn.w);
  d[1] = make_float4(qi.x, qi.y, qi.z, qi.w);
  d[2] = make_float4(__ldg(&G->world_pos[0]), __ldg(&G->world_pos[1]), __ldg(&G->world_pos[2]), __ldg(&G->diffuse));
  d[3] = make_float4(__ldg(&G->spec_mult), clampf_(1.0f - __ldg(&G->specular), 0.001f, 10.0f),
                     __int_as_float(__ldg(&G->feature_flag)), __uint_as_float(__ldg(&G->tid)));
}

// The atlas slot of level L of texture t (slot descriptor nums[...] = page <<
// 16 | slot; pages are powers of two, 16..2048, so the slot's row and column
// within its page are exact in integers): the texture level table entry.
__global__ void __launch_bounds__(256) k_texture_levels(const uint32_t* __restrict__ nums,
                                                        const uint32_t* __restrict__ sizes, uint32_t mipmap_start,
                                                        float4* __restrict__ texlv) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= mipmap_start * kTexLevels) return;
  const uint32_t t = i / kTexLevels, L = i % kTexLevels;
  const uint32_t nv = nums[L == 0 ? t : mipmap_start + t * kMipLevels + (L - 1)];
  const uint32_t page = nv >> 16, which = nv & 0xFFFFu;
  const uint32_t w = sizes[page];
  const uint32_t hnum = (uint32_t)kTexPage / w;
  const uint32_t row = which / hnum, col = which - row * hnum;
  texlv[i] = make_float4((float)(col * w), (float)(row * w), (float)w, __uint_as_float(page));
}

// World-space vertices of a triangle: from the scene's cache when there is
// one, else computed here with the same arithmetic as k_world.
__device__ __forceinline__ void load_world(const SceneDev& sc, uint32_t tri, f3 w[3], uint32_t* o_id) {
  if (!sc.world) {
    f3 v[3];
    load_tri_pos(sc.tris + tri, v, o_id);
    const gbr_obj_g_descriptor* G = sc.descs + *o_id;
    const f4 qn = fast_normalize4(ld4(G->world_rot_quat));
    const f3 wp = ld3(G->world_pos);
    const float scale = __ldg(&G->scale);
#pragma unroll
    for (int k = 0; k < 3; k++) w[k] = add3(rot_quat_n(mul3s(v[k], scale), qn), wp);
    return;
  }
  const float4* p = sc.world + (size_t)tri * 3;
  float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
  w[0] = mk3(a.x, a.y, a.z);
  w[1] = mk3(b.x, b.y, b.z);
  w[2] = mk3(c.x, c.y, c.z);
  *o_id = __float_as_uint(a.w);
}

// The camera half of full_rotate_quat (cl2.cl:700-729): world -> camera
// space, near/far clip, projection.
__device__ __forceinline__ int transform_clip(const f3 w[3], f3 cpos, f3 c, f3 s, float fov, float width,
                                              float height, f3 o0[3], f3 o1[3]) {
  f3 t0[3], t1[3];
  const int n = clip_tri_reg(rot_cs(w[0], cpos, c, s), rot_cs(w[1], cpos, c, s), rot_cs(w[2], cpos, c, s), t0, t1);
  if (n > 0) {
#pragma unroll
    for (int k = 0; k < 3; k++) o0[k] = depth_project1(t0[k], width, height, fov);
  }
  if (n > 1) {  // only a triangle with one vertex behind the near plane splits
#pragma unroll
    for (int k = 0; k < 3; k++) o1[k] = depth_project1(t1[k], width, height, fov);
  }
  return n;
}

// prearrange's handling of one (triangle, surface): up to two clip outputs,
// culled, as candidates c0 (first survivor) and c1.
__device__ __forceinline__ int make_cands(const f3 w[3], f3 cpos, f3 c, f3 s, float fov, float width, float height,
                                          bool two, uint32_t tri, Cand& c0, Cand& c1) {
  f3 o0[3], o1[3];
  const int num = transform_clip(w, cpos, c, s, fov, width, height, o0, o1);
  int n = 0;
  if (num > 0) {
    c0.p[0] = o0[0]; c0.p[1] = o0[1]; c0.p[2] = o0[2];
    c0.key = tri * 2u;
    if (cull_candidate(c0, two, width, height)) n = 1;
  }
  if (num > 1) {
    Cand& d = n ? c1 : c0;
    d.p[0] = o1[0]; d.p[1] = o1[1]; d.p[2] = o1[2];
    d.key = tri * 2u + 1u;
    if (cull_candidate(d, two, width, height)) n++;
  }
  return n;
}

// prearrange (cl2.cl:4271-4409), one thread per (triangle, view).
__global__ void __launch_bounds__(256) k_setup_views(SceneDev sc, const ViewParams* __restrict__ views,
                                                     const Surface* __restrict__ surfs, Workspace ws) {
  uint32_t tri = blockIdx.x * blockDim.x + threadIdx.x;
  const ViewParams& V = views[blockIdx.y];
  const Surface& S = surfs[V.surface];
  Cand c0, c1;
  int n = 0;
  // the object cull (k_object_cull), when the pass has one: the object id
  // alone decides
  bool live = tri < sc.ntris;
  if (live && ws.vis) {
    const uint32_t o_id = __float_as_uint(__ldg(&sc.world[(size_t)tri * 3].w));
    live = (__ldg(ws.vis + (size_t)blockIdx.y * ws.vis_words + (o_id >> 5)) >> (o_id & 31)) & 1u;
  }
  // a warp with nothing to set up (objects are mostly contiguous runs of
  // triangles) leaves before emit's warp-wide work
  if (!__any_sync(0xFFFFFFFFu, live)) return;
  if (live) {
    f3 wv[3];
    uint32_t o_id;
    load_world(sc, tri, wv, &o_id);
    const gbr_obj_g_descriptor* G = sc.descs + o_id;
    f3 cpos = mk3(V.cpos[0], V.cpos[1], V.cpos[2]);
    if (!(fast_length3(sub3(ld3(G->world_pos), cpos)) > kDepthFar)) {
      f3 c = mk3(V.ccos[0], V.ccos[1], V.ccos[2]);
      f3 s = mk3(V.csin[0], V.csin[1], V.csin[2]);
      const bool two = (__ldg(&G->feature_flag) & kFlagTwoSided) > 0;
      n = make_cands(wv, cpos, c, s, V.fov, (float)S.width, (float)S.height, two, tri, c0, c1);
    }
  }
  add_frags(ws, emit(c0, c1, n, V.surface, surfs, ws, true));
}

// prearrange_realtime_shadowing (cl2.cl:4419-4636), one thread per (triangle, light job).
__global__ void __launch_bounds__(128, 6) k_setup_shadow(SceneDev sc, const ShadowJob* __restrict__ jobs,
                                                      const Surface* __restrict__ surfs, Workspace ws) {
  uint32_t tri = blockIdx.x * blockDim.x + threadIdx.x;
  const ShadowJob& J = jobs[blockIdx.y];
  const float L = (float)kLightBufferDim;
  int mask = 0;
  f3 wv[3];
  f3 lpos = mk3(J.lpos[0], J.lpos[1], J.lpos[2]);
  bool two = false;
  if (tri < sc.ntris) {
    uint32_t o_id;
    load_world(sc, tri, wv, &o_id);
    const gbr_obj_g_descriptor* G = sc.descs + o_id;
    int ff = __ldg(&G->feature_flag);
    bool is_static = (ff & kFlagIsStatic) > 0;
    two = (ff & kFlagTwoSided) > 0;
    f3 wp = ld3(G->world_pos);
    if (is_static == (J.only_static != 0) && !(fast_length3(sub3(wp, lpos)) > kDepthFar)) {
      for (int k = 0; k < 3; k++) mask |= 1 << ret_cubeface(wv[k], lpos);
    }
  }
  unsigned long long frags = 0;
  for (int face = 0; face < 6; face++) {
    if (!__any_sync(0xFFFFFFFFu, mask & (1 << face))) continue;  // warp-uniform
    Cand c0, c1;
    int n = 0;
    if (mask & (1 << face)) {
      f3 c = mk3(sc.face_cos[face][0], sc.face_cos[face][1], sc.face_cos[face][2]);
      f3 s = mk3(sc.face_sin[face][0], sc.face_sin[face][1], sc.face_sin[face][2]);
      n = make_cands(wv, lpos, c, s, kLFov, L, L, two, tri, c0, c1);
    }
    frags += emit(c0, c1, n, J.surface_base + face, surfs, ws, false);
  }
  add_frags(ws, frags);
}

// Each fine tile's surface (binary search over tile_base) and global coarse
// tile: the raster's and kernel3's first loads.
__global__ void __launch_bounds__(256) k_tile_table(const Surface* __restrict__ surfs, uint32_t nsurf,
                                                    uint32_t nfine, int coarse_shift, uint2* __restrict__ tiles) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nfine) return;
  uint32_t lo = 0, hi = nsurf - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (surfs[mid].tile_base <= t) lo = mid; else hi = mid - 1;
  }
  const Surface& S = surfs[lo];
  const uint32_t lt = t - S.tile_base;
  const int tx = lt % S.tiles_x, ty = lt / S.tiles_x;
  tiles[t] = make_uint2(lo, S.ctile_base + (ty >> coarse_shift) * S.ctiles_x + (tx >> coarse_shift));
}

// Exclusive scan of fine and coarse tile counts (one block of 1024 threads);
// counts are reset to zero to serve as fill cursors.  Rounds of 8192 counts
// are staged in shared memory with coalesced loads, each thread scans 8
// contiguous values, and a block scan joins the threads.
constexpr int kScanThreads = 1024;
constexpr int kScanPer = 8;
constexpr int kScanChunk = kScanThreads * kScanPer;

__device__ __forceinline__ uint32_t block_scan_1024(uint32_t v, uint32_t* swarp, uint32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) swarp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const uint32_t w = swarp[lane];
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xFFFFFFFFu, wi, o);
      if (lane >= o) wi += t;
    }
    swarp[lane] = wi - w;
    if (lane == 31) *total = wi;
  }
  __syncthreads();
  return swarp[warp] + incl - v;
}

__device__ void block_scan_array(uint32_t* count, uint32_t* off, uint32_t n, uint32_t* total, uint32_t* sh,
                                 uint32_t* swarp, uint32_t* sctot) {
  uint32_t carry = 0;
  for (uint32_t c0 = 0; c0 < n; c0 += kScanChunk) {
    const uint32_t m = min((uint32_t)kScanChunk, n - c0);
    for (uint32_t i = threadIdx.x; i < (uint32_t)kScanChunk; i += kScanThreads) sh[i] = i < m ? count[c0 + i] : 0u;
    __syncthreads();
    uint32_t v[kScanPer], sum = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
      v[k] = sh[threadIdx.x * kScanPer + k];
      sum += v[k];
    }
    const uint32_t excl = block_scan_1024(sum, swarp, sctot);
    uint32_t run = carry + excl;
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
      sh[threadIdx.x * kScanPer + k] = run;
      run += v[k];
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < m; i += kScanThreads) {
      off[c0 + i] = sh[i];
      count[c0 + i] = 0;
    }
    carry += *sctot;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(kScanThreads) k_scan(Workspace ws) {
  __shared__ uint32_t sh[kScanChunk];
  __shared__ uint32_t swarp[32];
  __shared__ uint32_t sctot;
  block_scan_array(ws.fine_count, ws.fine_off, ws.nfine, &ws.ctr->fine_total, sh, swarp, &sctot);
  block_scan_array(ws.coarse_count, ws.coarse_off, ws.ncoarse, &ws.ctr->coarse_total, sh, swarp, &sctot);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint64_t need = (uint64_t)ws.ctr->fine_total + ws.ctr->coarse_total;
    if (need > ws.bin_cap) ws.ctr->overflow |= 2u;
  }
}

// Barycentrics (cl2.cl:5372-5384) split into the per-triangle part and the
// per-point part; bary_exact is barycentric() bit for bit.
struct BaryFrame {
  f3 a, v0, v1;
  float d00, d01, d11, denom;
};
__device__ __forceinline__ BaryFrame bary_frame(f3 a, f3 b, f3 c) {
  BaryFrame f;
  f.a = a;
  f.v0 = sub3(b, a);
  f.v1 = sub3(c, a);
  f.d00 = dot3(f.v0, f.v0);
  f.d01 = dot3(f.v0, f.v1);
  f.d11 = dot3(f.v1, f.v1);
  f.denom = f.d00 * f.d11 - f.d01 * f.d01;
  return f;
}
__device__ __forceinline__ void bary_exact(const BaryFrame& f, f3 p, float* u, float* v, float* w) {
  f3 v2 = sub3(p, f.a);
  float d20 = dot3(v2, f.v0), d21 = dot3(v2, f.v1);
  *v = fdiv(f.d11 * d20 - f.d01 * d21, f.denom);
  *w = fdiv(f.d00 * d21 - f.d01 * d20, f.denom);
  *u = (1.0f - *v) - *w;
}
// kernel3's per-triangle arithmetic for one view record, in place: the
// setup's projected vertices, rconst and triangle index become the
// barycentric frame (cl2.cl:5372-5384) of the scaled object-space vertices,
// get_vtdiff's 1/z plane through the rounded vertices (cl2.cl:5691-5760), the
// vertex normals, UVs and colours, and the facing (cl2.cl:491-494).  Every
// value is computed with the arithmetic kernel3 applies per pixel in the
// reference, so the pixels read exactly what they would compute.
__device__ __forceinline__ void prep_shade(const SceneDev& sc, ShadeRec* R) {
  const float4 q0 = R->a, q1 = R->e0, q2 = R->e1;  // the setup's output (this thread alone touches it)
  const f3 tp0 = mk3(q0.x, q0.y, q0.z), tp1 = mk3(q1.x, q1.y, q1.z), tp2 = mk3(q2.x, q2.y, q2.z);
  const uint32_t tri = __float_as_uint(q1.w);
  // the triangle as 9 float4 loads: per vertex pos, normal, (vt, object_id, vertex_col)
  const float4* tv = reinterpret_cast<const float4*>(sc.tris + tri);
  const float4 va0 = __ldg(tv + 0), vb0 = __ldg(tv + 1), vc0 = __ldg(tv + 2);
  const float4 va1 = __ldg(tv + 3), vb1 = __ldg(tv + 4), vc1 = __ldg(tv + 5);
  const float4 va2 = __ldg(tv + 6), vb2 = __ldg(tv + 7), vc2 = __ldg(tv + 8);
  const uint32_t o_id = __float_as_uint(vc0.z);
  const float scale = __ldg(&sc.descs[o_id].scale);
  const BaryFrame bf = bary_frame(mul3s(mk3(va0.x, va0.y, va0.z), scale), mul3s(mk3(va1.x, va1.y, va1.z), scale),
                                  mul3s(mk3(va2.x, va2.y, va2.z), scale));
  const f3 xpv = mk3(roundf(tp0.x), roundf(tp1.x), roundf(tp2.x));
  const f3 ypv = mk3(roundf(tp0.y), roundf(tp1.y), roundf(tp2.y));
  const f3 depths = mk3(rcp(tp0.z), rcp(tp1.z), rcp(tp2.z));
  float DA, DB, DC;
  plane_const(depths, xpv, ypv, q0.w, &DA, &DB, &DC);
  const uint32_t back = backface_front(tp0, tp1, tp2) ? 0u : 0x80000000u;
  R->a = make_float4(bf.a.x, bf.a.y, bf.a.z, bf.d00);
  R->e0 = make_float4(bf.v0.x, bf.v0.y, bf.v0.z, bf.d01);
  R->e1 = make_float4(bf.v1.x, bf.v1.y, bf.v1.z, bf.d11);
  R->plane = make_float4(DA, DB, DC, bf.denom);
  R->n1 = make_float4(vb0.x, vb0.y, vb0.z, vc0.x);
  R->n2 = make_float4(vb1.x, vb1.y, vb1.z, vc0.y);
  R->n3 = make_float4(vb2.x, vb2.y, vb2.z, vc1.x);
  R->t = make_float4(vc1.y, vc2.x, vc2.y, __uint_as_float(o_id | back));
  R->col = make_float4(vc0.w, vc1.w, vc2.w, __uint_as_float(tri));
}

// The shade constants of every record of a view pass (after the setup; it
// runs beside the scan, fill and raster, which do not read them).
__global__ void __launch_bounds__(256, 4) k_prep(SceneDev sc, Workspace ws) {
  if (ws.ctr->overflow) return;
  const uint32_t nrec = min(ws.ctr->nrec, ws.rec_cap);
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < nrec; r += gridDim.x * blockDim.x)
    prep_shade(sc, ws.srec + r);
}

// Many tiles (batches of views): the fine counts are scanned in chunks of
// kScanChunk, one block each, into offsets relative to the chunk, with each
// chunk's total in scan_part; one more block scans the coarse counts whole.
// k_scan_add then adds the totals of the chunks before each chunk.
__global__ void __launch_bounds__(kScanThreads) k_scan_chunks(Workspace ws, uint32_t nchunks) {
  __shared__ uint32_t sh[kScanChunk];
  __shared__ uint32_t swarp[32];
  __shared__ uint32_t sctot;
  if (blockIdx.x == nchunks) {
    block_scan_array(ws.coarse_count, ws.coarse_off, ws.ncoarse, &ws.ctr->coarse_total, sh, swarp, &sctot);
    return;
  }
  const uint32_t c0 = blockIdx.x * (uint32_t)kScanChunk;
  const uint32_t m = min((uint32_t)kScanChunk, ws.nfine - c0);
  block_scan_array(ws.fine_count + c0, ws.fine_off + c0, m, ws.scan_part + blockIdx.x, sh, swarp, &sctot);
}

__global__ void __launch_bounds__(kScanThreads) k_scan_add(Workspace ws, uint32_t nchunks) {
  __shared__ uint32_t base;
  if (threadIdx.x < 32) {
    uint32_t sum = 0;
    for (uint32_t i = threadIdx.x; i < blockIdx.x; i += 32) sum += ws.scan_part[i];
    sum = __reduce_add_sync(0xFFFFFFFFu, sum);
    if (threadIdx.x == 0) base = sum;
  }
  __syncthreads();
  const uint32_t c0 = blockIdx.x * (uint32_t)kScanChunk;
  const uint32_t m = min((uint32_t)kScanChunk, ws.nfine - c0);
  for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) ws.fine_off[c0 + i] += base;
  if (blockIdx.x == nchunks - 1 && threadIdx.x == 0) {
    const uint32_t total = base + ws.scan_part[blockIdx.x];
    ws.ctr->fine_total = total;
    if ((uint64_t)total + ws.ctr->coarse_total > ws.bin_cap) ws.ctr->overflow |= 2u;
  }
}

// Scatter record indices into their tile bins (cursor atomics aggregated
// across the warp).
__global__ void __launch_bounds__(256) k_fill(Workspace ws, const Surface* __restrict__ surfs) {
  const uint32_t nrec = min(ws.ctr->nrec, ws.rec_cap);
  if (ws.ctr->overflow) return;
  const uint32_t coarse_base = ws.ctr->fine_total;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t r0 = blockIdx.x * blockDim.x; r0 < nrec; r0 += stride) {
    const uint32_t r = r0 + threadIdx.x;
    const bool valid = r < nrec;
    Foot f{0, 0, 0, 0, false};
    const Surface* S = surfs;
    int total = 0;
    if (valid) {
      float4 q = __ldg(reinterpret_cast<const float4*>(ws.rec + r) + 3);
      S = surfs + __float_as_uint(q.z);
      f = footprint(__float_as_uint(q.x), __float_as_uint(q.y), ws);
      total = foot_count(f);
    }
    int maxt = total;
    for (int o = 16; o > 0; o >>= 1) maxt = max(maxt, __shfl_xor_sync(0xFFFFFFFFu, maxt, o));
    for (int it = 0; it < maxt; it++) {
      const bool act = it < total;
      const uint32_t tile = act ? foot_tile(f, it, *S) : 0u;
      const uint32_t pf = agg_inc(ws.fine_count, tile, act && !f.coarse);
      const uint32_t pc = agg_inc(ws.coarse_count, tile, act && f.coarse);
      if (act) {
        const uint32_t pos = f.coarse ? coarse_base + ws.coarse_off[tile] + pc : ws.fine_off[tile] + pf;
        ws.bins[pos] = r;
      }
    }
  }
}




// kernel1 + kernel2 for one 16x16 tile: depth min, then the canonical id.
//
// The tile's records (its fine bin, then its coarse tile's bin) are staged NT
// at a time in shared memory, keeping those whose bbox meets the tile.  Each
// contributes the horizontal pixel pairs of its bbox clipped to the tile (a
// test covers one pair: the record's loads and decode serve two pixels); one
// block scan (packing the record count and the pair count) compacts them and
// lays all (record, pair) tests of the chunk end to end.  Each warp takes one
// contiguous range of that list, finds its first record by binary search,
// and then maps 32 tests at a time to records with one ballot of the record
// starts inside the window (every staged record has at least one pair, so
// at most 32 start there), so small and large triangles are load-balanced
// alike.  Pass 0 resolves the minimum depth with shared-memory atomicMin;
// pass 1 the minimum packed (key << 32 | record) among tests within +-20 of
// the final depth.  Both are minima, so neither bin order nor thread order
// changes the result.  When the whole list fits one chunk and each lane has
// at most kRasterCache covered pixels, pass 1 reuses the covered pixels of
// pass 0 kept in shared memory.
constexpr int kRasterCache = 8;
// Cache slots of an NT-thread view raster: 512-thread CTAs keep none (their
// static shared memory stays under 48 KB) and re-test in the id pass.
template <int NT>
__host__ __device__ constexpr int raster_cache_slots() { return NT <= 256 ? kRasterCache : 0; }
constexpr uint32_t kSlotBits = 9;  // staged slots of a one-chunk tile: below 512

// Exclusive block scan with a single barrier: each warp scans its lanes,
// publishes its total, and after the barrier every thread adds up the totals
// of the warps before its own (and of all warps, the block total).
template <int NT>
__device__ __forceinline__ uint32_t block_excl_scan1(uint32_t v, uint32_t* swarp, uint32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) swarp[warp] = incl;
  __syncthreads();
  uint32_t before = 0, all = 0;
#pragma unroll
  for (int w = 0; w < NT / 32; w++) {
    const uint32_t t = swarp[w];
    all += t;
    if (w < warp) before += t;
  }
  *total = all;
  return before + incl - v;
}


// Shared-memory slot of tile pixel p = ly * 16 + lx in the per-pixel depth
// (32-bit words) and id (64-bit words) arrays: a row of 16 pixels fills 16
// of the 32 banks, so rows y and y + 2 (64-bit: y and y + 1) would share
// banks and a narrow triangle's tests collide.  32-bit: each 32-word line
// (a row pair) is rotated by 4 banks per line, so that a footprint up to 4
// pixels wide and 8 rows tall falls on distinct banks; 64-bit: the column is
// XOR-ed with the row.  Permutations within each line (row).
__device__ __forceinline__ int swz32(int p) {
  const int line = p >> 5;
  return (line << 5) | ((p + 4 * line) & 31);
}
__device__ __forceinline__ int swz64(int p) { return p ^ ((p >> 4) & 15); }

// kernel3's RGBA8 output word
__device__ __forceinline__ uint32_t pack_rgba(float r, float g, float b, float a) {
  return quant8(r) | (quant8(g) << 8) | (quant8(b) << 16) | (quant8(a) << 24);
}

// Shared memory of one tile's raster (NT threads; ID: views).
template <int NT, bool ID>
struct RasterSmem {
  float4 srec[4][NT];  // the staged records' four float4, one array each (conflict-free stores)
  uint32_t sidx[NT];
  uint32_t soff[NT + 1];
  uint32_t sgeo[NT];  // lx0 | ly0 << 4 | bw << 8 | ceil(65536 / pairs per row) << 13
  uint16_t sskip[NT];  // bit ly: the walk skips the record's left-column pixel in tile row ly
  // the covered pixels of pass 0 kept for the id pass: depth, and pixel |
  // staged record << 8; slot k of thread t at k * NT + t
  uint32_t scd[ID && raster_cache_slots<NT>() ? raster_cache_slots<NT>() * NT : 1];
  uint32_t scm[ID && raster_cache_slots<NT>() ? raster_cache_slots<NT>() * NT : 1];
  uint32_t sdepth[kTilePixels];
  unsigned long long sid[kTilePixels];
  uint32_t swarp[NT / 32];
  uint32_t sscan;
  uint32_t ssamples;
  Surface S;
  uint32_t s;  // the tile's surface
  uint32_t lists[4];
};

// NT threads per CTA (128, 256 or 512); ID: resolve the canonical id too
// (views) or only the depth (cube faces); CC: see chunk below.  surface: the
// tile's surface when the caller knows it, else -1 (ws.tiles, or the pass's
// only surface).  Every thread of the block calls it; the caller synchronises
// before reusing the shared memory.
template <int NT, bool ID, bool CC = false>
__device__ __forceinline__ void raster_tile(const Workspace& ws, const Surface* __restrict__ surfs, uint32_t nsurf,
                                            uint32_t tile, int surface, RasterSmem<NT, ID>& sm) {
  constexpr bool with_id = ID;
  constexpr int NW = NT / 32;
  constexpr uint32_t kCountShift = 18;  // scan word: pixels (< 2^18) | records << 18
  float4 (&srec)[4][NT] = sm.srec;
  uint32_t* sidx = sm.sidx;
  uint32_t* soff = sm.soff;
  uint32_t* sgeo = sm.sgeo;
  uint16_t* sskip = sm.sskip;
  uint32_t* sdepth = sm.sdepth;
  unsigned long long* sid = sm.sid;
  uint32_t* swarp = sm.swarp;
  uint32_t& sscan = sm.sscan;
  uint32_t& ssamples = sm.ssamples;
  Surface& S = sm.S;
  uint32_t* lists = sm.lists;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {  // the tile's surface and bins
    const uint32_t foff = ws.fine_off[tile], fcnt = ws.fine_count[tile], ftot = ws.ctr->fine_total;
    uint32_t s, ct;
    if (ws.tiles) {  // two rounds of loads
      const uint2 tt = ws.tiles[tile];
      s = surface >= 0 ? (uint32_t)surface : tt.x;
      ct = tt.y;
      S = surfs[s];
    } else {  // the surface is known (grid row, or the pass's only one)
      s = surface >= 0 ? (uint32_t)surface : 0u;
      S = surfs[s];
      const uint32_t lt = tile - S.tile_base;
      const int tx = lt % S.tiles_x, ty = lt / S.tiles_x;
      ct = S.ctile_base + (ty >> ws.coarse_shift) * S.ctiles_x + (tx >> ws.coarse_shift);
    }
    sm.s = s;
    lists[0] = foff;
    lists[1] = fcnt;
    lists[2] = ftot + ws.coarse_off[ct];
    lists[3] = ws.coarse_count[ct];
    ssamples = 0;
  }
  if (with_id) {
    for (int p = tid; p < kTilePixels; p += NT) {
      sdepth[p] = kDepthClear;
      sid[p] = ~0ull;
    }
  }
  __syncthreads();
  const uint32_t lt = tile - S.tile_base;
  const int tx0 = (lt % S.tiles_x) * kTile, ty0 = (lt / S.tiles_x) * kTile;
  if (with_id && lists[1] + lists[3] == 0) {  // no records: an empty tile
    // kernel3's output here is the clear colour and zero normals, unless the
    // view blends in another context's colour: write it, and mark the tile
    // (kernel3 then reads nothing of it, the record map included)
    uint32_t* rgba = nullptr;
    uint32_t* nrm = nullptr;
    uint32_t* rmap = S.rec;
    uint32_t clear = 0;
    if (ws.tile_empty) {
      const ViewParams& V = ws.views[sm.s];
      const bool direct = V.blend_depth == nullptr;
      if (direct) {
        rgba = reinterpret_cast<uint32_t*>(V.rgba);
        nrm = reinterpret_cast<uint32_t*>(V.normals);
        rmap = nullptr;
        clear = pack_rgba(V.clear[0], V.clear[1], V.clear[2], V.clear[3]);
      }
      if (tid == 0) ws.tile_empty[tile] = direct ? 1 : 0;
    }
    for (int lp = tid; lp < kTilePixels; lp += NT) {
      const int px = tx0 + (lp & (kTile - 1)), py = ty0 + (lp / kTile);
      if (px < S.width && py < S.height) {
        const size_t p = (size_t)py * S.width + px;
        S.depth[p] = kDepthClear;
        if (S.id) S.id[p] = kNoId;
        if (rmap) rmap[p] = kNoId;
        if (rgba) rgba[p] = clear;
        if (nrm) nrm[p] = 0;
      }
    }
    return;
  }
  if (with_id && ws.tile_empty && tid == 0) ws.tile_empty[tile] = 0;
  if (!with_id) {
    // depth-only passes: the surface was cleared and holds the small
    // triangles the setup rasterised; a tile without records keeps it as is
    if (lists[1] + lists[3] == 0) return;
    for (int p = tid; p < kTilePixels; p += NT) {
      const int px = tx0 + (p & (kTile - 1)), py = ty0 + p / kTile;
      sdepth[swz32(p)] = (px < S.width && py < S.height) ? S.depth[(size_t)py * S.width + px] : kDepthClear;
    }
  }
  // the walk's fragment size (Surface.chunk: op_size for views, op_size_light
  // for cube faces).  CC (passes of several view surfaces) takes it as the
  // constant op_size, so that the walk rule's modulos are multiplications:
  // 1.8 % faster batches; the one-view raster measured faster with the
  // runtime value
  const int chunk = CC ? kOpSize : S.chunk;
  const uint32_t nfine = lists[1], ntotal = lists[1] + lists[3];
  const int passes = ntotal == 0 ? 0 : (with_id ? 2 : 1);
  const bool resident = ntotal <= (uint32_t)NT;
  // A tile resolved in one chunk keeps the canonical id as 32 bits, key <<
  // kSlotBits | staged slot (keys of the scene below ws.pack_keys): a record
  // has one key, so the minimum of these picks the same record as the
  // minimum of (key << 32 | record), with half the shared-memory traffic.
  const bool packed = with_id && resident && ws.pack_keys;
  uint32_t* sid32 = reinterpret_cast<uint32_t*>(sid);
  // the covered tests of pass 0 (resident tiles), up to kRasterCache per
  // thread, kept in sm.scd / sm.scm; nh counts them
  uint32_t nh = 0;
  uint32_t wsamples = 0;  // covered tests of pass 0 seen by this warp
  bool cached = false;
  for (int pass = 0; pass < passes; pass++) {
    for (uint32_t c0 = 0; c0 < ntotal; c0 += NT) {
      const uint32_t m = min((uint32_t)NT, ntotal - c0);
      if (!(resident && pass == 1)) {
        if (pass != 0 || c0 != 0) __syncthreads();  // the previous chunk's readers are done
        uint32_t area = 0, r = 0, geo = 0, skip = 0;
        float4 q0, q1, q2, q3;
        if ((uint32_t)tid < m) {
          const uint32_t e = c0 + tid;
          r = e < nfine ? ws.bins[lists[0] + e] : ws.bins[lists[2] + (e - nfine)];
          const float4* src = reinterpret_cast<const float4*>(ws.rec + r);
          q0 = __ldg(src);
          q1 = __ldg(src + 1);
          q2 = __ldg(src + 2);
          q3 = __ldg(src + 3);
          const uint32_t xr = __float_as_uint(q3.x), yr = __float_as_uint(q3.y);
          const int bx0 = max((int)(xr & 0xFFFF), tx0), bx1 = min((int)(xr >> 16), tx0 + kTile);
          const int by0 = max((int)(yr & 0xFFFF), ty0), by1 = min((int)(yr >> 16), ty0 + kTile);
          if (bx1 > bx0 && by1 > by0) {
            // the tests are horizontal pixel pairs: ceil(bw / 2) per row
            const uint32_t bw = (uint32_t)(bx1 - bx0), pw = (bw + 1) >> 1;
            area = pw * (uint32_t)(by1 - by0);
            geo = (uint32_t)(bx0 - tx0) | ((uint32_t)(by0 - ty0) << 4) | (bw << 8) | (((65536u + pw - 1) / pw) << 13);
            // the walk rule of the bbox's left column, once per row of this tile
            if ((int)(xr & 0xFFFF) >= tx0) skip = walk_skip_rows(xr, yr, by0, by1, ty0, chunk);
          }
        }
        const uint32_t word = area ? (area | (1u << kCountShift)) : 0u;
        uint32_t tot = 0;
        const uint32_t off = block_excl_scan1<NT>(word, swarp, &tot);
        if (area) {
          const uint32_t slot = off >> kCountShift;
          srec[0][slot] = q0;
          srec[1][slot] = q1;
          srec[2][slot] = q2;
          srec[3][slot] = q3;
          sidx[slot] = r;
          sgeo[slot] = geo;
          sskip[slot] = (uint16_t)skip;
          soff[slot] = off & ((1u << kCountShift) - 1);
        }
        if (tid == 0) {
          soff[tot >> kCountShift] = tot & ((1u << kCountShift) - 1);
          sscan = tot;
        }
        __syncthreads();
      }
      const uint32_t nstaged = sscan >> kCountShift;
      const uint32_t total = soff[nstaged];
      if (resident && pass == 1 && cached) {
        // pass 1 from the tests pass 0 kept
        for (uint32_t g = 0; g < nh; g++) {
          const uint32_t cm = sm.scm[g * NT + tid];
          const int p = (int)(cm & 0xFF);
          const uint32_t lo = (cm >> 8) & 0x3FF;
          const uint32_t d = sm.scd[g * NT + tid], fd = sdepth[swz32(p)];
          if (d > fd - kBufError && d < fd + kBufError) {
            const uint32_t key = __float_as_uint(srec[2][lo].w);
            if (packed)
              atomicMin(sid32 + swz32(p), (key << kSlotBits) | lo);
            else
              atomicMin(&sid[swz64(p)], ((unsigned long long)key << 32) | sidx[lo]);
          }
        }
        continue;
      }
      // this warp's contiguous range of the test list, in windows of 32
      const uint32_t per = ((total + NW * 32 - 1) / (NW * 32)) * 32;
      const uint32_t start = min(total, (uint32_t)warp * per), end = min(total, start + per);
      const bool keep = resident && pass == 0 && with_id && raster_cache_slots<NT>() > 0;
      if (start < end) {
        // first record: the last staged record with soff <= start (warp-uniform)
        int rec = 0, hi = (int)nstaged - 1;
        while (rec < hi) {
          const int mid = (rec + hi + 1) >> 1;
          if (soff[mid] <= start) rec = mid; else hi = mid - 1;
        }
#pragma unroll 1
        for (uint32_t base = start; base < end; base += 32) {
          // record starts inside (base, base + 32): at most 32 records
          const uint32_t nxt = (uint32_t)rec + 1 + lane;
          const uint32_t pos = nxt < nstaged ? soff[nxt] - base : 32u;
          const uint32_t starts = __reduce_or_sync(0xFFFFFFFFu, pos < 32u ? (1u << pos) : 0u);
          const uint32_t upto = lane == 31 ? starts : starts & ((2u << lane) - 1u);
          const uint32_t lo = (uint32_t)rec + __popc(upto);
          const uint32_t t = base + lane;
          uint32_t nhit = 0;
          if (t < end) {
            // test t of the record: the pixel pair (lx, ly), (lx + 1, ly)
            const uint32_t geo = sgeo[lo];
            const uint32_t local = t - soff[lo];
            const uint32_t bw = (geo >> 8) & 0x1F, pw = (bw + 1) >> 1;
            const uint32_t ry = (local * (geo >> 13)) >> 16, rp = local - ry * pw;
            const int lx = (int)(geo & 0xF) + 2 * (int)rp, ly = (int)((geo >> 4) & 0xF) + (int)ry;
            const float4 q[4] = {srec[0][lo], srec[1][lo], srec[2][lo], srec[3][lo]};
            const int x = tx0 + lx, y = ty0 + ly;
            // covers_in_bbox, the walk rule from the staged mask (only the
            // first pixel of a pair can be the bbox's left column)
            const bool h0 = !(x == (int)(__float_as_uint(q[3].x) & 0xFFFF) && ((sskip[lo] >> ly) & 1)) &&
                            rec_in_tri(q, x, y);
            const bool h1 = 2 * rp + 1 < bw && rec_in_tri(q, x + 1, y);
            auto resolve = [&](int px, int plx) {
              const uint32_t d = depth_at(q[0].x, q[0].y, q[0].z, (float)px, (float)y);
              const int p = ly * kTile + plx;
              if (pass == 0) {
                atomicMin(&sdepth[swz32(p)], d);
                if (keep) {
                  if (nh < (uint32_t)raster_cache_slots<NT>()) {
                    sm.scd[nh * NT + tid] = d;
                    sm.scm[nh * NT + tid] = (uint32_t)p | (lo << 8);
                  }
                  nh++;
                }
              } else {
                const uint32_t fd = sdepth[swz32(p)];
                if (d > fd - kBufError && d < fd + kBufError) {
                  if (packed)
                    atomicMin(sid32 + swz32(p), (__float_as_uint(q[2].w) << kSlotBits) | lo);
                  else
                    atomicMin(&sid[swz64(p)], ((unsigned long long)__float_as_uint(q[2].w) << 32) | sidx[lo]);
                }
              }
            };
            if (h0) resolve(x, lx);
            if (h1) resolve(x + 1, lx + 1);
            nhit = (uint32_t)h0 + (uint32_t)h1;
          }
          if (pass == 0) wsamples += __reduce_add_sync(0xFFFFFFFFu, nhit);
          // the record of test base + 32: lane 31's, or the next one if it starts there
          rec = (int)((uint32_t)rec + __popc(starts));
          if ((uint32_t)rec + 1 < nstaged && soff[rec + 1] == base + 32) rec++;
        }
      }
    }
    if (pass == 0 && lane == 0 && wsamples) atomicAdd(&ssamples, wsamples);
    // a resident tile's id pass reads pass 0's kept tests when every thread's
    // fit (block-uniform)
    if (resident && with_id && pass == 0) {
      const bool over = __syncthreads_or(nh > (uint32_t)raster_cache_slots<NT>()) != 0;
      cached = raster_cache_slots<NT>() > 0 && !over;
    } else {
      __syncthreads();
    }
  }
  if (tid == 0 && ssamples) atomicAdd(&ws.ctr->samples, (unsigned long long)ssamples);
  for (int lp = tid; lp < kTilePixels; lp += NT) {
    const int px = tx0 + (lp & (kTile - 1)), py = ty0 + (lp / kTile);
    if (px < S.width && py < S.height) {
      const size_t p = (size_t)py * S.width + px;
      S.depth[p] = sdepth[swz32(lp)];
      if (with_id && packed) {
        const uint32_t v = sid32[swz32(lp)];
        if (S.id) S.id[p] = v == ~0u ? kNoId : v >> kSlotBits;
        S.rec[p] = v == ~0u ? kNoId : sidx[v & ((1u << kSlotBits) - 1)];
      } else if (with_id) {
        const unsigned long long v = sid[swz64(lp)];
        if (S.id) S.id[p] = v == ~0ull ? kNoId : (uint32_t)(v >> 32);
        S.rec[p] = v == ~0ull ? kNoId : (uint32_t)v;
      }
    }
  }
}

template <int NT, bool ID, bool CC = false>
__global__ void __launch_bounds__(NT, (ID ? 1024 : 1280) / NT) k_raster(Workspace ws, const Surface* __restrict__ surfs,
                                                          uint32_t nsurf, uint32_t tile0) {
  __shared__ RasterSmem<NT, ID> sm;
  if (ws.ctr->overflow) return;
  // surfaces of one size (cube faces) come as grid rows: surface = blockIdx.y
  const uint32_t tile = gridDim.y > 1 ? surfs[blockIdx.y].tile_base + blockIdx.x : tile0 + blockIdx.x;
  raster_tile<NT, ID, CC>(ws, surfs, nsurf, tile, gridDim.y > 1 ? (int)blockIdx.y : -1, sm);
}

// ---- kernel3 ------------------------------------------------------------------
struct ShadeCtx {
  SceneDev sc;
  const ViewParams* V;
  const Surface* S;
};

// (float)d / 2^32 * 350000: the division by 2^32 only shifts the exponent
// (no rounding, no underflow for d >= 1), so it is a multiplication by 2^-32.
constexpr float kInvMulInt = 2.3283064365386963e-10f;
__device__ __forceinline__ float depth_to_dist(uint32_t d) { return ((float)d * kInvMulInt) * kDepthFar; }

// Exact byte -> float without a conversion instruction: 2^23 + b, minus 2^23.
__device__ __forceinline__ float u8f(uint32_t b) { return __uint_as_float(0x4B000000u | b) - 8388608.0f; }

// read_tex_array_all_precalculated (cl2.cl:823-851) in one atlas slot of the
// texture level table: (ox, oy) is the slot origin in its page, tnum * width
// in the reference, an integer below 2048 and so exact in float, which makes
// fma(tnum, width, c) = ox + c.
struct TexSlot {
  float ox, oy, width;
  const uchar4* page;
};
__device__ __forceinline__ TexSlot level_slot(const SceneDev& sc, float4 lv) {
  TexSlot t;
  t.ox = lv.x;
  t.oy = lv.y;
  t.width = lv.z;
  t.page = sc.atlas + (size_t)__float_as_uint(lv.w) * kTexPage * kTexPage;
  return t;
}
__device__ __forceinline__ f4 texel(const TexSlot& ts, int ix, int iy) {
  const uint32_t t = __ldg(reinterpret_cast<const uint32_t*>(ts.page) + ((size_t)iy * kTexPage + ix));
  f4 r; r.x = u8f(t & 0xFF); r.y = u8f((t >> 8) & 0xFF); r.z = u8f((t >> 16) & 0xFF); r.w = u8f(t >> 24);
  return r;
}

// The column (row) of a texel of the bilinear footprint at pos (+ 1 for the
// second): the reference clamps the float coordinate to [0.001, w - 0.001]
// and truncates o + c, o the slot origin.  pos is an integer-valued float
// (floor), so that is o + clamp(pos, 0, w - 1) in integers: 0.001 truncates
// to 0, w - 0.001 to w - 1 (o + w <= 2048 keeps o + w - 0.001 below o + w in
// float), and a NaN coordinate clamps to 0.001, for both texels.
__device__ __forceinline__ int texel_coord(float pos, int plus, int w) {
  if (pos != pos) return 0;
  const int p = min((int)pos, w) + plus;  // saturating conversion; below INT_MAX after the min
  return min(max(p, 0), w - 1);
}

// COLOUR: the result only scales the colour (the texel colour), so the blend
// may contract; the normal map's fetch, which feeds the exact normal, keeps
// the plain products.
template <bool COLOUR>
__device__ f4 bilinear_pre(const TexSlot& ts, float mx, float my) {
  float posx = floorf(mx), posy = floorf(my);
  const int w = (int)ts.width, ox = (int)ts.ox, oy = (int)ts.oy;
  const int x0 = ox + texel_coord(posx, 0, w), x1 = ox + texel_coord(posx, 1, w);
  const int y0 = oy + texel_coord(posy, 0, w), y1 = oy + texel_coord(posy, 1, w);
  f4 c0 = texel(ts, x0, y0);
  f4 c1 = texel(ts, x1, y0);
  f4 c2 = texel(ts, x0, y1);
  f4 c3 = texel(ts, x1, y1);
  float ux = mx - posx, uy = my - posy;
  float bx = 1.0f - ux, by = 1.0f - uy;
  f4 r;
  if (COLOUR) {
    r.x = fma_(fma_(c2.x, bx, c3.x * ux), uy, fma_(c0.x, bx, c1.x * ux) * by);
    r.y = fma_(fma_(c2.y, bx, c3.y * ux), uy, fma_(c0.y, bx, c1.y * ux) * by);
    r.z = fma_(fma_(c2.z, bx, c3.z * ux), uy, fma_(c0.z, bx, c1.z * ux) * by);
    r.w = fma_(fma_(c2.w, bx, c3.w * ux), uy, fma_(c0.w, bx, c1.w * ux) * by);
  } else {
    r.x = fma_(c0.x, bx, c1.x * ux) * by + fma_(c2.x, bx, c3.x * ux) * uy;
    r.y = fma_(c0.y, bx, c1.y * ux) * by + fma_(c2.y, bx, c3.y * ux) * uy;
    r.z = fma_(c0.z, bx, c1.z * ux) * by + fma_(c2.z, bx, c3.z * ux) * uy;
    r.w = fma_(c0.w, bx, c1.w * ux) * by + fma_(c2.w, bx, c3.w * ux) * uy;
  }
  return r;
}

// texture_filter_diff (cl2.cl:1511-1573); COLOUR as for bilinear_pre.  The
// two mip levels come from the texture level table: level mip_lower (the
// texture itself at 0) and level min(mip_lower, 3) + 1, the slots the
// reference's tid_lower / tid_higher name.
template <bool COLOUR>
__device__ f4 texture_filter_diff(const SceneDev& sc, f2 vt, f2 vtdiff, int tid2) {
  const float4* lv = sc.texlv + (size_t)tid2 * kTexLevels;
  const float tsize = __ldg(&lv[0].z);
  f2 vtm = texture_mod(vt);
  float wx = vtdiff.x * tsize, wy = vtdiff.y * tsize;
  float worst = fsqrt(wx * wx + wy * wy);
  float wif = fmax_(log2_approx(worst), 0.0f);  // finite for every input
  float mip_lower = clampf_(floorf(wif), 0.0f, (float)kMipLevels);
  float fmd = wif - mip_lower;
  const int lo = (int)mip_lower, hi = min(lo, kMipLevels - 1) + 1;
  const TexSlot sl = level_slot(sc, __ldg(lv + lo)), sh = level_slot(sc, __ldg(lv + hi));
  f4 c1 = bilinear_pre<COLOUR>(sl, vtm.x * sl.width, vtm.y * sl.width);
  f4 c2 = bilinear_pre<COLOUR>(sh, vtm.x * sh.width, vtm.y * sh.width);
  const float i255 = 1.0f / 255.0f;
  f4 r;
  if (COLOUR) {
    r.x = fma_(c2.x - c1.x, fmd, c1.x) * i255;
    r.y = fma_(c2.y - c1.y, fmd, c1.y) * i255;
    r.z = fma_(c2.z - c1.z, fmd, c1.z) * i255;
    r.w = fma_(c2.w - c1.w, fmd, c1.w) * i255;
  } else {
    r.x = (c1.x + (c2.x - c1.x) * fmd) * i255;
    r.y = (c1.y + (c2.y - c1.y) * fmd) * i255;
    r.z = (c1.z + (c2.z - c1.z) * fmd) * i255;
    r.w = (c1.w + (c2.w - c1.w) * fmd) * i255;
  }
  return r;
}

// depth_to_dist(d) compared with a threshold t: (float)d * 2^-32 is exact and
// a scaling by a power of two commutes with rounding (every value here is a
// normal float), so depth_to_dist(d) = RN((float)d * 350000) * 2^-32, and
// depth_to_dist(d) > t exactly when RN((float)d * 350000) > t * 2^32.
constexpr float kTwo32 = 4294967296.0f;
__device__ __forceinline__ float depth_scaled(uint32_t d) { return (float)d * kDepthFar; }

// How many of the thresholds t0 < t1 < t2 < t3 < t4 lie below d2, i.e.
// (d2 > t0) + ... + (d2 > t4): the thresholds dep + z (z = -2..2, dep <=
// 350000) are strictly increasing in float, so the predicates are monotone and
// three comparisons find the count.
__device__ __forceinline__ int ssao_count(float d2, float t0, float t1, float t2, float t3, float t4) {
  return d2 > t2 ? (d2 > t4 ? 5 : (d2 > t3 ? 4 : 3)) : (d2 > t1 ? 2 : (d2 > t0 ? 1 : 0));
}

// A tap coordinate of generate_ssao: clamped to [1, n - 2] as the reference
// does; for views 1 or 2 pixels wide (high), where that range is empty and the
// reference reads outside its buffer, clamped into the view (0).
__device__ __forceinline__ int ssao_coord(float v, int n) {
  return max((int)clampf_(v, 1.0f, (float)n - 2.0f), 0);
}

// generate_ssao (cl2.cl:2194-2260).  The 25 taps share 5 rows and 5
// columns, whose offsets round(k * world_rad), k = -2..2, are the same five
// values: round is odd-symmetric (half away from zero) and 1 * r, 2 * r and
// -r, -2 * r are exact, so two roundings give all of them.  The depth
// thresholds dep + z are computed once, and the count (at most 125, exact in
// float) is kept in an integer.  Far from the camera (world_rad < 0.25) every
// offset rounds to 0 and all 25 taps read the same pixel; when that holds for
// the whole warp, the pixel is read once and its count taken 25 times.
// seed2 = rand_xorshift(wang_hash(x + W*H*y)), the pixel's first random
// number, which kernel3's normal jitter also draws.
// depth is read with plain (coherent) loads: in the fused pass other blocks
// wrote it during the same launch.
__device__ float generate_ssao(int x, int y, uint32_t seed2, const uint32_t* depth, int W, int H, float fov) {
  float foffset = (float)seed2 * kInvMulInt;
  float dep = depth_to_dist(__ldca(depth + (size_t)y * W + x));
  float rad = kSsaoRad + foffset * 0.5f;  // foffset / 2, exact
  float world_rad = fdiv(rad * fov, dep);
  // the thresholds dep + z, z = -2..2, scaled by 2^32 (depth_scaled)
  const float t0 = (dep + -2.0f) * kTwo32, t1 = (dep + -1.0f) * kTwo32, t2 = dep * kTwo32,
              t3 = (dep + 1.0f) * kTwo32, t4 = (dep + 2.0f) * kTwo32;
  int acc = 0;
  if (__all_sync(__activemask(), world_rad < 0.25f)) {
    const float d2 = depth_scaled(__ldca(depth + (size_t)ssao_coord((float)y, H) * W + ssao_coord((float)x, W)));
    acc = 25 * ssao_count(d2, t0, t1, t2, t3, t4);
  } else {
    const float r1 = roundf(world_rad), r2 = roundf(2.0f * world_rad), r0 = roundf(0.0f * world_rad);
    const float off[5] = {-r2, -r1, r0, r1, r2};
    int wx[5];
#pragma unroll
    for (int k = 0; k < 5; k++) wx[k] = ssao_coord((float)x + off[k], W);
#pragma unroll
    for (int k = 0; k < 5; k++) {
      const uint32_t* row = depth + (size_t)ssao_coord((float)y + off[k], H) * W;
#pragma unroll
      for (int xx = 0; xx < 5; xx++) {
        const float d2 = depth_scaled(__ldca(row + wx[xx]));
        acc += ssao_count(d2, t0, t1, t2, t3, t4);
      }
    }
  }
  // the occlusion scales the colour only: approximate divisions
  const float facc = (float)acc * (1.0f / 125.0f);
  return 1.0f - (1.0f - facc) * (1.0f / kSsaoDiv);
}


// generate_hard_occlusion (cl2.cl:2536-2701), SMOOTH_SHADOWS.  Inlined: as
// a call it cost kernel3 spills around it (1080p kernel3 0.236 -> 0.233 ms
// inlined)
__device__ __forceinline__ float hard_occlusion(const SceneDev& sc, f3 lpos, f3 normal, f3 ptl, const uint32_t* buf,
                                int face, f3 gpos, int shnum) {
  ptl = fast_normalize3(ptl);
  f3 c = mk3(sc.face_cos[face][0], sc.face_cos[face][1], sc.face_cos[face][2]);
  f3 s = mk3(sc.face_sin[face][0], sc.face_sin[face][1], sc.face_sin[face][2]);
  f3 local = rot_cs(gpos, lpos, c, s);
  f3 post = depth_project1(local, (float)kLightBufferDim, (float)kLightBufferDim, kLFov);
  float dpth = post.z;
  const uint32_t* map = buf + (size_t)(face + shnum * 6) * kLightBufferDim * kLightBufferDim;
  float px = clampf_(post.x, 3.0f, kLightBufferDim - 4.0f);
  float py = clampf_(post.y, 3.0f, kLightBufferDim - 4.0f);
  int ix = f2i_sat(px), iy = f2i_sat(py);
  float acos_res = rational_acos(clampf_(dot3(normal, ptl), 0.05f, 0.95f));
  float bias = clampf_(kShadowBias * gbr_tanf(acos_res), 0.1f * kShadowBias, kShadowBias);
  uint32_t cond = 0;  // bit (yy+1)*4 + (xx+1)
#pragma unroll
  for (int yy = -1; yy <= 2; yy++)
#pragma unroll
    for (int xx = -1; xx <= 2; xx++) {
      float ldp = depth_to_dist(__ldg(map + (iy + yy) * kLightBufferDim + ix + xx));
      if (dpth > ldp + bias) cond |= 1u << ((yy + 1) * 4 + xx + 1);
    }
  // The 3x3 bilinear blend of the 4x4 tests: every tap has the same
  // fractional offsets (ux, uy), so the sum of the nine bilinear_interpolate
  // calls is separable, with column weights (1 - ux, 1, 1, ux) and row
  // weights (1 - uy, 1, 1, uy).  The occlusion scales the colour only.
  const float mx = (px + 0.5f) - 0.5f, my = (py + 0.5f) - 0.5f;
  const float ux = mx - floorf(mx), uy = my - floorf(my);
  const float by = 1.0f - uy;
  // per column group (left, middle two, right): tests of the top row, the
  // middle two rows and the bottom row
  auto rows = [&](uint32_t top, uint32_t mid, uint32_t bot) {
    return fma_(uy, (float)__popc(cond & bot), fma_(by, (float)__popc(cond & top), (float)__popc(cond & mid)));
  };
  const float sl = rows(0x0001u, 0x0110u, 0x1000u);
  const float sm = rows(0x0006u, 0x0660u, 0x6000u);
  const float sr = rows(0x0008u, 0x0880u, 0x8000u);
  const float shadow = fma_(ux, sr, fma_(1.0f - ux, sl, sm));
  return shadow * (1.0f / 9.0f);
}

// Vertex colour channels (colour path: multiplication by 1/255).
__device__ __forceinline__ f4 vertex_col(uint32_t c) {
  const float k = 1.0f / 255.0f;
  f4 r;
  r.x = u8f(c >> 24) * k;
  r.y = u8f((c >> 16) & 0xFF) * k;
  r.z = u8f((c >> 8) & 0xFF) * k;
  r.w = u8f(c & 0xFF) * k;
  return r;
}


// Colour-only arithmetic of the light loop: every use below feeds the colour
// continuously (no comparison, rounding or index depends on it), so the
// approximate division is covered by the 1/255 colour tolerance.
__device__ __forceinline__ float crcp(float b) { return __fdividef(1.0f, b); }
__device__ __forceinline__ f3 cnormalize(f3 a) {
  float r = rsqrtf(dot3(a, a));
  return mk3(a.x * r, a.y * r, a.z * r);
}
// Colour-path dot product with contraction.
__device__ __forceinline__ float cdot3(f3 a, f3 b) { return fma_(a.z, b.z, fma_(a.y, b.y, a.x * b.x)); }
// rational_acos (cl2.cl:1919-1936) in Horner form: x (a + b x^2) / (1 + c x^2 + d x^4) + pi/2.
__device__ __forceinline__ float c_rational_acos(float x) {
  const float a = -0.939115566365855f, b = 0.9217841528914573f, c = -1.2845906244690837f,
              d = 0.295624144969963174f;
  const float x2 = x * x;
  return fma_(x * fma_(b, x2, a), crcp(fma_(x2, fma_(d, x2, c), 1.0f)), kPi / 2.0f);
}


// Colour-only square root (approximate; exact IEEE result for 0, negative,
// infinite and NaN inputs).
__device__ __forceinline__ float csqrt(float x) {
  return (x > 0.0f && x < 3.0e38f) ? x * rsqrtf(x) : fsqrt(x);
}
// gamma_inv (cl2.cl:5778-5782) on the colour path.
__device__ __forceinline__ float c_gamma_inv(float c) {
  float s1 = csqrt(c);
  float s2 = csqrt(s1);
  float s3 = csqrt(s2);
  return fma_(-0.368262736f, s3, fma_(0.783140355f, s2, 0.585122381f * s1));
}
// gamma_fwd (cl2.cl:5763-5770) in Horner form, for colours
__device__ __forceinline__ float c_gamma_fwd(float c) {
  return c * fma_(fma_(0.305306011f, c, 0.682171111f), c, 0.012522878f);
}

// kernel3's attenuation cutoff: a light adds (illum - 0.1) / 0.9 where that is positive
constexpr float kLightCutoff = 0.1f;

// A light as the shade loop reads it, staged once per CTA in shared memory
// as three float4: (pos, cut2), (colour, brightness, divided by 1 - cutoff
// for lights without shadows), (radius, 1 / radius approximated, diffuse,
// shadow | is_static << 1).  The colour is already in
// linear space when the view renders linearly (the same gamma_fwd every pixel
// would apply).  cut2 is a conservative squared distance beyond which a light
// without shadows stays under kernel3's attenuation cutoff, so the pixel
// skips it without computing the attenuation: brightness / (d / radius + 1)^2
// <= 0.1 holds beyond d = radius * (sqrt(10 * brightness) - 1), and the
// margins below cover the approximate colour-path arithmetic of that test
// (relative errors of a few 1e-7).  -1: always under the cutoff; +inf: no
// early test (shadow lights, whose cutoff decides the cubemap later shadow
// lights read, and degenerate radii).
constexpr int kLightQuads = 3;
__device__ __forceinline__ void stage_light(const gbr_light* L, bool linear, float4* dst) {
  f3 c = mk3(L->col[0], L->col[1], L->col[2]);
  if (linear) c = mk3(gamma_fwd(c.x), gamma_fwd(c.y), gamma_fwd(c.z));
  const float radius = L->radius, brightness = L->brightness;
  const float b10 = 10.0f * brightness;
  float cut2 = __int_as_float(0x7F800000);
  if (!L->shadow && radius > 0.0f && b10 == b10) {
    if (b10 <= 1.0f) {
      cut2 = -1.0f;
    } else {
      const float rs = radius * ((sqrtf(b10) * 1.00001f - 1.0f) * 1.00001f);
      cut2 = (rs * rs) * 1.00001f;
    }
  }
  // lights without shadows fold kernel3's cutoff into the brightness:
  // (b / tt^2 - 0.1) / 0.9 = (b / 0.9) / tt^2 - 0.1 / 0.9 (colour only)
  const float bw = L->shadow ? brightness : brightness * (1.0f / (1.0f - kLightCutoff));
  dst[0] = make_float4(L->pos[0], L->pos[1], L->pos[2], cut2);
  dst[1] = make_float4(c.x, c.y, c.z, bw);
  dst[2] = make_float4(radius, crcp(radius), L->diffuse,
                       __uint_as_float((L->shadow ? 1u : 0u) | (L->is_static ? 2u : 0u)));
}

// kernel3 (cl2.cl:5792-6408) for one pixel of a view.
// ENABLE_NORMAL_MAPPING (cl2.cl:5987-6027): the tangent-space normal from the
// object's normal map, in object space through the triangle's tangent frame,
// then rotated into world space.  It feeds the shadow bias, so it keeps the
// IEEE contract (normalize as fast_normalize).
// dp1 = p2 - p1 and dp2 = p3 - p1 are the barycentric frame's edges.
__device__ __forceinline__ f3 normal_map(const SceneDev& sc, f2 vt, f2 vtdiff, uint32_t rid, f3 dp1, f3 dp2,
                                      f2 vt1, f2 vt2, f2 vt3, f3 model_normal, f4 qn) {
  const f4 t4 = texture_filter_diff<false>(sc, vt, vtdiff, (int)rid);
  f3 tn = mk3(2.0f * t4.x - 1.0f, 2.0f * t4.y - 1.0f, 2.0f * t4.z - 1.0f);
  tn = fast_normalize3(tn);
  const f2 duv1 = mk2(vt2.x - vt1.x, vt2.y - vt1.y), duv2 = mk2(vt3.x - vt1.x, vt3.y - vt1.y);
  const float r = fdiv(1.0f, duv1.x * duv2.y - duv1.y * duv2.x);
  f3 tangent = mk3((dp1.x * duv2.y - dp2.x * duv1.y) * r, (dp1.y * duv2.y - dp2.y * duv1.y) * r,
                   (dp1.z * duv2.y - dp2.z * duv1.y) * r);
  f3 bitangent = mk3((dp2.x * duv1.x - dp1.x * duv2.x) * r, (dp2.y * duv1.x - dp1.y * duv2.x) * r,
                     (dp2.z * duv1.x - dp1.z * duv2.x) * r);
  tangent = fast_normalize3(tangent);
  bitangent = fast_normalize3(bitangent);
  tangent = fast_normalize3(sub3(tangent, mul3s(model_normal, dot3(model_normal, tangent))));
  if (dot3(cross3(model_normal, tangent), bitangent) < 0.0f) tangent = mul3s(tangent, -1.0f);
  const f3 ms = mk3((tangent.x * tn.x + bitangent.x * tn.y) + model_normal.x * tn.z,
                    (tangent.y * tn.x + bitangent.y * tn.y) + model_normal.y * tn.z,
                    (tangent.z * tn.x + bitangent.z * tn.y) + model_normal.z * tn.z);
  return rot_quat_n(ms, qn);
}

// generate_outline (cl2.cl:2315-2362): the largest depth step to the four
// neighbours, over 100, at most 1.
__device__ __forceinline__ float generate_outline(int x, int y, const uint32_t* depth, int W, int H) {
  const float d0 = depth_to_dist(__ldca(depth + (size_t)y * W + x));
  float furthest = d0;
  for (int xx = -1; xx <= 1; xx++) {
    const int px = x + xx;
    if (px < 0 || px >= W) continue;
    const float nd = depth_to_dist(__ldca(depth + (size_t)y * W + px));
    if (nd > furthest) furthest = nd;
  }
  for (int yy = -1; yy <= 1; yy++) {
    const int py = y + yy;
    if (py < 0 || py >= H) continue;
    const uint32_t d = __ldca(depth + (size_t)py * W + x);
    const float nd = depth_to_dist(d);
    if (fabsf(nd - d0) > fabsf(furthest - d0) && nd > kDepthCutoff && d != 0) furthest = nd;
  }
  return fmin_(fdiv(fabsf(furthest - d0), 100.0f), 1.0f);
}

// One RGBA8 texel of the blend source as read_imagef returns it (c / 255).
__device__ __forceinline__ f4 blend_texel(const uint8_t* __restrict__ rgba, size_t p) {
  const uchar4 t = reinterpret_cast<const uchar4*>(rgba)[p];
  f4 o;
  o.x = u8_over_255(t.x); o.y = u8_over_255(t.y);  // fdiv(t, 255.0f)
  o.z = u8_over_255(t.z); o.w = u8_over_255(t.w);
  return o;
}

// kernel3's output for a pixel with nothing to shade (depth d): the clear
// colour and zero normals.  FEAT: kernel3's optional switches (view flags)
// compiled in.
template <bool FEAT>
__device__ __forceinline__ void shade_clear(const ViewParams& V, size_t p, uint32_t d) {
  uint32_t* out = reinterpret_cast<uint32_t*>(V.rgba);
  if (out) {
    f4 c;
    c.x = V.clear[0]; c.y = V.clear[1]; c.z = V.clear[2]; c.w = V.clear[3];
    // CAN_INTEGRATED_BLEND (cl2.cl:5839-5851): the other context's colour
    // over the clear colour where it has depth; its .xyzz swizzle gives
    // alpha = blue
    if (FEAT && V.blend_depth && V.blend_depth[p] < d) {
      const f4 o = blend_texel(V.blend_rgba, p);
      c.x = fma_(o.x, o.w, c.x * (1.0f - o.w));
      c.y = fma_(o.y, o.w, c.y * (1.0f - o.w));
      c.z = fma_(o.z, o.w, c.z * (1.0f - o.w));
      c.w = c.z;
    }
    out[p] = pack_rgba(c.x, c.y, c.z, c.w);
  }
  if (V.normals) reinterpret_cast<uint32_t*>(V.normals)[p] = 0;
}

// kernel3 for a covered pixel: depth d, record r (< the pass's record count).
// colx[i] = ((float)(x0 + i) - W/2) / fov and rowy[j] likewise for the tile's
// 17 columns and rows: the per-column / per-row divisions of get_vtdiff.
template <bool FEAT>
__device__ void shade_covered(const SceneDev& sc, const ViewParams& V, const Surface& S,
                              const ShadeRec* __restrict__ srec, const float4* __restrict__ lights, int x, int y,
                              uint32_t d, uint32_t r, const float* __restrict__ colx,
                              const float* __restrict__ rowy) {
  const int W = S.width, H = S.height;
  const size_t p = (size_t)y * W + x;
  uint32_t* out = reinterpret_cast<uint32_t*>(V.rgba);
  const float fov = V.fov;
  const f3 cpos = mk3(V.cpos[0], V.cpos[1], V.cpos[2]);
  const f3 cc = mk3(V.ccos[0], V.ccos[1], V.ccos[2]);
  const f3 cs = mk3(V.csin[0], V.csin[1], V.csin[2]);
  // the triangle's shade constants (prep_shade) and its object's terms
  const ShadeRec* R = srec + r;
  BaryFrame bf;
  {
    const float4 fa = __ldg(&R->a), f0 = __ldg(&R->e0), f1 = __ldg(&R->e1), fp = __ldg(&R->plane);
    bf.a = mk3(fa.x, fa.y, fa.z);
    bf.v0 = mk3(f0.x, f0.y, f0.z);
    bf.v1 = mk3(f1.x, f1.y, f1.z);
    bf.d00 = fa.w; bf.d01 = f0.w; bf.d11 = f1.w; bf.denom = fp.w;
  }
  const float4 fn1 = __ldg(&R->n1), fn2 = __ldg(&R->n2), fn3 = __ldg(&R->n3), ft = __ldg(&R->t);
  const f2 vt1 = mk2(fn1.w, fn2.w), vt2 = mk2(fn3.w, ft.x), vt3 = mk2(ft.y, ft.z);
  const uint32_t obits = __float_as_uint(ft.w);
  const uint32_t o_id = obits & 0x7FFFFFFFu;
  const float4* OQ = sc.objq + (size_t)o_id * kObjQuads;
  const float4 oq0 = __ldg(OQ), oq1 = __ldg(OQ + 1), oq2 = __ldg(OQ + 2), oq3 = __ldg(OQ + 3);
  f4 qn, qi;  // rot_quat's and back_rot_quat's normalised quaternions
  qn.x = oq0.x; qn.y = oq0.y; qn.z = oq0.z; qn.w = oq0.w;
  qi.x = oq1.x; qi.y = oq1.y; qi.z = oq1.z; qi.w = oq1.w;
  const f3 wpos = mk3(oq2.x, oq2.y, oq2.z);

  const float ldepth = depth_to_dist(d);
  const float fx = (float)x, fy = (float)y;
  f3 local = mk3(fdiv((fx - (float)W / 2.0f) * ldepth, fov), fdiv((fy - (float)H / 2.0f) * ldepth, fov),
                 ldepth);
  const f3 zero = mk3(0, 0, 0);
  const f3 gpos = add3(back_rot_cs(local, zero, cc, cs), cpos);
  f3 olocal = rot_quat_n(sub3(gpos, wpos), qi);
  float l1, l2, l3;
  bary_exact(bf, olocal, &l1, &l2, &l3);
  f2 vt = mk2(fma_(vt1.x, l1, fma_(vt2.x, l2, vt3.x * l3)), fma_(vt1.y, l1, fma_(vt2.y, l2, vt3.y * l3)));
  f3 normal = mk3(fma_(fn1.x, l1, fma_(fn2.x, l2, fn3.x * l3)), fma_(fn1.y, l1, fma_(fn2.y, l2, fn3.y * l3)),
                  fma_(fn1.z, l1, fma_(fn2.z, l2, fn3.z * l3)));
  const f3 model_normal = normal;
  normal = rot_quat_n(normal, qn);

  f4 col;
  const float4 fcol = __ldg(&R->col);
  const uint32_t vc0 = __float_as_uint(fcol.x);
  // normal map of the object (ENABLE_NORMAL_MAPPING), 0xFFFFFFFF if none
  const uint32_t rid = (FEAT && (V.flags & GBR_VIEW_NORMAL_MAPPING)) ? __ldg(&sc.descs[o_id].rid) : 0xFFFFFFFFu;
  f2 vtdiff = mk2(0.0f, 0.0f);
  if (vc0 == 0 || rid != 0xFFFFFFFFu) {
    // get_vtdiff (cl2.cl:5691-5760), its 1/z plane from the shade constants.
    // The plane extrapolated to the neighbouring pixels is ill-conditioned
    // for triangles seen edge-on (it can cross zero), so this stays in IEEE
    // arithmetic: rounding differences there would pick other mip levels.
    const float4 fp = __ldg(&R->plane);
    float dmx = fma_(fp.x, fx + 1.0f, fma_(fp.y, fy, fp.z));
    float dmy = fma_(fp.x, fx, fma_(fp.y, fy + 1.0f, fp.z));
    const int lx = x & (kTile - 1), ly = y & (kTile - 1);
    f3 lmx = mk3(colx[lx + 1], rowy[ly], 1.0f);  // fdiv((fx + 1) - hw, fov), fdiv(fy - hh, fov)
    f3 lmy = mk3(colx[lx], rowy[ly + 1], 1.0f);  // fdiv(fx - hw, fov), fdiv((fy + 1) - hh, fov)
    lmx = mk3(fdiv(lmx.x, dmx), fdiv(lmx.y, dmx), fdiv(lmx.z, dmx));
    lmy = mk3(fdiv(lmy.x, dmy), fdiv(lmy.y, dmy), fdiv(lmy.z, dmy));
    f3 gmx = rot_quat_n(sub3(add3(back_rot_cs(lmx, zero, cc, cs), cpos), wpos), qi);
    f3 gmy = rot_quat_n(sub3(add3(back_rot_cs(lmy, zero, cc, cs), cpos), wpos), qi);
    float lx1, lx2, lx3, ly1, ly2, ly3;
    bary_exact(bf, gmx, &lx1, &lx2, &lx3);
    bary_exact(bf, gmy, &ly1, &ly2, &ly3);
    f2 vtx = mk2(fma_(vt1.x, lx1, fma_(vt2.x, lx2, vt3.x * lx3)), fma_(vt1.y, lx1, fma_(vt2.y, lx2, vt3.y * lx3)));
    f2 vty = mk2(fma_(vt1.x, ly1, fma_(vt2.x, ly2, vt3.x * ly3)), fma_(vt1.y, ly1, fma_(vt2.y, ly2, vt3.y * ly3)));
    const float mip_bias = 1.0f / kMipBias;
    vtdiff = mk2((fabsf(vtx.x - vt.x) + fabsf(vty.x - vt.x)) * mip_bias,
                 (fabsf(vtx.y - vt.y) + fabsf(vty.y - vt.y)) * mip_bias);
  }
  // (the reference replaces the normal after its colour and jitter seeds,
  // neither of which reads it)
  if (FEAT && rid != 0xFFFFFFFFu)
    normal = normal_map(sc, vt, vtdiff, rid, bf.v0, bf.v1, vt1, vt2, vt3, model_normal, qn);
  if (vc0 != 0) {
    f4 c0 = vertex_col(vc0), c1 = vertex_col(__float_as_uint(fcol.y)), c2 = vertex_col(__float_as_uint(fcol.z));
    col.x = fma_(c0.x, l1, fma_(c1.x, l2, c2.x * l3));
    col.y = fma_(c0.y, l1, fma_(c1.y, l2, c2.y * l3));
    col.z = fma_(c0.z, l1, fma_(c1.z, l2, c2.z * l3));
    col.w = fma_(c0.w, l1, fma_(c1.w, l2, c2.w * l3));
  } else {
    col = texture_filter_diff<true>(sc, vt, vtdiff, (int)__float_as_uint(oq3.w));
  }
  if (V.use_linear) {
    col.x = c_gamma_fwd(col.x);
    col.y = c_gamma_fwd(col.y);
    col.z = c_gamma_fwd(col.z);
  }
  uint32_t seed2 = rand_xorshift(wang_hash((uint32_t)x + (uint32_t)y * (uint32_t)W * (uint32_t)H));
  uint32_t seed3 = rand_xorshift(seed2);
  uint32_t seed4 = rand_xorshift(seed3);
  f3 rseed = mk3(((float)seed2 * kInvMulInt - 0.5f) * 2.0f, ((float)seed3 * kInvMulInt - 0.5f) * 2.0f,
                 ((float)seed4 * kInvMulInt - 0.5f) * 2.0f);
  const f3 l2p = cnormalize(sub3(cpos, gpos));
  const int ff = (int)__float_as_uint(oq3.z);
  const bool two = (ff & kFlagTwoSided) > 0;
  const bool recv_dyn = !((ff & kFlagNoDynShadows) > 0);
  if ((obits >> 31) && two) normal = neg3(normal);  // back-facing (cl2.cl:491-494)
  const float ssao = generate_ssao(x, y, seed2, S.depth, W, H, fov);
  normal = fast_normalize3(normal);
  const f3 lnormal = cnormalize(add3(normal, mk3(rseed.x * 0.01f, rseed.y * 0.01f, rseed.z * 0.01f)));
  const float ambient = V.use_linear ? gamma_fwd(kAmbient) : kAmbient;
  const float g_diffuse = oq2.w, g_spec_mult = oq3.x;
  const float rough = oq3.y;  // clamp(1 - specular, 0.001, 10)
  // per-pixel factors of the light loop (colour only)
  const float ndv_raw = cdot3(normal, l2p);
  const float ndv = fmax_(0.0f, ndv_raw);
  const float r_pndv = crcp(kPi * ndv);  // spec / (pi ndv)
  const float nr2 = -crcp(rough * rough);  // Gaussian exponent -alpha^2 / rough^2
  const float spec_k = 0.4f * g_spec_mult;
  const float amb1 = 1.0f - ambient;
  f3 dsum = mk3(0, 0, 0), ssum = mk3(0, 0, 0);
  int shnum = 0, static_num = 0;
  for (uint32_t i = 0; i < sc.nlights; i++) {
    const float4 LA = lights[kLightQuads * i];
    const f3 lpos = mk3(LA.x, LA.y, LA.z);
    f3 ptl = sub3(lpos, gpos);
    // The distance only feeds the colour, except through the cutoff below,
    // which for a shadow light also decides which cubemap later shadow lights
    // read (shnum): IEEE arithmetic for shadow lights (a warp-uniform branch),
    // approximate otherwise, after the conservative early test (whose margins
    // cover the contracted dot product).
    const float d2 = cdot3(ptl, ptl);
    if (d2 > LA.w) continue;
    const float4 LB = lights[kLightQuads * i + 1], LC = lights[kLightQuads * i + 2];
    const uint32_t lflags = __float_as_uint(LC.w);
    const f3 lcol = mk3(LB.x, LB.y, LB.z);
    const float rinv = rsqrtf(d2);
    if (lflags & 1u) {  // a shadow light: its distance in IEEE arithmetic
      const float d2s = dot3(ptl, ptl);
      float occlusion = 1.0f;
      if (lflags & 2u) {  // is_static
        int face = ret_cubeface(gpos, lpos);
        occlusion = 1.0f - hard_occlusion(sc, lpos, normal, ptl, sc.shadow_static, face, gpos, static_num);
        static_num++;
      }
      const float tt = fdiv(fsqrt(d2s), LC.x) + 1.0f;
      float illum = fdiv(LB.w, tt * tt);
      illum -= kLightCutoff;
      illum *= 1.0f / (1.0f - kLightCutoff);
      if (illum <= 0) continue;
      if (recv_dyn) {
        int face = ret_cubeface(gpos, lpos);
        float dyn = 1.0f - hard_occlusion(sc, lpos, normal, ptl, sc.shadow_dyn, face, gpos, shnum);
        occlusion = fmin_(occlusion, dyn);
        shnum++;
      }
      ptl = mul3s(ptl, rinv);  // cnormalize(ptl), the dot contracted (colour only)
      // Lambert + ambient
      const float light = fmax_(cdot3(ptl, lnormal) * occlusion, 0.0f);
      const float dscale = fma_(amb1, light, ambient) * ((LC.z * g_diffuse) * illum);
      dsum = mk3(fma_(lcol.x, dscale, dsum.x), fma_(lcol.y, dscale, dsum.y), fma_(lcol.z, dscale, dsum.z));
      // Cook-Torrance: F0 0.4, Gaussian microfacet 0.8346, geometric term
      const f3 Hv = cnormalize(add3(l2p, ptl));
      const float ndh = fmax_(0.0f, cdot3(normal, Hv));
      const float vdh = fmax_(0.0f, cdot3(l2p, Hv));
      const float ndl = fmax_(0.0f, cdot3(normal, ptl));
      const float omv = 1.0f - vdh, omv2 = omv * omv;
      const float fresnel = fma_(0.6f, (omv2 * omv2) * omv, 0.4f);
      const float alpha = c_rational_acos(ndh);
      const float microfacet = 0.8346f * __expf((alpha * alpha) * nr2);
      const float sv = (2.0f * ndh) * crcp(vdh);
      const float geometric = min3f(1.0f, sv * ndv, sv * ndl);
      const float spec = ((fresnel * microfacet) * geometric) * r_pndv;
      const float sscale = spec * (spec_k * illum);
      ssum = mk3(fmax_(fma_(lcol.x, sscale, ssum.x), 0.0f) * occlusion,
                 fmax_(fma_(lcol.y, sscale, ssum.y), 0.0f) * occlusion,
                 fmax_(fma_(lcol.z, sscale, ssum.z), 0.0f) * occlusion);
      continue;
    }
    // a light without shadows: its occlusion is 1
    // the approximate square root; 0, +inf and NaN are their own square roots
    const float distance = (d2 > 0.0f && d2 <= 3.4028235e38f) ? d2 * rinv : d2;
    const float tt = fma_(distance, LC.y, 1.0f);
    const float illum = fma_(LB.w, crcp(tt * tt), -kLightCutoff / (1.0f - kLightCutoff));
    if (illum <= 0) continue;
    ptl = mul3s(ptl, rinv);
    const float light = fmax_(cdot3(ptl, lnormal), 0.0f);
    const float dscale = fma_(amb1, light, ambient) * ((LC.z * g_diffuse) * illum);
    dsum = mk3(fma_(lcol.x, dscale, dsum.x), fma_(lcol.y, dscale, dsum.y), fma_(lcol.z, dscale, dsum.z));
    // the half vector H = (v + l) / |v + l| of the unit vectors v (l2p) and l
    // (ptl) through dot products: |v + l|^2 = 2 + 2 v.l, n.H = (n.v + n.l) /
    // |v + l|, v.H = (1 + v.l) / |v + l|
    const float nl = cdot3(normal, ptl), vl = cdot3(l2p, ptl);
    const float rh = rsqrtf(fma_(2.0f, vl, 2.0f));
    const float vdh = fmax_(0.0f, (1.0f + vl) * rh);
    const float ndh = fmax_(0.0f, (ndv_raw + nl) * rh);
    const float ndl = fmax_(0.0f, nl);
    const float omv = 1.0f - vdh, omv2 = omv * omv;
    const float fresnel = fma_(0.6f, (omv2 * omv2) * omv, 0.4f);
    const float alpha = c_rational_acos(ndh);
    const float microfacet = 0.8346f * __expf((alpha * alpha) * nr2);
    const float sv = (2.0f * ndh) * crcp(vdh);
    const float geometric = min3f(1.0f, sv * ndv, sv * ndl);
    const float spec = ((fresnel * microfacet) * geometric) * r_pndv;
    const float sscale = spec * (spec_k * illum);
    ssum = mk3(fmax_(fma_(lcol.x, sscale, ssum.x), 0.0f), fmax_(fma_(lcol.y, sscale, ssum.y), 0.0f),
               fmax_(fma_(lcol.z, sscale, ssum.z), 0.0f));
  }
  ssum = mul3s(ssum, ssao);
  dsum = mul3s(dsum, ssao);
  const float rsc = 0.7f;
  f3 colclamp = add3(add3(mk3(col.x, col.y, col.z), zero), mul3s(ssum, rsc));
  f3 sp2 = mul3s(ssum, 1.0f - rsc);
  f3 fin = mk3(fma_(colclamp.x, dsum.x, sp2.x), fma_(colclamp.y, dsum.y, sp2.y), fma_(colclamp.z, dsum.z, sp2.z));
  // CAN_INTEGRATED_BLEND (cl2.cl:6339-6351): alpha_blend of the other
  // context's colour where it is nearer, before the output gamma
  if (FEAT && V.blend_depth && V.blend_depth[p] < d) {
    const f4 o = blend_texel(V.blend_rgba, p);
    fin = mk3(fma_(o.x, o.w, fin.x * (1.0f - o.w)), fma_(o.y, o.w, fin.y * (1.0f - o.w)),
              fma_(o.z, o.w, fin.z * (1.0f - o.w)));
  }
  if (V.use_linear) fin = mk3(c_gamma_inv(fin.x), c_gamma_inv(fin.y), c_gamma_inv(fin.z));
  if (FEAT && (V.flags & GBR_VIEW_OUTLINE) && (ff & kFlagOutline) > 0) {
    const float o = generate_outline(x, y, S.depth, W, H);
    fin = mk3(fin.x + o, fin.y + o, fin.z + o);
  }
  if (out) out[p] = pack_rgba(fin.x, fin.y, fin.z, col.w);
  if (V.normals) {
    // encode_normal (cl2.cl:5618-5628)
    float nx = normal.x, ny = normal.y, nz = normal.z;
    if (nx * nx + ny * ny < 0.0001f) nx = 0.01f;
    float l = fsqrt(nx * nx + ny * ny);
    float sq = fsqrt(fmax_(nz * 0.5f + 0.5f, 0.0f));
    // (v / 2 = v * 0.5 exactly: both are the correctly rounded v / 2)
    float ex = ((fdiv(nx, l) * sq + 1.0f) * 0.5f) * 65536.0f - 1.0f;
    float ey = ((fdiv(ny, l) * sq + 1.0f) * 0.5f) * 65536.0f - 1.0f;
    uint32_t ux = min(f2u_sat(ex), 65535u), uy = min(f2u_sat(ey), 65535u);
    reinterpret_cast<uint32_t*>(V.normals)[p] = ux | (uy << 16);
  }
}

// kernel3 for one pixel.  nrec: the records this pass wrote; the raster
// stores only indices below it in the record map, and any other value is
// treated as an empty pixel, so no index read from the map can leave the
// record arrays.
template <bool FEAT>
__device__ __forceinline__ void shade_pixel(const SceneDev& sc, const ViewParams& V, const Surface& S,
                                            const ShadeRec* __restrict__ srec, uint32_t nrec,
                                            const float4* __restrict__ lights, int x, int y,
                                            const float* __restrict__ colx, const float* __restrict__ rowy) {
  const size_t p = (size_t)y * S.width + x;
  const uint32_t d = S.depth[p];
  const uint32_t r = S.rec[p];
  if (d == kDepthClear || r >= nrec)
    shade_clear<FEAT>(V, p, d);
  else
    shade_covered<FEAT>(sc, V, S, srec, lights, x, y, d, r, colx, rowy);
}

// Shared memory of one tile's shading.
struct ShadeSmem {
  float4 lights[kMaxLights * kLightQuads];
  float colx[kTile + 1], rowy[kTile + 1];
};

// kernel3 over one 16x16 tile of view surface `sid` (NT threads, 256 / NT
// pixels each).  Every thread of the block calls it; the caller synchronises
// before reusing the shared memory.
template <bool FEAT, int NT>
__device__ __forceinline__ void shade_tile(const SceneDev& sc, const ViewParams* __restrict__ views,
                                           const Surface* __restrict__ surfs, const ShadeRec* __restrict__ srec,
                                           uint32_t nrec, uint32_t tile, uint32_t sid, ShadeSmem& sm) {
  const Surface& S = surfs[sid];
  const ViewParams& V = views[sid];
  const uint32_t lt = tile - S.tile_base;
  const int x0 = (lt % S.tiles_x) * kTile, y0 = (lt / S.tiles_x) * kTile;
  const bool linear = V.use_linear != 0;
  for (uint32_t i = threadIdx.x; i < sc.nlights; i += NT) stage_light(sc.lights + i, linear, sm.lights + kLightQuads * i);
  if (threadIdx.x < 2 * (kTile + 1)) {
    const int i = threadIdx.x % (kTile + 1);
    if (threadIdx.x <= kTile)
      sm.colx[i] = fdiv((float)(x0 + i) - (float)S.width / 2.0f, V.fov);
    else
      sm.rowy[i] = fdiv((float)(y0 + i) - (float)S.height / 2.0f, V.fov);
  }
  __syncthreads();
  if (NT == kTilePixels) {  // one pixel per thread
    const int x = x0 + (threadIdx.x & (kTile - 1)), y = y0 + threadIdx.x / kTile;
    if (x < S.width && y < S.height) shade_pixel<FEAT>(sc, V, S, srec, nrec, sm.lights, x, y, sm.colx, sm.rowy);
    return;
  }
#pragma unroll 1
  for (int lp = threadIdx.x; lp < kTilePixels; lp += NT) {
    const int x = x0 + (lp & (kTile - 1)), y = y0 + lp / kTile;
    if (x < S.width && y < S.height) shade_pixel<FEAT>(sc, V, S, srec, nrec, sm.lights, x, y, sm.colx, sm.rowy);
  }
}

// A pass whose setup or binning overflowed its scratch leaves the depth and
// record map unwritten (the raster returns at once); shading returns too, and
// the host re-runs the pass with grown scratch.
// kernel3 over the tiles of a pass, one 256-thread CTA per 16x16 tile.
// tile_empty (or null): tiles whose output the raster wrote, which return at
// once; tiles (null for one view): each tile's surface (Workspace).  Each
// thread reads its pixel; empty pixels get the clear colour, covered ones are
// compacted in pixel order into the first threads, which shade them.
template <bool FEAT>
__global__ void __launch_bounds__(256, 4) k_shade(SceneDev sc, const ViewParams* __restrict__ views,
                                               const Surface* __restrict__ surfs, uint32_t nviews,
                                               const ShadeRec* __restrict__ srec, const Counters* __restrict__ ctr,
                                               uint32_t rec_cap, uint32_t tile0,
                                               const uint8_t* __restrict__ tile_empty,
                                               const uint2* __restrict__ tiles) {
  constexpr int NW = kTilePixels / 32;
  __shared__ ShadeSmem sm;
  __shared__ uint32_t s_warp[NW];
  __shared__ uint32_t s_px[kTilePixels], s_d[kTilePixels], s_r[kTilePixels];
  if (ctr->overflow) return;
  const uint32_t nrec = min(ctr->nrec, rec_cap);
  const uint32_t tile = tile0 + blockIdx.x;
  // every thread reads the tile's flag and surface (the same words): the
  // return is block-uniform and needs no barrier
  if (tile_empty && tile_empty[tile]) return;
  const uint32_t sid = tiles ? tiles[tile].x : 0u;  // null: one view
  const Surface& S = surfs[sid];
  const ViewParams& V = views[sid];
  const uint32_t lt = tile - S.tile_base;
  const int x0 = (lt % S.tiles_x) * kTile, y0 = (lt / S.tiles_x) * kTile;
  // the thread's own pixel: empty pixels are written at once; covered ones
  // are compacted (in pixel order) so that whole warps shade them
  const int lp = threadIdx.x, lane = lp & 31, warp = lp >> 5;
  const int x = x0 + (lp & (kTile - 1)), y = y0 + lp / kTile;
  const bool inside = x < S.width && y < S.height;
  const size_t p = (size_t)y * S.width + x;
  uint32_t d = kDepthClear, r = kNoId;
  if (inside) {
    d = S.depth[p];
    r = S.rec[p];
  }
  const bool cov = inside && d != kDepthClear && r < nrec;
  const unsigned m = __ballot_sync(0xFFFFFFFFu, cov);
  if (lane == 0) s_warp[warp] = __popc(m);
  if (inside && !cov) shade_clear<FEAT>(V, p, d);
  const bool linear = V.use_linear != 0;
  for (uint32_t i = threadIdx.x; i < sc.nlights; i += kTilePixels)
    stage_light(sc.lights + i, linear, sm.lights + kLightQuads * i);
  if (threadIdx.x < 2 * (kTile + 1)) {
    const int i = threadIdx.x % (kTile + 1);
    if (threadIdx.x <= kTile)
      sm.colx[i] = fdiv((float)(x0 + i) - (float)S.width / 2.0f, V.fov);
    else
      sm.rowy[i] = fdiv((float)(y0 + i) - (float)S.height / 2.0f, V.fov);
  }
  __syncthreads();
  uint32_t base = 0, total = 0;
#pragma unroll
  for (int w = 0; w < NW; w++) {
    const uint32_t c = s_warp[w];
    base += w < warp ? c : 0u;
    total += c;
  }
  if (cov) {
    const uint32_t k = base + __popc(m & ((1u << lane) - 1u));
    s_px[k] = (uint32_t)lp;
    s_d[k] = d;
    s_r[k] = r;
  }
  __syncthreads();
  if (threadIdx.x < total) {
    const uint32_t q = s_px[threadIdx.x];
    shade_covered<FEAT>(sc, V, S, srec, sm.lights, x0 + (int)(q & (kTile - 1)), y0 + (int)(q / kTile),
                        s_d[threadIdx.x], s_r[threadIdx.x], sm.colx, sm.rowy);
  }
}

// ---- the fused raster -> shade pass of many views ------------------------------
// One persistent, cooperative launch (every block resident) takes the pass's
// tiles from a work queue: each view's raster tiles (kernel1 + kernel2), and
// each view's shade tiles (kernel3), which the host orders after at least a
// grid's worth of later views' raster tiles.  kernel3's SSAO reads depth
// anywhere in its view (its tap offsets grow as the depth shrinks), so a
// shade tile waits until every raster tile of its view is done: a per-view
// counter, polled with a bounded wait.  Every item depends only on items
// taken before it, so the waits always end; a wait that reaches its limit
// anyway sets bit 2 of the pass's overflow word and leaves that tile
// unshaded (the host reports GBR_DEVICE_TIMEOUT).  One view's shading thus
// overlaps later views' rasters: the raster waits on block barriers, the
// shading is bound by instruction issue.
//
// queue: [0] next item, [1] unused, [2 + v] raster tiles done of view v
// (zeroed by the host before the launch).  sched: seg_start[nseg + 1] (first
// item of each segment; seg_start[nseg] = item count), then seg_view[nseg]
// (view | 1 << 31 for shade segments).
constexpr uint32_t kWaitPolls = 1u << 22;  // with ~0.25 us sleeps: about a second

__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

template <int NT, bool FEAT>
__global__ void __launch_bounds__(NT, 1024 / NT) k_raster_shade(Workspace ws, const Surface* __restrict__ surfs,
                                                                uint32_t nsurf, SceneDev sc,
                                                                const ViewParams* __restrict__ views,
                                                                const uint32_t* __restrict__ sched, uint32_t nseg,
                                                                uint32_t* __restrict__ queue) {
  union Smem {
    RasterSmem<NT, true> r;
    ShadeSmem s;
  };
  __shared__ Smem sm;
  __shared__ uint32_t s_item[2];
  __shared__ int s_ok;
  if (ws.ctr->overflow) return;
  const uint32_t nrec = min(ws.ctr->nrec, ws.rec_cap);
  const uint32_t total = __ldg(sched + nseg);
  if (threadIdx.x == 0) s_item[0] = atomicAdd(&queue[0], 1u);
  __syncthreads();
#pragma unroll 1
  for (int cur = 0;; cur ^= 1) {
    const uint32_t item = s_item[cur];
    if (item >= total) break;
    if (threadIdx.x == 0) s_item[cur ^ 1] = atomicAdd(&queue[0], 1u);  // the next item, taken early
    int seg = 0, hi = (int)nseg - 1;
    while (seg < hi) {
      const int mid = (seg + hi + 1) >> 1;
      if (__ldg(sched + mid) <= item) seg = mid; else hi = mid - 1;
    }
    const uint32_t info = __ldg(sched + nseg + 1 + seg);
    const uint32_t v = info & 0x7FFFFFFFu;
    const uint32_t tile = surfs[v].tile_base + (item - __ldg(sched + seg));
    if (!(info >> 31)) {
      raster_tile<NT, true>(ws, surfs, nsurf, tile, (int)v, sm.r);
      __threadfence();  // this thread's depth / id / record-map writes, before the count
      __syncthreads();
      if (threadIdx.x == 0) atomicAdd(&queue[2 + v], 1u);
    } else {
      if (threadIdx.x == 0) {
        const uint32_t need = (uint32_t)(surfs[v].tiles_x * surfs[v].tiles_y);
        int ok = 1;
        for (uint32_t polls = 0; ld_acquire_gpu(&queue[2 + v]) < need; polls++) {
          if (polls >= kWaitPolls) {
            ok = 0;
            atomicOr(&ws.ctr->overflow, 4u);
            break;
          }
          __nanosleep(256);
        }
        s_ok = ok;
      }
      __syncthreads();
      if (s_ok) shade_tile<FEAT, NT>(sc, views, surfs, ws.srec, nrec, tile, v, sm.s);
    }
    __syncthreads();
  }
}

// ---- texture atlas ----------------------------------------------------------------
// Slot origin of texture descriptor tid as write_tex_array computes it
// (cl2.cl:856-889).
__device__ __forceinline__ void tex_slot(const uint32_t* nums, const uint32_t* sizes, uint32_t tid,
                                         float* tnx, float* tny, int* slice, float* width) {
  uint32_t nv = nums[tid];
  *slice = (int)(nv >> 16);
  int which = (int)(nv & 0xFFFF);
  *width = (float)sizes[*slice];
  float hnum = floorf(fdiv(2048.0f, *width));
  float tnumy = floorf(fdiv((float)which, hnum));
  *tny = tnumy;
  *tnx = fma_(-tnumy, hnum, (float)which);
}

__device__ __forceinline__ void write_tex(uchar4* atlas, const uint32_t* nums, const uint32_t* sizes,
                                          uint32_t tid, float cx, float cy, uchar4 c) {
  float tnx, tny, w;
  int slice;
  tex_slot(nums, sizes, tid, &tnx, &tny, &slice, &w);
  float tx = tnx * w, ty = tny * w;
  cx = clampf_(fmodf(cx, w), 0.001f, w - 0.001f);
  cy = clampf_(fmodf(cy, w), 0.001f, w - 0.001f);
  int ix = (int)(tx + cx), iy = (int)(ty + cy);
  atlas[(size_t)slice * kTexPage * kTexPage + (size_t)iy * kTexPage + ix] = c;
}

__device__ __forceinline__ float4 read_tex(const uchar4* atlas, const uint32_t* nums, const uint32_t* sizes,
                                           uint32_t tid, float cx, float cy) {
  float tnx, tny, w;
  int slice;
  tex_slot(nums, sizes, tid, &tnx, &tny, &slice, &w);
  cx = clampf_(cx, 0.001f, w - 0.001f);
  cy = clampf_(cy, 0.001f, w - 0.001f);
  int ix = f2i_sat(fma_(tnx, w, cx)), iy = f2i_sat(fma_(tny, w, cy));
  uchar4 t = atlas[(size_t)slice * kTexPage * kTexPage + (size_t)iy * kTexPage + ix];
  return make_float4(t.x, t.y, t.z, t.w);
}

// update_gpu_tex with flip (cl2.cl:923-953); blockIdx.z = texture.
__global__ void k_tex_upload(uchar4* atlas, const uint32_t* nums, const uint32_t* sizes, const uint8_t* pixels,
                             const uint64_t* offsets, const int32_t* tsizes) {
  const uint32_t t = blockIdx.z;
  const int s = tsizes[t];
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= s || y >= s) return;
  uchar4 c = reinterpret_cast<const uchar4*>(pixels + offsets[t])[(size_t)y * s + x];
  float w = (float)sizes[nums[t] >> 16];
  write_tex(atlas, nums, sizes, t, (float)x, w - (float)y, c);
}

// generate_mips / generate_mip_mips (cl2.cl:1070-1189): level src -> src+1
// for every texture (blockIdx.z), grid over the base texture size.
__global__ void k_mip(uchar4* atlas, const uint32_t* nums, const uint32_t* sizes, uint32_t mipmap_start,
                      const int32_t* tsizes, int level) {
  const uint32_t t = blockIdx.z;
  const int s = tsizes[t];
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= s || y >= s) return;
  uint32_t src = level == 0 ? t : t * kMipLevels + mipmap_start + (uint32_t)(level - 1);
  uint32_t dst = t * kMipLevels + mipmap_start + (uint32_t)level;
  float w = (float)sizes[nums[src] >> 16];
  if ((float)x >= w || (float)y >= w) return;
  const float g[3] = {1.f, 2.f, 1.f};
  float a0 = 0, a1 = 0, a2 = 0, a3 = 0, div = 0;
  for (int j = -1; j <= 1; j++)
    for (int i = -1; i <= 1; i++) {
      float4 c = read_tex(atlas, nums, sizes, src, (float)(x * 2 + i), (float)(y * 2 + j));
      c.w = fdiv(c.w, 255.f);
      c.x *= c.w; c.y *= c.w; c.z *= c.w;
      float gw = g[j + 1] * g[i + 1];
      a0 += c.x * gw; a1 += c.y * gw; a2 += c.z * gw; a3 += c.w * gw;
      div += gw;
    }
  a0 = fdiv(a0, div); a1 = fdiv(a1, div); a2 = fdiv(a2, div); a3 = fdiv(a3, div);
  if (a3 > 0.00000001f) { a0 = fdiv(a0, a3); a1 = fdiv(a1, a3); a2 = fdiv(a2, a3); }
  a3 *= 255.f;
  float nw = (float)sizes[nums[dst] >> 16];
  float yx0 = fdiv((float)(x * 2), w) * nw, yx1 = fdiv((float)(y * 2), w) * nw;
  if (yx0 >= nw || yx1 >= nw) return;
  uchar4 c = make_uchar4((unsigned char)f2u_sat(a0), (unsigned char)f2u_sat(a1), (unsigned char)f2u_sat(a2),
                         (unsigned char)f2u_sat(a3));
  write_tex(atlas, nums, sizes, dst, yx0, yx1, c);
}

// object::g_flush's writes (object.cpp:652-860): pose, scale, texture id and
// feature flags of the listed descriptors.
__global__ void k_flush_objects(gbr_obj_g_descriptor* descs, const gbr_object_flush* objs, uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const gbr_object_flush f = objs[i];
  gbr_obj_g_descriptor* G = descs + f.index;
  for (int k = 0; k < 4; k++) {
    G->world_pos[k] = f.world_pos[k];
    G->world_rot_quat[k] = f.world_rot_quat[k];
  }
  G->scale = f.scale;
  G->tid = f.tid;
  G->feature_flag = f.feature_flag;
}

// Clear every surface of a depth-only pass to UINT_MAX before its setup
// rasterises small candidates into them (blockIdx.y = surface).
__global__ void __launch_bounds__(256) k_clear_surfaces(const Surface* __restrict__ surfs) {
  const Surface& S = surfs[blockIdx.y];
  const size_t n = (size_t)S.width * S.height;
  uint4* d4 = reinterpret_cast<uint4*>(S.depth);
  const uint4 v = make_uint4(kDepthClear, kDepthClear, kDepthClear, kDepthClear);
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n / 4; i += (size_t)gridDim.x * blockDim.x)
    d4[i] = v;
  if (blockIdx.x == 0 && threadIdx.x < (n & 3)) S.depth[(n & ~(size_t)3) + threadIdx.x] = kDepthClear;
}

// Atomic-rate probe (diagnostics): every thread issues `iters` 32-bit
// atomicMin.  Shared mode: each lane its own word of the block's 256 (a lane
// XOR keeps a warp's 32 words distinct, in 32 banks).  Global mode: words
// spread over an L2-resident array of nwords.
__global__ void __launch_bounds__(256) k_atomic_rate(uint32_t* g, uint32_t nwords, int iters, int shared_mode) {
  __shared__ uint32_t s[256];
  s[threadIdx.x] = 0xFFFFFFFFu;
  __syncthreads();
  const uint32_t v = blockIdx.x * 256u + threadIdx.x;
  if (shared_mode) {
    for (int i = 0; i < iters; i++) atomicMin(&s[threadIdx.x ^ (uint32_t)(i & 31)], v - (uint32_t)i);
    __syncthreads();
    if (s[threadIdx.x] == 0x12345u) g[0] = 0;  // keeps the shared result live
  } else {
    const uint32_t base = v % nwords;
    for (int i = 0; i < iters; i++) atomicMin(g + (base + (uint32_t)i * 4099u) % nwords, v - (uint32_t)i);
  }
}

__global__ void k_fill_u32(uint32_t* p, uint32_t v, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    p[i] = v;
}

int g_num_sms = 0;
int num_sms() {
  if (!g_num_sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 152;
  }
  return g_num_sms;
}

}  // namespace

cudaError_t launch_world(const SceneDev& sc, float4* world, float4* objq, uint32_t* objr, cudaStream_t st) {
  if (sc.ndescs) k_objects<<<(sc.ndescs + 255) / 256, 256, 0, st>>>(sc, objq);
  if (sc.ntris && world) {
    if (!objr) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(objr, 0, sizeof(uint32_t) * sc.ndescs, st);
    if (e != cudaSuccess) return e;
    k_world<<<(sc.ntris + 255) / 256, 256, 0, st>>>(sc, world, objr);
  }
  return cudaGetLastError();
}

cudaError_t launch_object_cull(const SceneDev& sc, const ViewParams* d_views, const Surface* d_surf, uint32_t nviews,
                               const uint32_t* objr, uint32_t words, uint32_t* vis, cudaStream_t st) {
  if (!nviews || !words) return cudaSuccess;
  if (!sc.objq || !objr || !vis || nviews > 65535) return cudaErrorInvalidValue;
  k_object_cull<<<dim3((words * 32 + 255) / 256, nviews), 256, 0, st>>>(sc, d_views, d_surf, objr, words, vis);
  return cudaGetLastError();
}

cudaError_t launch_texture_levels(const uint32_t* nums, const uint32_t* sizes, uint32_t mipmap_start, float4* texlv,
                                  cudaStream_t st) {
  const uint32_t n = mipmap_start * kTexLevels;
  if (n) k_texture_levels<<<(n + 255) / 256, 256, 0, st>>>(nums, sizes, mipmap_start, texlv);
  return cudaGetLastError();
}

cudaError_t launch_setup_views(const SceneDev& sc, const ViewParams* d_views, uint32_t nviews,
                               const Surface* d_surf, const Workspace& ws, cudaStream_t st) {
  if (!sc.ntris || !nviews) return cudaSuccess;
  dim3 grid((sc.ntris + 255) / 256, nviews);
  k_setup_views<<<grid, 256, 0, st>>>(sc, d_views, d_surf, ws);
  return cudaGetLastError();
}

cudaError_t launch_setup_shadow(const SceneDev& sc, const ShadowJob* d_jobs, uint32_t njobs,
                                const Surface* d_surf, const Workspace& ws, cudaStream_t st) {
  if (!sc.ntris || !njobs) return cudaSuccess;
  dim3 grid((sc.ntris + 127) / 128, njobs);  // small blocks: lanes' direct rasters differ in length
  k_setup_shadow<<<grid, 128, 0, st>>>(sc, d_jobs, d_surf, ws);
  return cudaGetLastError();
}

cudaError_t launch_tile_table(const Workspace& ws, const Surface* d_surf, uint32_t nsurf, cudaStream_t st) {
  if (!ws.nfine) return cudaSuccess;
  if (!ws.tiles || !nsurf) return cudaErrorInvalidValue;
  k_tile_table<<<(ws.nfine + 255) / 256, 256, 0, st>>>(d_surf, nsurf, ws.nfine, ws.coarse_shift,
                                                       const_cast<uint2*>(ws.tiles));
  return cudaGetLastError();
}

cudaError_t launch_scan(const Workspace& ws, cudaStream_t st) {
  const uint32_t nchunks = (ws.nfine + kScanChunk - 1) / kScanChunk;
  if (nchunks <= 1 || !ws.scan_part) {
    k_scan<<<1, kScanThreads, 0, st>>>(ws);
  } else {
    k_scan_chunks<<<nchunks + 1, kScanThreads, 0, st>>>(ws, nchunks);
    k_scan_add<<<nchunks, kScanThreads, 0, st>>>(ws, nchunks);
  }
  return cudaGetLastError();
}

uint32_t scan_chunks(uint32_t nfine) { return (nfine + kScanChunk - 1) / kScanChunk; }

cudaError_t launch_prep(const SceneDev& sc, const Workspace& ws, cudaStream_t st) {
  if (!ws.srec) return cudaErrorInvalidValue;
  k_prep<<<num_sms() * 4, 256, 0, st>>>(sc, ws);
  return cudaGetLastError();
}

cudaError_t launch_fill(const Workspace& ws, const Surface* d_surf, cudaStream_t st) {
  k_fill<<<num_sms() * 8, 256, 0, st>>>(ws, d_surf);
  return cudaGetLastError();
}

cudaError_t launch_raster(const Workspace& ws, const Surface* d_surf, uint32_t nsurf, uint32_t ntiles,
                          bool with_id, int threads, cudaStream_t st, uint32_t tiles_per_surface, uint32_t tile0) {
  if (!ntiles) return cudaSuccess;
  const int wid = with_id ? 1 : 0;
  // surfaces of equal size: one grid row per surface, no search for the owner
  const dim3 grid = (tile0 == 0 && tiles_per_surface && nsurf > 1 && nsurf <= 65535 &&
                     tiles_per_surface * nsurf == ntiles) ? dim3(tiles_per_surface, nsurf) : dim3(ntiles);
  if (with_id && ws.tiles) {
    switch (threads) {
      case 128: k_raster<128, true, true><<<grid, 128, 0, st>>>(ws, d_surf, nsurf, tile0); break;
      case 512: k_raster<512, true, true><<<grid, 512, 0, st>>>(ws, d_surf, nsurf, tile0); break;
      default: k_raster<256, true, true><<<grid, 256, 0, st>>>(ws, d_surf, nsurf, tile0); break;
    }
    return cudaGetLastError();
  }
  switch (threads * 2 + wid) {
    case 256: k_raster<128, false><<<grid, 128, 0, st>>>(ws, d_surf, nsurf, tile0); break;
    case 257: k_raster<128, true><<<grid, 128, 0, st>>>(ws, d_surf, nsurf, tile0); break;
    case 1024: k_raster<512, false><<<grid, 512, 0, st>>>(ws, d_surf, nsurf, tile0); break;
    case 1025: k_raster<512, true><<<grid, 512, 0, st>>>(ws, d_surf, nsurf, tile0); break;
    case 513: k_raster<256, true><<<grid, 256, 0, st>>>(ws, d_surf, nsurf, tile0); break;
    default: k_raster<256, false><<<grid, 256, 0, st>>>(ws, d_surf, nsurf, tile0); break;
  }
  return cudaGetLastError();
}

cudaError_t launch_shade(const SceneDev& sc, const ViewParams* d_views, uint32_t nviews, const Surface* d_surf,
                         uint32_t ntiles, const Workspace& ws, cudaStream_t st, bool features, uint32_t tile0) {
  if (!ntiles) return cudaSuccess;
  if (!sc.objq || !sc.texlv || !ws.srec || (nviews > 1 && !ws.tiles)) return cudaErrorInvalidValue;
  if (features)
    k_shade<true><<<ntiles, 256, 0, st>>>(sc, d_views, d_surf, nviews, ws.srec, ws.ctr, ws.rec_cap, tile0,
                                          ws.tile_empty, ws.tiles);
  else
    k_shade<false><<<ntiles, 256, 0, st>>>(sc, d_views, d_surf, nviews, ws.srec, ws.ctr, ws.rec_cap, tile0,
                                           ws.tile_empty, ws.tiles);
  return cudaGetLastError();
}

// Blocks of the fused pass that fit on the device at once (cooperative grid).
template <int NT, bool FEAT>
uint32_t fused_grid() {
  static uint32_t cached[2] = {0, 0};
  int dev = 0;
  cudaGetDevice(&dev);
  uint32_t& g = cached[dev > 0 ? 1 : 0];
  if (!g || dev > 1) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_raster_shade<NT, FEAT>, NT, 0) != cudaSuccess)
      per_sm = 0;
    g = (uint32_t)std::max(per_sm, 0) * (uint32_t)num_sms();
  }
  return g;
}

template <int NT, bool FEAT>
cudaError_t launch_fused_t(const SceneDev& sc, const ViewParams* d_views, const Surface* d_surf, uint32_t nsurf,
                           const Workspace& ws, const uint32_t* sched, uint32_t nseg, uint32_t* queue,
                           cudaStream_t st) {
  const uint32_t grid = fused_grid<NT, FEAT>();
  if (!grid) return cudaErrorInvalidConfiguration;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(NT);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_raster_shade<NT, FEAT>, ws, d_surf, nsurf, sc, d_views, sched, nseg, queue);
}

cudaError_t launch_raster_shade(const SceneDev& sc, const ViewParams* d_views, const Surface* d_surf, uint32_t nsurf,
                                const Workspace& ws, const uint32_t* sched, uint32_t nseg, uint32_t* queue,
                                int threads, cudaStream_t st, bool features) {
  if (!sc.objq || !sc.texlv || !ws.srec || !sched || !queue || !nseg) return cudaErrorInvalidValue;
  if (threads == 128)
    return features ? launch_fused_t<128, true>(sc, d_views, d_surf, nsurf, ws, sched, nseg, queue, st)
                    : launch_fused_t<128, false>(sc, d_views, d_surf, nsurf, ws, sched, nseg, queue, st);
  return features ? launch_fused_t<256, true>(sc, d_views, d_surf, nsurf, ws, sched, nseg, queue, st)
                  : launch_fused_t<256, false>(sc, d_views, d_surf, nsurf, ws, sched, nseg, queue, st);
}

uint32_t fused_blocks(int threads, bool features) {
  if (threads == 128) return features ? fused_grid<128, true>() : fused_grid<128, false>();
  return features ? fused_grid<256, true>() : fused_grid<256, false>();
}

cudaError_t launch_texture_upload(uchar4* atlas, const uint32_t* nums, const uint32_t* sizes,
                                  const uint8_t* pixels, const uint64_t* offsets, const int32_t* tsizes,
                                  uint32_t ntex, int32_t max_size, cudaStream_t st) {
  if (!ntex) return cudaSuccess;
  dim3 block(16, 16), grid((max_size + 15) / 16, (max_size + 15) / 16, ntex);
  k_tex_upload<<<grid, block, 0, st>>>(atlas, nums, sizes, pixels, offsets, tsizes);
  return cudaGetLastError();
}

cudaError_t launch_mips(uchar4* atlas, const uint32_t* nums, const uint32_t* sizes, uint32_t mipmap_start,
                        const int32_t* tsizes, uint32_t ntex, int32_t max_size, cudaStream_t st) {
  if (!ntex) return cudaSuccess;
  dim3 block(16, 16), grid((max_size + 15) / 16, (max_size + 15) / 16, ntex);
  for (int level = 0; level < kMipLevels; level++) {
    k_mip<<<grid, block, 0, st>>>(atlas, nums, sizes, mipmap_start, tsizes, level);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_flush_objects(gbr_obj_g_descriptor* descs, const gbr_object_flush* objs, uint32_t n,
                                 cudaStream_t st) {
  if (!n) return cudaSuccess;
  k_flush_objects<<<(n + 255) / 256, 256, 0, st>>>(descs, objs, n);
  return cudaGetLastError();
}

cudaError_t launch_clear_surfaces(const Surface* d_surf, uint32_t nsurf, cudaStream_t st) {
  if (!nsurf) return cudaSuccess;
  k_clear_surfaces<<<dim3(64, nsurf), 256, 0, st>>>(d_surf);
  return cudaGetLastError();
}

cudaError_t launch_atomic_rate(uint32_t* g, uint32_t nwords, int iters, int shared_mode, uint32_t blocks,
                               cudaStream_t st) {
  k_atomic_rate<<<blocks, 256, 0, st>>>(g, nwords, iters, shared_mode);
  return cudaGetLastError();
}

cudaError_t launch_fill_u32(uint32_t* p, uint32_t v, size_t n, cudaStream_t st) {
  if (!n) return cudaSuccess;
  k_fill_u32<<<num_sms() * 4, 256, 0, st>>>(p, v, n);
  return cudaGetLastError();
}

}  // namespace gbr

// Post passes over a rendered view (godrays, pseudo-AA, motion blur,
// reflections): they share the device helpers above.
#include "gbr_post.cuh"
