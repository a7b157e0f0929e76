// gbr_post.cuh -- post passes over a rendered view: the reference's
// screenspace_godrays, do_pseudo_aa, do_motion_blur and
// screenspace_reflections (cl2.cl:1792-1917, 6437-7356), behind
// engine::draw_godrays / do_pseudo_aa / do_motion_blur /
// draw_screenspace_reflections (engine.cpp:1463-1536).  Included at the end
// of gbr_kernels.cu, whose device helpers they use.  Every pass reads one
// RGBA8 image and writes another; a pixel the reference leaves unwritten keeps
// its input colour.
#pragma once

namespace gbr {

// screenspace_godrays (cl2.cl:1792-1917) for pixel (x, y) of a view: light
// shafts of every light with godray_intensity > 0, marched from the pixel
// towards the light's screen position over the depth buffer.  cc / cs: the
// camera's cosines and sines.  Returns the RGBA colour before quantisation.
__device__ f4 godrays_pixel(int x, int y, const uint32_t* depth, const uint8_t* rgba_in, int W, int H, float fov,
                        const gbr_light* __restrict__ lights, uint32_t nlights, f3 cpos, f3 cc, f3 cs) {
  const float samples = 80.f;
  const uint32_t my_depth = depth[(size_t)y * W + x];
  f4 my_col = read_linear_rgba8(rgba_in, W, H, (float)x - 0.25f, (float)y - 0.25f);
  const float decay_factor = 0.97f, weight = 0.01f;
  const float step = 400.f / samples;  // max_length / samples
  for (uint32_t i = 0; i < nlights; i++) {
    const gbr_light& L = lights[i];
    const float ray_intensity = L.godray_intensity;
    if (ray_intensity <= 0) continue;
    float idecay = 1.f;
    f3 iter_col = mk3(0, 0, 0);
    const f3 lpos = mk3(L.pos[0], L.pos[1], L.pos[2]);
    const f3 slpos = depth_project1(rot_cs(lpos, cpos, cc, cs), (float)W, (float)H, fov);
    f3 current = mk3((float)x, (float)y, depth_to_dist(my_depth));
    f3 dest = slpos;
    const f3 original = current;
    if (slpos.z < 0) dest = add3(sub3(current, dest), current);
    const float vx = fabsf(current.x - dest.x), vy = fabsf(current.y - dest.y);
    const float mnum = vx > vy ? vx : vy;
    f3 dir = sub3(dest, current);
    dir = mk3(fdiv(dir.x, mnum), fdiv(dir.y, mnum), fdiv(dir.z, mnum));
    dir = mul3s(dir, step);
    const f3 cval = mul3s(mk3(L.col[0], L.col[1], L.col[2]), ray_intensity);
    const float thr = original.z - 5.0f;
    // depth_to_dist(d) < thr exactly when depth_scaled(d) < thr * 2^32 (the
    // scaling by 2^-32 commutes with rounding): one multiplication per step
    const float thr_scaled = thr * kTwo32;
    const float xmax = (float)W - 1.0f, ymax = (float)H - 1.0f;
    // steps j with (float)j < mnum and j < samples
    const int n = mnum > 0.0f ? (int)fminf(ceilf(mnum), samples) : 0;
    float cx = current.x, cy = current.y;
    // A march whose whole segment, one step past its end, keeps 0.05 px inside
    // the screen needs no bounds tests: the positions move monotonically along
    // dir, and 80 float additions below 4096 stray from the exact line by less
    // than 0.01 px.  (Every comparison fails on NaN.)
    const float ex = cx + (float)n * dir.x, ey = cy + (float)n * dir.y;
    const bool inside = cx >= 0.05f && ex >= 0.05f && cx <= xmax - 0.05f && ex <= xmax - 0.05f &&
                        cy >= 0.05f && ey >= 0.05f && cy <= ymax - 0.05f && ey <= ymax - 0.05f;
    // Eight steps at a time: their positions (the same running sums as the
    // reference's current += dir), then their depth loads in flight together,
    // then the decay chain in order.  The reference skips the rest of the
    // march once it leaves the screen; an unoccluded step adds exactly 0.
    for (int j0 = 0; j0 < n; j0 += 8) {
      float px[8], py[8];
#pragma unroll
      for (int k = 0; k < 8; k++) {
        px[k] = cx;
        py[k] = cy;
        cx += dir.x;
        cy += dir.y;
      }
      int m = min(8, n - j0);
      if (!inside) {
#pragma unroll
        for (int k = 7; k >= 0; k--)
          if (px[k] < 0 || py[k] < 0 || px[k] >= xmax || py[k] >= ymax) m = min(m, k);
      }
      uint32_t dv[8];
#pragma unroll
      // (cvt.rzi: truncation, NaN -> 0, so a NaN march stays in bounds as in the oracle)
      for (int k = 0; k < 8; k++)
        dv[k] = k < m ? __ldg(depth + (size_t)__float2int_rz(py[k]) * W + __float2int_rz(px[k])) : 0u;
#pragma unroll
      for (int k = 0; k < 8; k++) {
        if (k < m) {
          // (the reference also requires cdepth != UINT_MAX; an empty pixel is at
          // 350000, never below thr = the pixel's own distance - 5 <= 349995)
          if (depth_scaled(dv[k]) < thr_scaled) {
            idecay *= 0.9f;
            iter_col = add3(iter_col, mul3s(mul3s(cval, idecay), weight));
          }
          idecay *= decay_factor;
        }
      }
      if (m < 8) break;
    }
    my_col.x += iter_col.x;
    my_col.y += iter_col.y;
    my_col.z += iter_col.z;
  }
  my_col.w = 1.0f;
  const float exposure = 0.99f;
  f4 r;
  r.x = my_col.x * exposure; r.y = my_col.y * exposure; r.z = my_col.z * exposure; r.w = my_col.w * exposure;
  return r;
}

// engine::draw_godrays (engine.cpp:1463-1482): one thread per pixel.
__global__ void __launch_bounds__(256) k_godrays(const uint32_t* __restrict__ depth, const uint8_t* __restrict__ in,
                                                 uint8_t* __restrict__ out, int W, int H, float fov,
                                                 const gbr_light* __restrict__ lights, uint32_t nlights, f3 cpos,
                                                 f3 cc, f3 cs) {
  const int x = blockIdx.x * 16 + (threadIdx.x & 15), y = blockIdx.y * 16 + (threadIdx.x >> 4);
  if (x >= W || y >= H) return;
  const f4 c = godrays_pixel(x, y, depth, in, W, H, fov, lights, nlights, cpos, cc, cs);
  reinterpret_cast<uint32_t*>(out)[(size_t)y * W + x] = pack_rgba(c.x, c.y, c.z, c.w);
}

cudaError_t launch_godrays(const uint32_t* depth, const uint8_t* in, uint8_t* out, int W, int H, float fov,
                           const gbr_light* lights, uint32_t nlights, const float cpos[3], const float cc[3],
                           const float cs[3], cudaStream_t st) {
  dim3 grid((W + 15) / 16, (H + 15) / 16);
  k_godrays<<<grid, 256, 0, st>>>(depth, in, out, W, H, fov, lights, nlights, mk3(cpos[0], cpos[1], cpos[2]),
                                  mk3(cc[0], cc[1], cc[2]), mk3(cs[0], cs[1], cs[2]));
  return cudaGetLastError();
}

// ---- do_pseudo_aa (cl2.cl:6437-6657) ---------------------------------------
// Pixel (x, y) is an edge when exactly one horizontal and one vertical
// neighbour, and at least one diagonal, differ from it: by more than 100 depth
// units (test 0), or by more than 20 degrees of normal (test 1).  The first
// test that finds an edge replaces the colour with 0.65 x the mean of the
// similar neighbours + 0.35 x the mean of the differing ones.
// The 8 neighbours in the reference's order (dy = -1..1, then dx = -1..1),
// bit j of an edge mask: diagonals j = 0, 2, 5, 7; horizontal 3, 4; vertical
// 1, 6.
constexpr uint32_t kAADiag = 0xA5u, kAAHoriz = 0x18u, kAAVert = 0x42u;
// A block covers 32x8 pixels, one row per warp (so that a warp's halo reads
// are 32 consecutive words, free of bank conflicts); with their neighbours,
// a 34x10 halo.
constexpr int kAABlockW = 32, kAABlockH = 8;
constexpr int kAAHalo = kAABlockW + 2, kAAHaloH = kAABlockH + 2;

// The pixel at halo index h (distances and decoded normals staged in shared
// memory): the edge masks of both tests, then, for the first test that
// finds an edge, the colour means in the reference's accumulation order.
// The colours are read only for edge pixels: the other test's sums never
// reach the output.
__device__ __forceinline__ bool pseudo_aa_pixel(int x, int y, int W, int h, const float* sd, const float* snx,
                                                const float* sny, const float* snz,
                                                const uchar4* __restrict__ in, f3* out) {
  const float here = sd[h];
  const f3 n0 = fast_normalize3(mk3(snx[h], sny[h], snz[h]));
  uint32_t e0 = 0, e1 = 0;
  int j = 0;
#pragma unroll
  for (int dy = -1; dy <= 1; dy++) {
#pragma unroll
    for (int dx = -1; dx <= 1; dx++) {
      if (dx == 0 && dy == 0) continue;
      const int hq = h + dy * kAAHalo + dx;
      if (fabsf(sd[hq] - here) > 100.0f) e0 |= 1u << j;
      if (dot3(n0, mk3(snx[hq], sny[hq], snz[hq])) < kAACos) e1 |= 1u << j;
      j++;
    }
  }
  auto is_edge = [](uint32_t e) {
    return __popc(e & kAAHoriz) == 1 && __popc(e & kAAVert) == 1 && (e & kAADiag) != 0;
  };
  uint32_t e;
  if (is_edge(e0)) e = e0;
  else if (is_edge(e1)) e = e1;
  else return false;
  f3 same = mk3(0, 0, 0), other = mk3(0, 0, 0);
  float nsame = 0, nother = 0;
  j = 0;
#pragma unroll
  for (int dy = -1; dy <= 1; dy++) {
#pragma unroll
    for (int dx = -1; dx <= 1; dx++) {
      if (dx == 0 && dy == 0) continue;
      const uchar4 t = in[(size_t)(y + dy) * W + (x + dx)];
      const f3 c = mk3(u8_over_255(t.x), u8_over_255(t.y), u8_over_255(t.z));  // fdiv(t, 255.0f)
      if ((e >> j) & 1u) {
        other = add3(other, c);
        nother += 1.0f;
      } else {
        same = add3(same, c);
        nsame += 1.0f;
      }
      j++;
    }
  }
  const f3 m = mk3(fdiv(same.x, nsame), fdiv(same.y, nsame), fdiv(same.z, nsame));
  const f3 o = mk3(fdiv(other.x, nother), fdiv(other.y, nother), fdiv(other.z, nother));
  *out = add3(mul3s(m, 0.65f), mul3s(o, 0.35f));
  return true;
}

// engine::do_pseudo_aa (engine.cpp:1513-1516): one thread per pixel, 32x8
// pixels per block.  The block's 34x10 neighbourhood of distances and
// decoded normals is staged in shared memory first: each is decoded once
// instead of by each of its nine readers.
__global__ void __launch_bounds__(256) k_pseudo_aa(const uint32_t* __restrict__ depth, const uint32_t* __restrict__ ids,
                                                   const ushort2* __restrict__ nrm, const uchar4* __restrict__ in,
                                                   uchar4* __restrict__ out, int W, int H) {
  constexpr int E = kAAHalo, N = kAAHalo * kAAHaloH;
  __shared__ float sd[N], snx[N], sny[N], snz[N];
  const int bx = blockIdx.x * kAABlockW, by = blockIdx.y * kAABlockH;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const int hx = bx - 1 + i % E, hy = by - 1 + i / E;
    float d = 0.0f;
    f3 n = mk3(0, 0, 0);
    if (hx >= 0 && hy >= 0 && hx < W && hy < H) {
      const size_t q = (size_t)hy * W + hx;
      d = depth_to_dist(depth[q]);
      const ushort2 nq = nrm[q];
      n = decode_normal(nq.x, nq.y);
    }
    sd[i] = d;
    snx[i] = n.x;
    sny[i] = n.y;
    snz[i] = n.z;
  }
  __syncthreads();
  const int lx = threadIdx.x % kAABlockW, ly = threadIdx.x / kAABlockW;
  const int x = bx + lx, y = by + ly;
  if (x >= W || y >= H) return;
  const size_t p = (size_t)y * W + x;
  f3 c;
  const bool inner = x >= 1 && y >= 1 && x < W - 1 && y < H - 1;
  if (inner && depth[p] != kDepthClear && ids[p] != kNoId &&
      pseudo_aa_pixel(x, y, W, (ly + 1) * E + lx + 1, sd, snx, sny, snz, in, &c)) {
    reinterpret_cast<uint32_t*>(out)[p] = pack_rgba(c.x, c.y, c.z, 1.0f);
  } else {
    out[p] = in[p];
  }
}

cudaError_t launch_pseudo_aa(const uint32_t* depth, const uint32_t* ids, const uint16_t* normals, const uint8_t* in,
                             uint8_t* out, int W, int H, cudaStream_t st) {
  dim3 grid((W + kAABlockW - 1) / kAABlockW, (H + kAABlockH - 1) / kAABlockH);
  k_pseudo_aa<<<grid, kAABlockW * kAABlockH, 0, st>>>(depth, ids, reinterpret_cast<const ushort2*>(normals),
                                    reinterpret_cast<const uchar4*>(in), reinterpret_cast<uchar4*>(out), W, H);
  return cudaGetLastError();
}

// ---- do_motion_blur (cl2.cl:6714-6860) ---------------------------------------
// The pixel's surface point, in its object's frame, is carried through the
// object's pose of the previous frame (history slot 1 on even frame ids, 2 on
// odd) and projected with this frame's and the previous frame's camera; the
// blend of the two screen motions (camera_contribution), times strength and
// capped at 50 px, is averaged over that many bilinear taps centred on the
// pixel.  Objects with a pixel on screen are marked in seen[] for the history
// update.
struct MotionCam {
  f3 cpos, cc, cs, opos, oc, os;
  float fov, strength, cam_w;
  uint32_t frame_id;
};

__global__ void __launch_bounds__(256) k_motion_blur(const gbr_triangle* __restrict__ tris,
                                                     const gbr_obj_g_descriptor* __restrict__ descs,
                                                     const uint32_t* __restrict__ depth,
                                                     const uint32_t* __restrict__ ids, const uint8_t* __restrict__ in,
                                                     uint8_t* __restrict__ out, int W, int H, MotionCam a,
                                                     uint32_t* __restrict__ seen, uint32_t ntris) {
  // the 256 quotients c / 255 of a channel byte (u8_over_255), read by every
  // bilinear tap from shared memory
  __shared__ float s255[256];
  s255[threadIdx.x] = u8_over_255(threadIdx.x);
  __syncthreads();
  struct Tab {
    const float* t;
    __device__ float operator()(uint32_t c) const { return t[c]; }
  };
  const Tab tab{s255};
  const int x = blockIdx.x * 16 + (threadIdx.x & 15), y = blockIdx.y * 16 + (threadIdx.x >> 4);
  if (x >= W || y >= H) return;
  const size_t p = (size_t)y * W + x;
  const uint32_t d = depth[p], id = ids[p];
  uint32_t* o32 = reinterpret_cast<uint32_t*>(out);
  if (d == kDepthClear || id == kNoId || (id >> 1) >= ntris) {  // (an id past the triangles: left as it is)
    o32[p] = reinterpret_cast<const uint32_t*>(in)[p];
    return;
  }
  const uint32_t obj = __ldg(&tris[id >> 1].vertices[0].object_id);
  if (!seen[obj]) seen[obj] = 1u;
  const gbr_obj_g_descriptor* G = descs + obj;
  const float dist = depth_to_dist(d);
  const f3 local = mk3(fdiv(((float)x - (float)W / 2.0f) * dist, a.fov), fdiv(((float)y - (float)H / 2.0f) * dist, a.fov),
                       dist);
  const f3 world = add3(back_rot_cs(local, mk3(0, 0, 0), a.cc, a.cs), a.cpos);
  const f3 objl = back_rot_quat(sub3(world, ld3(G->world_pos)), ld4(G->world_rot_quat));
  const bool even = (a.frame_id & 1u) == 0;
  const f3 opos = ld3(even ? G->old_world_pos_1 : G->old_world_pos_2);
  const f4 oq = ld4(even ? G->old_world_rot_quat_1 : G->old_world_rot_quat_2);
  const f3 last = add3(rot_quat(objl, oq), opos);
  const f3 nocam = depth_project1(rot_cs(last, a.cpos, a.cc, a.cs), (float)W, (float)H, a.fov);
  const f3 prev = depth_project1(rot_cs(last, a.opos, a.oc, a.os), (float)W, (float)H, a.fov);
  f4 acc;
  if (prev.z < 20.0f) {
    acc = read_linear_rgba8_with(in, W, H, (float)x + 0.5f, (float)y + 0.5f, tab);
  } else {
    float mx = (float)x - prev.x, my = (float)y - prev.y;
    const float nx = (float)x - nocam.x, ny = (float)y - nocam.y;
    mx = a.cam_w * mx + (1.0f - a.cam_w) * nx;
    my = a.cam_w * my + (1.0f - a.cam_w) * ny;
    mx = mx * a.strength;
    my = my * a.strength;
    int n = f2i_sat(fmax_(fabsf(mx), fabsf(my)) + 1.0f);
    if (n > 50) {
      mx = fdiv(mx, (float)n) * 50.0f;
      my = fdiv(my, (float)n) * 50.0f;
      n = 50;
    }
    float sx = 0.0f, sy = 0.0f;
    if (n != 0) {
      sx = fdiv(mx, (float)n);
      sy = fdiv(my, (float)n);
    }
    float cx = (float)x - mx * 0.5f, cy = (float)y - my * 0.5f;  // mx / 2 exactly
    acc.x = acc.y = acc.z = acc.w = 0.0f;
    float cnt = 0.0f;
    for (int i = 0; i < n; i++, cx += sx, cy += sy) {
      if (cx < 0 || cx >= (float)W || cy < 0 || cy >= (float)H) continue;
      const f4 c = read_linear_rgba8_with(in, W, H, cx + 0.5f, cy + 0.5f, tab);
      acc.x += c.x; acc.y += c.y; acc.z += c.z; acc.w += c.w;
      cnt += 1.0f;
    }
    if (cnt != 0.0f) {
      acc.x = fdiv(acc.x, cnt); acc.y = fdiv(acc.y, cnt); acc.z = fdiv(acc.z, cnt); acc.w = fdiv(acc.w, cnt);
    }
  }
  o32[p] = pack_rgba(acc.x, acc.y, acc.z, acc.w);
}

// The pose-history writes of do_motion_blur (cl2.cl:6771-6786): every object
// with a pixel on screen stores its current pose in the slot the next frame
// reads (2 on even frame ids, 1 on odd); the marks are cleared.
__global__ void k_motion_history(gbr_obj_g_descriptor* descs, uint32_t* seen, uint32_t n, uint32_t frame_id) {
  const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= n || !seen[o]) return;
  seen[o] = 0;
  gbr_obj_g_descriptor* G = descs + o;
  float* pos = (frame_id & 1u) == 0 ? G->old_world_pos_2 : G->old_world_pos_1;
  float* q = (frame_id & 1u) == 0 ? G->old_world_rot_quat_2 : G->old_world_rot_quat_1;
  for (int k = 0; k < 3; k++) pos[k] = G->world_pos[k];
  for (int k = 0; k < 4; k++) q[k] = G->world_rot_quat[k];
}

cudaError_t launch_motion_blur(const gbr_triangle* tris, uint32_t ntris, gbr_obj_g_descriptor* descs, uint32_t ndescs,
                               const uint32_t* depth, const uint32_t* ids, const uint8_t* in, uint8_t* out, int W,
                               int H, float fov, const float cpos[3], const float cc[3], const float cs[3],
                               const float opos[3], const float oc[3], const float os[3], uint32_t frame_id,
                               float strength, float camera_contribution, uint32_t* seen, cudaStream_t st) {
  MotionCam a;
  a.cpos = mk3(cpos[0], cpos[1], cpos[2]);
  a.cc = mk3(cc[0], cc[1], cc[2]);
  a.cs = mk3(cs[0], cs[1], cs[2]);
  a.opos = mk3(opos[0], opos[1], opos[2]);
  a.oc = mk3(oc[0], oc[1], oc[2]);
  a.os = mk3(os[0], os[1], os[2]);
  a.fov = fov;
  a.strength = strength;
  a.cam_w = camera_contribution;
  a.frame_id = frame_id;
  dim3 grid((W + 15) / 16, (H + 15) / 16);
  k_motion_blur<<<grid, 256, 0, st>>>(tris, descs, depth, ids, in, out, W, H, a, seen, ntris);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || !ndescs) return e;
  k_motion_history<<<(ndescs + 255) / 256, 256, 0, st>>>(descs, seen, ndescs, frame_id);
  return cudaGetLastError();
}

// ---- screenspace_reflections (cl2.cl:6862-7355) -----------------------------
// interpolate_single_line_depth (cl2.cl:6862-6873): the point at parameter a
// on the screen-space segment s -> f, depth interpolated in 1/z.
__device__ __forceinline__ f3 line_depth_point(f3 s, f3 f, float a) {
  s.z = rcp(s.z);
  f.z = rcp(f.z);
  const float b = 1.0f - a;
  const f3 r = mk3(fma_(s.x, b, f.x * a), fma_(s.y, b, f.y * a), fma_(s.z, b, f.z * a));
  return mk3(r.x, r.y, rcp(r.z));
}

struct ReflectCam {
  f3 cpos, cc, cs;
  float fov;
};

// A pixel of an object with FEATURE_FLAG_SS_REFLECTIVE: the eye ray mirrored
// in the interpolated normal is marched in screen space from a point 10.5
// units along it (at most 200 steps, until it passes more than 1 unit behind
// the depth buffer), refined in tenths of a step, and the colour there mixed
// in by a contact fade (400 units, fading towards the screen edge) times the
// object's reflection map (ssid) when it has one.  Returns 0 when the pixel
// keeps its colour.  Background pixels become 0.
__device__ int reflection_pixel(const SceneDev& sc, const ReflectCam& v, int x, int y, int W, int H,
                                const uint32_t* __restrict__ depth, const uint32_t* __restrict__ ids,
                                const uint8_t* __restrict__ in, f4* out) {
  const size_t p = (size_t)y * W + x;
  const uint32_t d = depth[p];
  if (d == kDepthClear) {
    out->x = out->y = out->z = out->w = 0.0f;
    return 1;
  }
  const uint32_t id = ids[p];
  if (id == kNoId || (id >> 1) >= sc.ntris) return 0;
  const uint32_t tri = id >> 1, sub = id & 1u;
  const gbr_triangle* T = sc.tris + tri;
  const uint32_t o_id = __ldg(&T->vertices[0].object_id);
  const gbr_obj_g_descriptor* G = sc.descs + o_id;
  if (!((__ldg(&G->feature_flag) & 1) > 0)) return 0;
  const float dist = depth_to_dist(d);
  const f3 local = mk3(fdiv(((float)x - (float)W / 2.0f) * dist, v.fov), fdiv(((float)y - (float)H / 2.0f) * dist, v.fov),
                       dist);
  const f3 zero = mk3(0, 0, 0);
  const f3 world = add3(back_rot_cs(local, zero, v.cc, v.cs), v.cpos);
  const f3 ray = sub3(world, v.cpos);
  const float scale = __ldg(&G->scale);
  f3 pv[3], nv[3];
  f2 tv[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    pv[k] = mul3s(ld3(T->vertices[k].pos), scale);
    nv[k] = ld3(T->vertices[k].normal);
    tv[k] = mk2(__ldg(&T->vertices[k].vt[0]), __ldg(&T->vertices[k].vt[1]));
  }
  const f4 q = ld4(G->world_rot_quat);
  const f3 wpos = ld3(G->world_pos);
  const BaryFrame bf = bary_frame(pv[0], pv[1], pv[2]);
  float l1, l2, l3;
  bary_exact(bf, back_rot_quat(sub3(world, wpos), q), &l1, &l2, &l3);
  f3 normal = mk3(fma_(nv[0].x, l1, fma_(nv[1].x, l2, nv[2].x * l3)), fma_(nv[0].y, l1, fma_(nv[1].y, l2, nv[2].y * l3)),
                  fma_(nv[0].z, l1, fma_(nv[1].z, l2, nv[2].z * l3)));
  normal = fast_normalize3(rot_quat(normal, q));
  const f2 vt = mk2(fma_(tv[0].x, l1, fma_(tv[1].x, l2, tv[2].x * l3)), fma_(tv[0].y, l1, fma_(tv[1].y, l2, tv[2].y * l3)));
  float refl = 1.0f;
  const uint32_t ssid = __ldg(&G->ssid);
  if (ssid != 0xFFFFFFFFu) {
    // the pixel's clip output, as prearrange wrote it to cutdown_tris
    f3 w[3], o0[3], o1[3];
    uint32_t oid;
    load_world(sc, tri, w, &oid);
    const int n = transform_clip(w, v.cpos, v.cc, v.cs, v.fov, (float)W, (float)H, o0, o1);
    if ((int)sub >= n) return 0;
    const f3* tp = sub ? o1 : o0;
    const f3 xpv = mk3(roundf(tp[0].x), roundf(tp[1].x), roundf(tp[2].x));
    const f3 ypv = mk3(roundf(tp[0].y), roundf(tp[1].y), roundf(tp[2].y));
    const float rc = rconstant(xpv, ypv);
    // get_vtdiff (cl2.cl:5691-5760), per pixel
    const f3 depths = mk3(rcp(tp[0].z), rcp(tp[1].z), rcp(tp[2].z));
    float DA, DB, DC;
    plane_const(depths, xpv, ypv, rc, &DA, &DB, &DC);
    const float fx = (float)x, fy = (float)y;
    const float dmx = fma_(DA, fx + 1.0f, fma_(DB, fy, DC));
    const float dmy = fma_(DA, fx, fma_(DB, fy + 1.0f, DC));
    const float hw = (float)W / 2.0f, hh = (float)H / 2.0f;
    f3 lmx = mk3(fdiv((fx + 1.0f) - hw, v.fov), fdiv(fy - hh, v.fov), 1.0f);
    f3 lmy = mk3(fdiv(fx - hw, v.fov), fdiv((fy + 1.0f) - hh, v.fov), 1.0f);
    lmx = mk3(fdiv(lmx.x, dmx), fdiv(lmx.y, dmx), fdiv(lmx.z, dmx));
    lmy = mk3(fdiv(lmy.x, dmy), fdiv(lmy.y, dmy), fdiv(lmy.z, dmy));
    const f3 gmx = back_rot_quat(sub3(add3(back_rot_cs(lmx, zero, v.cc, v.cs), v.cpos), wpos), q);
    const f3 gmy = back_rot_quat(sub3(add3(back_rot_cs(lmy, zero, v.cc, v.cs), v.cpos), wpos), q);
    float lx1, lx2, lx3, ly1, ly2, ly3;
    bary_exact(bf, gmx, &lx1, &lx2, &lx3);
    bary_exact(bf, gmy, &ly1, &ly2, &ly3);
    const f2 vtx = mk2(fma_(tv[0].x, lx1, fma_(tv[1].x, lx2, tv[2].x * lx3)),
                       fma_(tv[0].y, lx1, fma_(tv[1].y, lx2, tv[2].y * lx3)));
    const f2 vty = mk2(fma_(tv[0].x, ly1, fma_(tv[1].x, ly2, tv[2].x * ly3)),
                       fma_(tv[0].y, ly1, fma_(tv[1].y, ly2, tv[2].y * ly3)));
    const float mip_bias = 1.0f / kMipBias;
    const f2 vtdiff = mk2((fabsf(vtx.x - vt.x) + fabsf(vty.x - vt.x)) * mip_bias,
                          (fabsf(vtx.y - vt.y) + fabsf(vty.y - vt.y)) * mip_bias);
    refl = texture_filter_diff<false>(sc, vt, vtdiff, (int)ssid).x;
    if (refl < 0.1f) return 0;
  }
  // reflect (cl2.cl:169-176) normalises the normal once more
  const f3 nn = fast_normalize3(normal);
  const float k2 = 2.0f * dot3(ray, nn);
  const f3 refd = fast_normalize3(sub3(ray, mul3s(nn, k2)));
  const f3 jit = add3(world, mul3s(refd, 10.5f));
  const f3 sj = depth_project1(rot_cs(jit, v.cpos, v.cc, v.cs), (float)W, (float)H, v.fov);
  const f3 ss = depth_project1(rot_cs(world, v.cpos, v.cc, v.cs), (float)W, (float)H, v.fov);
  const float dx = sj.x - ss.x, dy = sj.y - ss.y;
  const float sdist = fsqrt(dx * dx + dy * dy);
  const float back = 1.0f - fdiv(sdist - 3.0f, sdist);
  f3 vprev = mk3(ss.x * back + sj.x * (1.0f - back), ss.y * back + sj.y * (1.0f - back),
                 rcp(ss.z) * back + rcp(sj.z) * (1.0f - back));
  vprev.z = rcp(vprev.z);
  const f3 vstart = sj;
  const float fw = (float)W, fh = (float)H;
  if (sj.x < 0 || sj.y < 0 || sj.x >= fw || sj.y >= fh) return 0;
  // The march: step i at sj (i = 0) or line_depth_point(vprev, vstart, 1 + i),
  // i < 200, until the depth buffer is more than 1 unit in front of the ray;
  // a step off screen ends it unmet.  Step 0 first, then four steps at a
  // time: positions first (they do not depend on the loads), then their
  // depth loads in flight together, then the tests in order.
  const float ipz = rcp(vprev.z), isz = rcp(vstart.z);  // line_depth_point's reciprocals, loop-invariant
  // a step on screen has 0 <= x < W and 0 <= y < H, or a NaN coordinate
  // (every comparison of the test fails on NaN): f2i_sat is then a
  // truncation, or 0 for NaN
  auto on_screen_int = [](float c) { return c == c ? (int)c : 0; };
  float a = 1.0f, stop = 0.0f;
  bool found = false;
  {
    const float dd = depth_to_dist(__ldg(depth + (size_t)on_screen_int(sj.y) * W + on_screen_int(sj.x)));
    if (dd < sj.z - 1.0f) {
      found = true;
      stop = dd;  // the refinement reads the depth where the march stopped on every try
    }
  }
  for (int i0 = 1; i0 < 200 && !found; i0 += 4) {
    f3 pt[4];
    int m = min(4, 200 - i0);  // the first step off screen, or past the last
    const float fi0 = (float)i0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      // ai = 1 + i and b = 1 - ai = -i, both exact (integers below 2^24)
      const float fi = fi0 + (float)k, ai = fi + 1.0f;
      pt[k] = mk3(fma_(vprev.x, -fi, vstart.x * ai), fma_(vprev.y, -fi, vstart.y * ai), rcp(fma_(ipz, -fi, isz * ai)));
    }
#pragma unroll
    for (int k = 3; k >= 0; k--)
      if (pt[k].x < 0 || pt[k].y < 0 || pt[k].x >= fw || pt[k].y >= fh) m = min(m, k);
    uint32_t dv[4];
#pragma unroll
    for (int k = 0; k < 4; k++)
      dv[k] = k < m ? __ldg(depth + (size_t)on_screen_int(pt[k].y) * W + on_screen_int(pt[k].x)) : 0u;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      if (found) break;
      if (k >= m) return 0;  // off screen (or past step 199) before the ray met anything
      const float dd = depth_to_dist(dv[k]);
      if (dd < pt[k].z - 1.0f) {
        found = true;
        a = fi0 + (float)(k + 1);  // 1 + i
        stop = dd;
      }
    }
  }
  if (!found) return 0;
  float ta = a;
  f3 hit = sj;
  bool ok = false;
  for (int i = 0; i < 10; i++) {
    // line_depth_point(vprev, vstart, ta) with its two reciprocals hoisted
    const float tb = 1.0f - ta;
    hit = mk3(fma_(vprev.x, tb, vstart.x * ta), fma_(vprev.y, tb, vstart.y * ta), rcp(fma_(ipz, tb, isz * ta)));
    if (stop < hit.z + 1.0f && stop > hit.z - 20.0f) {
      ok = true;
      break;
    }
    ta += 0.1f;  // fdiv(1.0f, 10.0f) = RN(0.1)
  }
  if (!ok) return 0;
  const f3 te = line_depth_point(vstart, hit, 1.35f);
  float fextra = 0.0f;
  if (te.x < 0) fextra += fabsf(te.x);
  if (te.y < 0) fextra += fabsf(te.y);
  if (te.x >= fw) fextra += te.x - fw;
  if (te.y >= fh) fextra += te.y - fh;
  fextra = clampf_(fdiv(fextra, 200.0f), 0.0f, 1.0f);
  f3 gl = mk3(fdiv((hit.x - fw / 2.0f) * hit.z, v.fov), fdiv((hit.y - fh / 2.0f) * hit.z, v.fov), hit.z);
  gl = add3(back_rot_cs(gl, zero, v.cc, v.cs), v.cpos);
  const float ray_len = fast_length3(sub3(gl, world));
  float fade = 1.0f - fdiv(ray_len, 400.0f);
  fade = fade - fextra;
  fade = clampf_(fade, 0.0f, 1.0f) * refl;
  const f4 fc = read_linear_rgba8(in, W, H, hit.x, hit.y);
  const uchar4 t = reinterpret_cast<const uchar4*>(in)[p];
  const float den = 1.0f + fade;
  out->x = fdiv(u8_over_255(t.x) + fc.x * fade, den);  // u8_over_255(t) = fdiv(t, 255.0f)
  out->y = fdiv(u8_over_255(t.y) + fc.y * fade, den);
  out->z = fdiv(u8_over_255(t.z) + fc.z * fade, den);
  out->w = 1.0f;
  return 1;
}

// engine::draw_screenspace_reflections (engine.cpp:1483-1511): one thread per pixel.
__global__ void __launch_bounds__(256, 4) k_reflections(SceneDev sc, ReflectCam v, const uint32_t* __restrict__ depth,
                                                     const uint32_t* __restrict__ ids, const uint8_t* __restrict__ in,
                                                     uint8_t* __restrict__ out, int W, int H) {
  const int x = blockIdx.x * 16 + (threadIdx.x & 15), y = blockIdx.y * 16 + (threadIdx.x >> 4);
  if (x >= W || y >= H) return;
  const size_t p = (size_t)y * W + x;
  f4 c;
  uint32_t* o32 = reinterpret_cast<uint32_t*>(out);
  if (reflection_pixel(sc, v, x, y, W, H, depth, ids, in, &c))
    o32[p] = pack_rgba(c.x, c.y, c.z, c.w);
  else
    o32[p] = reinterpret_cast<const uint32_t*>(in)[p];
}

cudaError_t launch_reflections(const SceneDev& sc, const uint32_t* depth, const uint32_t* ids, const uint8_t* in,
                               uint8_t* out, int W, int H, float fov, const float cpos[3], const float cc[3],
                               const float cs[3], cudaStream_t st) {
  ReflectCam v;
  v.cpos = mk3(cpos[0], cpos[1], cpos[2]);
  v.cc = mk3(cc[0], cc[1], cc[2]);
  v.cs = mk3(cs[0], cs[1], cs[2]);
  v.fov = fov;
  dim3 grid((W + 15) / 16, (H + 15) / 16);
  k_reflections<<<grid, 256, 0, st>>>(sc, v, depth, ids, in, out, W, H);
  return cudaGetLastError();
}

}  // namespace gbr
