// gbr_math.h — the determinism contract of the triangle pipeline.
//
// The reference pipeline (cl2.cl, built with -cl-fast-relaxed-math and
// FP_CONTRACT ON) leaves many float operations implementation-defined.  This
// header pins every one of them to a single definition that compiles
// identically for the CUDA kernels (nvcc, --fmad=false) and for host C++
// (g++ -ffp-contract=off), so that integer outputs (depth, canonical id) are
// bit-identical between the GPU path and any CPU restatement:
//
//   mad(a,b,c)          -> fmaf(a,b,c)                (only where cl2.cl writes mad)
//   a*b+c elsewhere     -> two roundings, never contracted
//   native_divide, '/'  -> IEEE round-to-nearest division
//   native_recip(x)     -> 1.0f / x (IEEE)
//   fast_length/normalize -> IEEE sqrt, then IEEE division
//   native_cos/sin of view-uniform angles (camera Euler angles, the six cube
//                          face rotations) -> computed once on the host in
//                          double precision and rounded to float
//   round               -> half away from zero (roundf)
//   float -> uint       -> truncation, saturating to [0, UINT_MAX], NaN -> 0
//   pow(x, n), n small integer -> repeated multiplication
//   tan (shadow bias)   -> gbr_tanf below (Taylor series of sin and cos)
//   denormals           -> kept (IEEE) on both sides; the reference flushes them,
//                          but no denormal reaches the depth or id arithmetic
//
// Everything here is plain arithmetic written for this project; nothing is
// taken from CUDA's math library.
#pragma once

#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define GBR_HD __host__ __device__ __forceinline__
#else
#define GBR_HD inline
#endif

namespace gbr {

// Constants of the reference pipeline (cl2.cl:5-27, 4247-4252, 5387, ocl.h:234).
constexpr float kDepthFar = 350000.0f;        // depth_far
constexpr float kDepthCutoff = 20.0f;         // depth_icutoff
constexpr float kMulInt = 4294967296.0f;      // (float)UINT_MAX
constexpr uint32_t kDepthClear = 0xFFFFFFFFu; // UINT_MAX
constexpr int kOpSize = 500;                  // op_size (pixels per view fragment)
constexpr int kOpSizeLight = 300;             // op_size_light (pixels per cube fragment)
constexpr uint32_t kBufError = 20;            // BUF_ERROR
constexpr int kMipLevels = 4;                 // MIP_LEVELS
constexpr float kShadowBias = 50.0f;          // SHADOWBIAS
constexpr int kLightBufferDim = 1024;         // LIGHTBUFFERDIM (engine l_size)
constexpr float kLFov = 512.0f;               // LFOV_CONST = LIGHTBUFFERDIM/2
constexpr float kPi = 3.1415927f;             // M_PI as cl2.cl defines it
constexpr float kAmbient = 0.2f;              // -D AMBIENT=0.2f (main.cpp:82)
constexpr float kSsaoRad = 2.0f;              // -D SSAO_RAD=2.f (main.cpp:83)
constexpr float kSsaoDiv = 2.5f;              // SSAO_DIV
constexpr float kMipBias = 1.1f;              // MIP_BIAS
constexpr int kTexPage = 2048;                // max_tex_size / TEXTURE_CONTEXT_MAX_SIZE_IMAGE
constexpr uint32_t kNoId = 0xFFFFFFFFu;       // canonical id of an empty pixel

// feature_flag bits (cl2.cl:90-97)
constexpr int kFlagTwoSided = 2;
constexpr int kFlagOutline = 4;
constexpr int kFlagIsStatic = 8;
constexpr int kFlagNoDynShadows = 16;

struct f2 { float x, y; };
struct f3 { float x, y, z; };
struct f4 { float x, y, z, w; };

GBR_HD f3 mk3(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
GBR_HD f2 mk2(float x, float y) { f2 r; r.x = x; r.y = y; return r; }

// ---- pinned scalar primitives -------------------------------------------
GBR_HD float fdiv(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fdiv_rn(a, b);
#else
  return a / b;
#endif
}
GBR_HD float fsqrt(float a) {
#if defined(__CUDA_ARCH__)
  return __fsqrt_rn(a);
#else
  return sqrtf(a);
#endif
}
GBR_HD float fma_(float a, float b, float c) { return fmaf(a, b, c); }
GBR_HD float rcp(float x) { return fdiv(1.0f, x); }
// OpenCL float min/max are undefined for NaN operands; pinned to IEEE
// minNum/maxNum (a NaN operand is ignored), which is what GPU min/max do.
GBR_HD float fmin_(float x, float y) { return fminf(x, y); }
GBR_HD float fmax_(float x, float y) { return fmaxf(x, y); }
GBR_HD float clampf_(float x, float lo, float hi) { return fmin_(fmax_(x, lo), hi); }
GBR_HD float min3f(float a, float b, float c) { return fmin_(fmin_(a, b), c); }
GBR_HD float max3f(float a, float b, float c) { return fmax_(fmax_(a, b), c); }

// float -> uint32 conversion: truncate, saturate, NaN -> 0.
GBR_HD uint32_t f2u_sat(float q) {
  if (!(q > 0.0f)) return 0u;
  if (q >= 4294967296.0f) return 0xFFFFFFFFu;
  return (uint32_t)q;
}
// float -> int32 conversion (convert_int): truncate, saturate, NaN -> 0.
GBR_HD int32_t f2i_sat(float q) {
  if (q != q) return 0;
  if (q >= 2147483648.0f) return 2147483647;
  if (q <= -2147483648.0f) return (-2147483647 - 1);
  return (int32_t)q;
}

// ---- pinned vector helpers (component order as OpenCL evaluates) ----------
GBR_HD f3 add3(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
GBR_HD f3 sub3(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
GBR_HD f3 mul3s(f3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
GBR_HD f3 smul3(float s, f3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
GBR_HD f3 neg3(f3 a) { return mk3(-a.x, -a.y, -a.z); }
GBR_HD float dot3(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
GBR_HD float dot4(f4 a, f4 b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
GBR_HD f3 cross3(f3 a, f3 b) {
  return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
GBR_HD float fast_length3(f3 a) { return fsqrt(dot3(a, a)); }
GBR_HD f3 fast_normalize3(f3 a) {
  float l = fsqrt(dot3(a, a));
  return mk3(fdiv(a.x, l), fdiv(a.y, l), fdiv(a.z, l));
}
GBR_HD f4 fast_normalize4(f4 q) {
  float l = fsqrt(dot4(q, q));
  f4 r; r.x = fdiv(q.x, l); r.y = fdiv(q.y, l); r.z = fdiv(q.z, l); r.w = fdiv(q.w, l);
  return r;
}

// Camera / face rotation with precomputed cosines c and sines s of the Euler
// angles (cl2.cl:220-271, rot; mad -> fmaf).
GBR_HD f3 rot_cs(f3 p, f3 cpos, f3 c, f3 s) {
  f3 rel = sub3(p, cpos);
  float a = fma_(s.z, rel.y, c.z * rel.x);
  float b = fma_(c.y, rel.z, s.y * a);
  float d = fma_(c.z, rel.y, (-s.z) * rel.x);
  f3 r;
  r.x = fma_(c.y, a, (-s.y) * rel.z);
  r.y = fma_(s.x, b, c.x * d);
  r.z = fma_(c.x, b, (-s.x) * d);
  return r;
}

// Inverse camera rotation (cl2.cl:275-348, back_rot; transposed, with mads).
GBR_HD f3 back_rot_cs(f3 p, f3 cpos, f3 c, f3 s) {
  f3 rel = sub3(p, cpos);
  f3 r;
  r.x = c.z * fma_(c.y, rel.x, fma_(s.x, s.y * rel.y, (c.x * s.y) * rel.z)) +
        s.z * (s.x * rel.z - c.x * rel.y);
  r.y = fma_(s.z, c.y * rel.x,
             fma_(fma_(c.x, c.z, (s.x * s.y) * s.z), rel.y,
                  fma_(-s.x, c.z, (c.x * s.y) * s.z) * rel.z));
  r.z = fma_(-s.y, rel.x, c.y * fma_(s.x, rel.y, c.x * rel.z));
  return r;
}

// Quaternion rotation (cl2.cl:350-357, rot_quat).
GBR_HD f3 rot_quat(f3 p, f4 q) {
  q = fast_normalize4(q);
  f3 qv = mk3(q.x, q.y, q.z);
  f3 t = smul3(2.0f, cross3(qv, p));
  return add3(add3(p, smul3(q.w, t)), cross3(qv, t));
}

// rot_quat with the normalisation of q already done (qn = fast_normalize4(q)):
// the same arithmetic, for callers that rotate several points by one q.
GBR_HD f3 rot_quat_n(f3 p, f4 qn) {
  f3 qv = mk3(qn.x, qn.y, qn.z);
  f3 t = smul3(2.0f, cross3(qv, p));
  return add3(add3(p, smul3(qn.w, t)), cross3(qv, t));
}

// Inverse quaternion rotation (cl2.cl:359-370, back_rot_quat).
GBR_HD f3 back_rot_quat(f3 p, f4 q) {
  f4 conj; conj.x = -q.x; conj.y = -q.y; conj.z = -q.z; conj.w = q.w;
  float len_sq = dot4(conj, conj);
  f4 n; n.x = fdiv(conj.x, len_sq); n.y = fdiv(conj.y, len_sq);
  n.z = fdiv(conj.z, len_sq); n.w = fdiv(conj.w, len_sq);
  return rot_quat(p, n);
}

// Perspective projection of a camera-space point (cl2.cl:535-570).
GBR_HD f3 depth_project1(f3 p, float width, float height, float fovc) {
  float k = fdiv(fovc, p.z);
  return mk3(fma_(p.x, k, width / 2.0f), fma_(p.y, k, height / 2.0f), p.z);
}

// Near/far clip (cl2.cl:577-663, generate_new_triangles).  Returns 0, 1 or 2
// triangles in out[0..1].  Vertices with z <= 20 or z > 350000 count as behind
// and are always clipped against z = 20, exactly as the reference does.
GBR_HD int clip_tri(const f3 pts[3], f3 out[2][3]) {
  int ids_behind[3] = {0, 0, 0};
  int n_behind = 0;
  int id_valid = 0;
  for (int i = 0; i < 3; i++) {
    if (pts[i].z <= kDepthCutoff || pts[i].z > kDepthFar) {
      ids_behind[n_behind] = i;
      n_behind++;
    } else {
      id_valid = i;
    }
  }
  if (n_behind > 2) return 0;
  if (n_behind == 0) {
    out[0][0] = pts[0]; out[0][1] = pts[1]; out[0][2] = pts[2];
    return 1;
  }
  int g1, g2, g3;
  if (n_behind == 1) {
    int id = ids_behind[0];
    g1 = id;
    g2 = (id + 1) >= 3 ? id - 2 : id + 1;
    g3 = (id + 2) >= 3 ? id - 1 : id + 2;
  } else {
    g2 = ids_behind[0];
    g3 = ids_behind[1];
    g1 = id_valid;
  }
  // p = v + ((20 - v.z) * (g1 - v)) / (g1.z - v.z), componentwise
  f3 a = pts[g1], b = pts[g2], c = pts[g3];
  float kb = kDepthCutoff - b.z, db = a.z - b.z;
  float kc = kDepthCutoff - c.z, dc = a.z - c.z;
  f3 p1 = mk3(b.x + fdiv(kb * (a.x - b.x), db), b.y + fdiv(kb * (a.y - b.y), db),
              b.z + fdiv(kb * (a.z - b.z), db));
  f3 p2 = mk3(c.x + fdiv(kc * (a.x - c.x), dc), c.y + fdiv(kc * (a.y - c.y), dc),
              c.z + fdiv(kc * (a.z - c.z), dc));
  if (n_behind == 1) {
    out[0][0] = p1; out[0][1] = b; out[0][2] = c;
    out[1][0] = p1; out[1][1] = c; out[1][2] = p2;
    return 2;
  }
  out[0][ids_behind[0]] = p1;
  out[0][ids_behind[1]] = p2;
  out[0][id_valid] = a;
  return 1;
}

// clip_tri with the same arithmetic and outputs, written with selects instead
// of runtime-indexed arrays so that GPU code keeps everything in registers.
GBR_HD f3 sel3(int i, f3 a, f3 b, f3 c) { return i == 0 ? a : (i == 1 ? b : c); }
GBR_HD int clip_tri_reg(f3 a0, f3 a1, f3 a2, f3 o0[3], f3 o1[3]) {
  const bool b0 = a0.z <= kDepthCutoff || a0.z > kDepthFar;
  const bool b1 = a1.z <= kDepthCutoff || a1.z > kDepthFar;
  const bool b2 = a2.z <= kDepthCutoff || a2.z > kDepthFar;
  const int n_behind = (int)b0 + (int)b1 + (int)b2;
  if (n_behind > 2) return 0;
  if (n_behind == 0) {
    o0[0] = a0; o0[1] = a1; o0[2] = a2;
    return 1;
  }
  // the same g1/g2/g3 choice as generate_new_triangles
  int g1, g2, g3, ib0 = 0, ib1 = 0, iv = 0;
  if (n_behind == 1) {
    const int id = b0 ? 0 : (b1 ? 1 : 2);
    g1 = id;
    g2 = (id + 1) >= 3 ? id - 2 : id + 1;
    g3 = (id + 2) >= 3 ? id - 1 : id + 2;
  } else {
    ib0 = b0 ? 0 : 1;
    ib1 = (b0 && b1) ? 1 : 2;
    iv = !b0 ? 0 : (!b1 ? 1 : 2);
    g2 = ib0;
    g3 = ib1;
    g1 = iv;
  }
  const f3 a = sel3(g1, a0, a1, a2), b = sel3(g2, a0, a1, a2), c = sel3(g3, a0, a1, a2);
  float kb = kDepthCutoff - b.z, db = a.z - b.z;
  float kc = kDepthCutoff - c.z, dc = a.z - c.z;
  f3 p1 = mk3(b.x + fdiv(kb * (a.x - b.x), db), b.y + fdiv(kb * (a.y - b.y), db),
              b.z + fdiv(kb * (a.z - b.z), db));
  f3 p2 = mk3(c.x + fdiv(kc * (a.x - c.x), dc), c.y + fdiv(kc * (a.y - c.y), dc),
              c.z + fdiv(kc * (a.z - c.z), dc));
  if (n_behind == 1) {
    o0[0] = p1; o0[1] = b; o0[2] = c;
    o1[0] = p1; o1[1] = c; o1[2] = p2;
    return 2;
  }
  for (int j = 0; j < 3; j++) o0[j] = (j == ib0) ? p1 : ((j == ib1) ? p2 : a);
  return 1;
}

// Backface test on projected vertices (cl2.cl:491-494): 1 when front facing.
GBR_HD int backface_front(f3 p0, f3 p1, f3 p2) {
  return cross3(sub3(p1, p0), sub3(p2, p0)).z < 0.0f;
}

// 1 / (2 * signed area) of the rounded projected triangle (cl2.cl:408-411).
GBR_HD float rconstant(f3 x, f3 y) {
  return rcp(((x.y * y.z + x.x * (y.y - y.z)) - x.z * y.y) + (x.z - x.y) * y.x);
}

// Plane f = A*x + B*y + C through the rounded vertices (cl2.cl:413-418).
GBR_HD void plane_const(f3 f, f3 x, f3 y, float rc, float* A, float* B, float* C) {
  *A = (((f.y * y.z + f.x * (y.y - y.z)) - f.z * y.y) + (f.z - f.y) * y.x) * rc;
  *B = (-(((f.y * x.z + f.x * (x.y - x.z)) - f.z * x.y) + (f.z - f.y) * x.x)) * rc;
  *C = (f.x - (*A) * x.x) - (*B) * y.x;
}

// Bounding box (cl2.cl:420-441, calc_min_max): [minx,maxx) x [miny,maxy) on
// rounded vertices, min-1, clamped to [0, w-1] and [0, h-1].
GBR_HD void bbox4(f3 p0, f3 p1, f3 p2, float width, float height, float mm[4]) {
  float x0 = roundf(p0.x), x1 = roundf(p1.x), x2 = roundf(p2.x);
  float y0 = roundf(p0.y), y1 = roundf(p1.y), y2 = roundf(p2.y);
  mm[0] = clampf_(min3f(x0, x1, x2) - 1.0f, 0.0f, width - 1.0f);
  mm[1] = clampf_(max3f(x0, x1, x2), 0.0f, width - 1.0f);
  mm[2] = clampf_(min3f(y0, y1, y2) - 1.0f, 0.0f, height - 1.0f);
  mm[3] = clampf_(max3f(y0, y1, y2), 0.0f, height - 1.0f);
}

// Edge-function coverage test of integer pixel (px,py) against the rounded
// triangle (cl2.cl:4798-4807, point_in_tri), split into per-triangle
// constants and a per-pixel part with the same evaluation tree.
struct EdgeTest {
  float s0, sa, sb;  // s = ((s0 + sa*px) + sb*py) * sign
  float t0, ta, tb;  // t = ((t0 + ta*px) + tb*py) * sign
  float sign;
  float bound;       // (2.0001f * A) * sign
};
GBR_HD EdgeTest make_edge(float p0x, float p0y, float p1x, float p1y, float p2x, float p2y) {
  EdgeTest e;
  float A = 0.5f * ((((-p1y) * p2x + p0y * ((-p1x) + p2x)) + p0x * (p1y - p2y)) + p1x * p2y);
  e.sign = A < 0.0f ? -1.0f : 1.0f;
  e.s0 = p0y * p2x - p0x * p2y;
  e.sa = p2y - p0y;
  e.sb = p0x - p2x;
  e.t0 = p0x * p1y - p0y * p1x;
  e.ta = p0y - p1y;
  e.tb = p1x - p0x;
  e.bound = (2.0001f * A) * e.sign;
  return e;
}
GBR_HD bool edge_inside(const EdgeTest& e, float px, float py) {
  float s = ((e.s0 + e.sa * px) + e.sb * py) * e.sign;
  float t = ((e.t0 + e.ta * px) + e.tb * py) * e.sign;
  return s > -0.0001f && t > -0.0001f && (s + t) < e.bound;
}

// Quantised depth of a covered pixel (cl2.cl:5113-5115).
GBR_HD uint32_t depth_at(float A, float B, float C, float px, float py) {
  float f = fma_(A, px, fma_(B, py, C));
  return f2u_sat(fdiv(kMulInt, f));
}

// ---- the fragment walk ------------------------------------------------------
// kernel1/kernel2 (cl2.cl:5046-5126) visit the bbox of a triangle in chunks of
// op_size+1 pixels with an incremental float state machine.  Row changes are
// decided by y = floor(fmaf(k, 1.f/w, miny)).  An exhaustive host check over
// every width w <= 3840, top row miny < 2160 and row boundary r*w (r <= 2160 -
// miny) shows the row change is never early and never more than one step
// late; when it is one step late the left-column pixel (minx, miny+r) of that
// row is never visited, except that a fragment starting exactly at
// k = (r+1)*w re-visits (minx, miny+r).  walk_row_late / walk_visits encode
// that rule; the CPU oracle replays the literal state machine instead.
GBR_HD bool walk_row_late(int w, float miny, int r) {
  float iw = fdiv(1.0f, (float)w);
  float y = floorf(fma_((float)(r * w), iw, miny));
  return y != miny + (float)r;
}
// Is relative pixel (j, r) of a w x h bbox visited by the walk with chunk size
// `chunk` (500 for views, 300 for cube faces)?
GBR_HD bool walk_visits(int j, int r, int w, int h, float miny, int chunk) {
  if (j != 0 || r == 0) return true;
  if (!walk_row_late(w, miny, r)) return true;
  int r1 = r + 1;
  return r1 < h && ((r1 * w) % chunk) == 0 && walk_row_late(w, miny, r1);
}

// Largest resolution for which walk_visits is proven exact.
constexpr int kMaxWalkWidth = 3840;
constexpr int kMaxWalkHeight = 2160;

// ---- shading helpers (kernel3 colour path) --------------------------------
// tan(x) for |x| <= pi/2 from the Taylor series of sin and cos about 0
// (degree 15 / 16), in Horner form on x^2, then an IEEE division.  Stands in
// for the vendor tan of the shadow bias (cl2.cl:2606).
GBR_HD float gbr_tanf(float x) {
  float x2 = x * x;
  // sin x = x * (1 - x^2/3! + x^4/5! - ... - x^14/15!)
  float p = -1.0f / 1307674368000.0f;
  p = p * x2 + 1.0f / 6227020800.0f;
  p = p * x2 - 1.0f / 39916800.0f;
  p = p * x2 + 1.0f / 362880.0f;
  p = p * x2 - 1.0f / 5040.0f;
  p = p * x2 + 1.0f / 120.0f;
  p = p * x2 - 1.0f / 6.0f;
  p = p * x2 + 1.0f;
  // cos x = 1 - x^2/2! + x^4/4! - ... + x^16/16!
  float q = 1.0f / 20922789888000.0f;
  q = q * x2 - 1.0f / 87178291200.0f;
  q = q * x2 + 1.0f / 479001600.0f;
  q = q * x2 - 1.0f / 3628800.0f;
  q = q * x2 + 1.0f / 40320.0f;
  q = q * x2 - 1.0f / 720.0f;
  q = q * x2 + 1.0f / 24.0f;
  q = q * x2 - 0.5f;
  q = q * x2 + 1.0f;
  return fdiv(p * x, q);
}

// rational_acos (cl2.cl:2469-2477) with pow(x, 4) as (x*x)*(x*x).
GBR_HD float rational_acos(float x) {
  const float a = -0.939115566365855f;
  const float b = 0.9217841528914573f;
  const float c = -1.2845906244690837f;
  const float d = 0.295624144969963174f;
  float x2 = x * x;
  float x4 = x2 * x2;
  return kPi / 2.0f + fdiv(a * x + ((b * x) * x) * x, (1.0f + (c * x) * x) + d * x4);
}

// sRGB approximations (cl2.cl:5763-5782).
GBR_HD float gamma_fwd(float c) {
  return (0.012522878f * c + (0.682171111f * c) * c) + ((0.305306011f * c) * c) * c;
}
GBR_HD float gamma_inv(float c) {
  float s1 = fsqrt(c);
  float s2 = fsqrt(s1);
  float s3 = fsqrt(s2);
  return (0.585122381f * s1 + 0.783140355f * s2) - 0.368262736f * s3;
}

// fast log2 (cl2.cl:1498-1505).
GBR_HD float log2_approx(float val) {
  union { float f; int32_t i; } u;
  u.f = val;
  float l = (float)(((u.i >> 23) & 255) - 128);
  u.i &= ~(255 << 23);
  u.i += 127 << 23;
  l += ((-0.3358287811f) * u.f + 2.0f) * u.f - 0.65871759316667f;
  return l;
}

// Hashes of the normal jitter and SSAO offset (cl2.cl:1919-1936).
GBR_HD uint32_t wang_hash(uint32_t seed) {
  seed = (seed ^ 61u) ^ (seed >> 16);
  seed *= 9u;
  seed = seed ^ (seed >> 4);
  seed *= 0x27d4eb2du;
  seed = seed ^ (seed >> 15);
  return seed;
}
GBR_HD uint32_t rand_xorshift(uint32_t s) {
  s ^= (s << 13);
  s ^= (s >> 17);
  s ^= (s << 5);
  return s;
}

// Cube face of a point around a light (cl2.cl:1745-1790).
GBR_HD int ret_cubeface(f3 p, f3 l) {
  f3 rel = sub3(p, l);
  float ax = fabsf(rel.x), ay = fabsf(rel.y), az = fabsf(rel.z);
  if (ax >= ay && ax >= az) return rel.x < 0.0f ? 4 : 5;
  if (ay > ax && ay >= az) return rel.y < 0.0f ? 1 : 3;
  if (az > ax && az > ay) {
    if (rel.z < 0.0f) return 2;
  }
  return 0;
}

// Barycentrics (cl2.cl:5372-5384).
GBR_HD void barycentric(f3 p, f3 a, f3 b, f3 c, float* u, float* v, float* w) {
  f3 v0 = sub3(b, a), v1 = sub3(c, a), v2 = sub3(p, a);
  float d00 = dot3(v0, v0), d01 = dot3(v0, v1), d11 = dot3(v1, v1);
  float d20 = dot3(v2, v0), d21 = dot3(v2, v1);
  float denom = d00 * d11 - d01 * d01;
  *v = fdiv(d11 * d20 - d01 * d21, denom);
  *w = fdiv(d00 * d21 - d01 * d20, denom);
  *u = (1.0f - *v) - *w;
}

// Mirror wrap of texture coordinates (cl2.cl:1457-1468).
GBR_HD f2 texture_mod(f2 v) {
  v.x = v.x >= 1.0f ? 1.0f - (v.x - floorf(v.x)) : v.x;
  v.y = v.y >= 1.0f ? 1.0f - (v.y - floorf(v.y)) : v.y;
  v.x = v.x < 0.0f ? (1.0f + fabsf(v.x)) - fabsf(floorf(v.x)) : v.x;
  v.y = v.y < 0.0f ? (1.0f + fabsf(v.y)) - fabsf(floorf(v.y)) : v.y;
  return v;
}

// RGBA8 quantisation of a colour channel: round(clamp(v,0,1) * 255).
GBR_HD uint32_t quant8(float v) {
  v = clampf_(v, 0.0f, 1.0f);
  return (uint32_t)floorf(v * 255.0f + 0.5f);
}

// ---- post passes -----------------------------------------------------------
// fdiv(t, 255.0f) and fdiv(t, 65535.0f) for the integers t of a byte and of a
// 16-bit word, without a division: the product q = t * r with r = RN(1 / d),
// corrected once by its exact residual, q + (t - d q) r (Markstein's
// correction step, P. Markstein, "Computation of elementary functions on the
// IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990).  Equal to
// the correctly rounded quotient for every t of the range, checked
// exhaustively against the IEEE division (tests/cpp/div_const_check.cpp);
// the post passes' GPU parity tests compare their outputs bit for bit.
GBR_HD float u8_over_255(uint32_t t) {
  const float x = (float)t, r = 0x1.010102p-8f;  // RN(1 / 255)
  const float q = x * r;
  return fma_(fma_(-255.0f, q, x), r, q);
}
GBR_HD float u16_over_65535(uint32_t t) {
  const float x = (float)t, r = 0x1.0001p-16f;  // RN(1 / 65535)
  const float q = x * r;
  return fma_(fma_(-65535.0f, q, x), r, q);
}

// Pixel p of an RGBA8 image as one word, R in bits 0-7 (the image is 4-byte
// aligned: the entry points check it; on the device one 32-bit load).
GBR_HD uint32_t rgba8_word(const uint8_t* img, size_t p) {
#if defined(__CUDA_ARCH__)
  return __ldg(reinterpret_cast<const uint32_t*>(img) + p);
#else
  const uint8_t* q = img + 4 * p;
  return (uint32_t)q[0] | ((uint32_t)q[1] << 8) | ((uint32_t)q[2] << 16) | ((uint32_t)q[3] << 24);
#endif
}

// Bilinear read of an RGBA8 image at unnormalised float coordinates with
// clamp-to-edge: OpenCL 1.2 section 8.2's linear filter (i0 = floor(x - 0.5),
// a = frac(x - 0.5)) with float weights, the device precision pinned.  conv
// maps a channel byte c to fdiv(c, 255.0f).
struct ByteOver255 {
  GBR_HD float operator()(uint32_t c) const { return u8_over_255(c); }
};
template <typename Conv>
GBR_HD f4 read_linear_rgba8_with(const uint8_t* img, int W, int H, float cx, float cy, Conv conv) {
  const float u = cx - 0.5f, v = cy - 0.5f;
  const float fi = floorf(u), fj = floorf(v);
  const float a = u - fi, b = v - fj;
  const int i0 = (int)fi, j0 = (int)fj;
  const int xs[2] = {i0 < 0 ? 0 : (i0 >= W ? W - 1 : i0), i0 + 1 < 0 ? 0 : (i0 + 1 >= W ? W - 1 : i0 + 1)};
  const int ys[2] = {j0 < 0 ? 0 : (j0 >= H ? H - 1 : j0), j0 + 1 < 0 ? 0 : (j0 + 1 >= H ? H - 1 : j0 + 1)};
  float t[4][4];
  for (int k = 0; k < 4; k++) {
    const uint32_t w = rgba8_word(img, (size_t)ys[k >> 1] * W + xs[k & 1]);
    for (int c = 0; c < 4; c++) t[k][c] = conv((w >> (8 * c)) & 0xFFu);
  }
  f4 r;
  float* rc = &r.x;
  for (int c = 0; c < 4; c++)
    rc[c] = ((((1.0f - a) * (1.0f - b)) * t[0][c] + (a * (1.0f - b)) * t[1][c]) + ((1.0f - a) * b) * t[2][c]) +
            (a * b) * t[3][c];
  return r;
}
GBR_HD f4 read_linear_rgba8(const uint8_t* img, int W, int H, float cx, float cy) {
  return read_linear_rgba8_with(img, W, H, cx, cy, ByteOver255());
}

// short_to_float + decode_normal (cl2.cl:5597-5642): the ushort2 of the
// normals buffer back to a unit vector; xy carry the direction, their length
// the z component.
GBR_HD f3 decode_normal(uint32_t sx, uint32_t sy) {
  const float vx = u16_over_65535(sx) * 2.0f - 1.0f;  // fdiv(sx, 65535.0f)
  const float vy = u16_over_65535(sy) * 2.0f - 1.0f;
  const float z = (vx * vx + vy * vy) * 2.0f - 1.0f;
  const float l = fsqrt(vx * vx + vy * vy);
  const float g = fsqrt(fmax_(1.0f - z * z, 0.0f));
  return mk3(fdiv(vx, l) * g, fdiv(vy, l) * g, z);
}

// do_pseudo_aa's edge angle: cos(20.f * 2 * M_PI / 360.f) with the float
// M_PI of cl2.cl, the argument rounded in float and the cosine rounded from
// double (0.9396926f).
constexpr float kAACos = 0x1.e11f64p-1f;

// Six cube-face Euler rotations (cl2.cl:4487-4511, 2538-2558) as float
// angles; their cosines and sines are rounded from double on the host.
GBR_HD f3 face_angles(int face) {
  switch (face) {
    case 1: return mk3(kPi / 2.0f, 0.0f, 0.0f);
    case 2: return mk3(0.0f, kPi, 0.0f);
    case 3: return mk3(3.0f * kPi / 2.0f, 0.0f, 0.0f);
    case 4: return mk3(0.0f, 3.0f * kPi / 2.0f, 0.0f);
    case 5: return mk3(0.0f, kPi / 2.0f, 0.0f);
    default: return mk3(0.0f, 0.0f, 0.0f);
  }
}

}  // namespace gbr
