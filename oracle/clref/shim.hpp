// shim.hpp — TEST INFRASTRUCTURE ONLY: just enough OpenCL C 1.2 for the
// reference's triangle-pipeline kernels (extracted from cl2.cl by extract.py)
// to compile as C++ on the host and run as the parity pin of the oracle.
//
// Vector types with the swizzles those kernels use, the builtins they call,
// images, atomics and work-item ids.  Every implementation-defined builtin
// follows the determinism contract of openclrenderer_gb300/csrc/gbr_math.h
// (the same one the CUDA pipeline and the oracle restatement use):
// mad = fmaf; native_divide/recip, fast_normalize/length = IEEE; native_sin/cos
// = double precision rounded to float; pow(x, n) for small integer n by
// repeated multiplication; tan = gbr_tanf; min/max = IEEE minNum/maxNum;
// float->int conversions truncate and saturate.  Compile with
// -ffp-contract=off -fno-strict-aliasing -Wno-narrowing.
#pragma once

#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>

#include "../../openclrenderer_gb300/csrc/gbr_math.h"

#define __kernel
#define __global
#define __local
#define __constant const
#define __private
#define __read_only
#define __write_only
#define global
#define kernel

#ifndef UINT_MAX
#define UINT_MAX 0xffffffffu
#endif

// Everything OpenCL lives in namespace clref, so that its scalar overloads
// (tan, pow, round, min, ...) hide the C library's for the extracted kernels.
namespace clref {

typedef uint32_t uint;
typedef uint8_t uchar;
typedef uint16_t ushort;

// ---- swizzle proxies --------------------------------------------------------
// A proxy overlays the storage of its vector (union member) and reads or
// writes the selected components.
template <class V, class T, int NS, int... I>
struct swz {
  T v[NS];
  operator V() const { return V(v[I]...); }
  swz& operator=(const V& o) {
    const int idx[] = {I...};
    T tmp[sizeof...(I)];
    for (int k = 0; k < (int)sizeof...(I); k++) tmp[k] = o.s[k];
    for (int k = 0; k < (int)sizeof...(I); k++) v[idx[k]] = tmp[k];
    return *this;
  }
  swz& operator=(const swz& o) { return *this = V(o); }
  swz& operator*=(T s) {
    const int idx[] = {I...};
    for (int k = 0; k < (int)sizeof...(I); k++) v[idx[k]] = v[idx[k]] * s;
    return *this;
  }
  swz& operator/=(T s) {
    const int idx[] = {I...};
    for (int k = 0; k < (int)sizeof...(I); k++) v[idx[k]] = v[idx[k]] / s;
    return *this;
  }
  swz& operator+=(const V& o) {
    const int idx[] = {I...};
    for (int k = 0; k < (int)sizeof...(I); k++) v[idx[k]] = v[idx[k]] + o.s[k];
    return *this;
  }
};

struct float2;
struct float3;
struct float4;
struct int2;

struct alignas(8) float2 {
  union {
    struct { float x, y; };
    float s[2];
    swz<float2, float, 2, 0, 1> xy;
    swz<float4, float, 2, 0, 0, 1, 1> xxyy;
  };
  float2() : x(0), y(0) {}
  float2(float a) : x(a), y(a) {}
  float2(float a, float b) : x(a), y(b) {}
  float2(const float2& o) { memcpy(s, o.s, sizeof s); }
  float2& operator=(const float2& o) { memcpy(s, o.s, sizeof s); return *this; }
};

struct alignas(16) float3 {
  union {
    struct { float x, y, z; };
    float s[3];
    swz<float2, float, 3, 0, 1> xy;
    swz<float3, float, 3, 0, 1, 2> xyz;
    swz<float4, float, 3, 0, 1, 2, 2> xyzz;
  };
  float3() : x(0), y(0), z(0) {}
  float3(float a) : x(a), y(a), z(a) {}
  float3(float a, float b, float c) : x(a), y(b), z(c) {}
  float3(float2 a, float c) : x(a.x), y(a.y), z(c) {}
  float3(const float3& o) { memcpy(s, o.s, sizeof s); }
  float3& operator=(const float3& o) { memcpy(s, o.s, sizeof s); return *this; }
};

struct alignas(16) float4 {
  union {
    struct { float x, y, z, w; };
    float s[4];
    swz<float2, float, 4, 0, 1> xy;
    swz<float3, float, 4, 0, 1, 2> xyz;
    swz<float4, float, 4, 0, 1, 2, 2> xyzz;
  };
  float4() : x(0), y(0), z(0), w(0) {}
  float4(float a) : x(a), y(a), z(a), w(a) {}
  float4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
  float4(float3 a, float d) : x(a.x), y(a.y), z(a.z), w(d) {}
  float4(const float4& o) { memcpy(s, o.s, sizeof s); }
  float4& operator=(const float4& o) { memcpy(s, o.s, sizeof s); return *this; }
};

struct alignas(8) int2 {
  union {
    struct { int x, y; };
    int s[2];
  };
  int2() : x(0), y(0) {}
  int2(int a) : x(a), y(a) {}
  int2(int a, int b) : x(a), y(b) {}
  int2(const int2& o) { memcpy(s, o.s, sizeof s); }
  int2& operator=(const int2& o) { memcpy(s, o.s, sizeof s); return *this; }
};
inline int2 operator+(int2 a, int2 b) { return int2(a.x + b.x, a.y + b.y); }
// vector relational operators (-1 where true) and any() (cl2.cl screenspace_godrays)
inline int2 operator<(float2 a, float b) { return int2(a.x < b ? -1 : 0, a.y < b ? -1 : 0); }
inline int2 operator>=(float2 a, float2 b) { return int2(a.x >= b.x ? -1 : 0, a.y >= b.y ? -1 : 0); }
inline int any(int2 v) { return (v.x < 0 || v.y < 0) ? 1 : 0; }

struct alignas(16) int4 {
  union {
    struct { int x, y, z, w; };
    int s[4];
    swz<int2, int, 4, 0, 1> xy;
  };
  int4() : x(0), y(0), z(0), w(0) {}
  int4(int a, int b, int c, int d) : x(a), y(b), z(c), w(d) {}
  int4(const int4& o) { memcpy(s, o.s, sizeof s); }
  int4& operator=(const int4& o) { memcpy(s, o.s, sizeof s); return *this; }
};

struct alignas(16) uint4 {
  uint x, y, z, w;
  uint4() : x(0), y(0), z(0), w(0) {}
  uint4(uint a) : x(a), y(a), z(a), w(a) {}
  uint4(uint a, uint b, uint c, uint d) : x(a), y(b), z(c), w(d) {}
};

struct alignas(4) uchar4 {
  uchar x, y, z, w;
};
struct alignas(2) uchar2 {
  uchar x, y;
};
struct alignas(4) ushort2 {
  ushort x, y;
};

// ---- arithmetic -------------------------------------------------------------
#define GBR_VEC_OPS(V, N)                                                                   \
  inline V operator+(V a, V b) { V r; for (int i = 0; i < N; i++) r.s[i] = a.s[i] + b.s[i]; return r; } \
  inline V operator-(V a, V b) { V r; for (int i = 0; i < N; i++) r.s[i] = a.s[i] - b.s[i]; return r; } \
  inline V operator*(V a, V b) { V r; for (int i = 0; i < N; i++) r.s[i] = a.s[i] * b.s[i]; return r; } \
  inline V operator/(V a, V b) { V r; for (int i = 0; i < N; i++) r.s[i] = a.s[i] / b.s[i]; return r; } \
  inline V operator+(V a, float b) { V r; for (int i = 0; i < N; i++) r.s[i] = a.s[i] + b; return r; }  \
  inline V operator-(V a, float b) { V r; for (int i = 0; i < N; i++) r.s[i] = a.s[i] - b; return r; }  \
  inline V operator*(V a, float b) { V r; for (int i = 0; i < N; i++) r.s[i] = a.s[i] * b; return r; }  \
  inline V operator/(V a, float b) { V r; for (int i = 0; i < N; i++) r.s[i] = a.s[i] / b; return r; }  \
  inline V operator+(float a, V b) { V r; for (int i = 0; i < N; i++) r.s[i] = a + b.s[i]; return r; }  \
  inline V operator-(float a, V b) { V r; for (int i = 0; i < N; i++) r.s[i] = a - b.s[i]; return r; }  \
  inline V operator*(float a, V b) { V r; for (int i = 0; i < N; i++) r.s[i] = a * b.s[i]; return r; }  \
  inline V operator/(float a, V b) { V r; for (int i = 0; i < N; i++) r.s[i] = a / b.s[i]; return r; }  \
  inline V operator-(V a) { V r; for (int i = 0; i < N; i++) r.s[i] = -a.s[i]; return r; }              \
  inline V& operator+=(V& a, V b) { a = a + b; return a; }                                              \
  inline V& operator-=(V& a, V b) { a = a - b; return a; }                                              \
  inline V& operator*=(V& a, V b) { a = a * b; return a; }                                              \
  inline V& operator/=(V& a, V b) { a = a / b; return a; }                                              \
  inline V& operator+=(V& a, float b) { a = a + b; return a; }                                          \
  inline V& operator-=(V& a, float b) { a = a - b; return a; }                                          \
  inline V& operator*=(V& a, float b) { a = a * b; return a; }                                          \
  inline V& operator/=(V& a, float b) { a = a / b; return a; }                                          \
  inline float dot(V a, V b) { float r = a.s[0] * b.s[0]; for (int i = 1; i < N; i++) r = r + a.s[i] * b.s[i]; return r; } \
  inline V mad(V a, V b, V c) { V r; for (int i = 0; i < N; i++) r.s[i] = fmaf(a.s[i], b.s[i], c.s[i]); return r; } \
  inline V mad(V a, float b, V c) { V r; for (int i = 0; i < N; i++) r.s[i] = fmaf(a.s[i], b, c.s[i]); return r; } \
  inline V round(V a) { V r; for (int i = 0; i < N; i++) r.s[i] = roundf(a.s[i]); return r; }        \
  inline V floor(V a) { V r; for (int i = 0; i < N; i++) r.s[i] = floorf(a.s[i]); return r; }        \
  inline V fabs(V a) { V r; for (int i = 0; i < N; i++) r.s[i] = fabsf(a.s[i]); return r; }          \
  inline V sqrt(V a) { V r; for (int i = 0; i < N; i++) r.s[i] = sqrtf(a.s[i]); return r; }          \
  inline V fmod(V a, float b) { V r; for (int i = 0; i < N; i++) r.s[i] = fmodf(a.s[i], b); return r; } \
  inline V clamp(V a, float lo, float hi) { V r; for (int i = 0; i < N; i++) r.s[i] = fminf(fmaxf(a.s[i], lo), hi); return r; } \
  inline V clamp(V a, float lo, V hi) { V r; for (int i = 0; i < N; i++) r.s[i] = fminf(fmaxf(a.s[i], lo), hi.s[i]); return r; } \
  inline V clamp(V a, V lo, V hi) { V r; for (int i = 0; i < N; i++) r.s[i] = fminf(fmaxf(a.s[i], lo.s[i]), hi.s[i]); return r; } \
  inline V max(V a, float b) { V r; for (int i = 0; i < N; i++) r.s[i] = fmaxf(a.s[i], b); return r; } \
  inline V min(V a, float b) { V r; for (int i = 0; i < N; i++) r.s[i] = fminf(a.s[i], b); return r; } \
  inline V native_recip(V a) { V r; for (int i = 0; i < N; i++) r.s[i] = 1.0f / a.s[i]; return r; }    \
  inline V native_divide(V a, float b) { V r; for (int i = 0; i < N; i++) r.s[i] = a.s[i] / b; return r; } \
  inline V native_divide(V a, V b) { V r; for (int i = 0; i < N; i++) r.s[i] = a.s[i] / b.s[i]; return r; } \
  inline V mix(V a, V b, float t) { V r; for (int i = 0; i < N; i++) r.s[i] = a.s[i] + (b.s[i] - a.s[i]) * t; return r; } \
  inline V native_cos(V a) { V r; for (int i = 0; i < N; i++) r.s[i] = (float)std::cos((double)a.s[i]); return r; } \
  inline V native_sin(V a) { V r; for (int i = 0; i < N; i++) r.s[i] = (float)std::sin((double)a.s[i]); return r; } \
  inline float fast_length(V a) { return sqrtf(dot(a, a)); }                                          \
  inline V fast_normalize(V a) { float l = sqrtf(dot(a, a)); V r; for (int i = 0; i < N; i++) r.s[i] = a.s[i] / l; return r; } \
  inline V normalize(V a) { float l = sqrtf(dot(a, a)); V r; for (int i = 0; i < N; i++) r.s[i] = a.s[i] / l; return r; }

GBR_VEC_OPS(float2, 2)
GBR_VEC_OPS(float3, 3)
GBR_VEC_OPS(float4, 4)
#undef GBR_VEC_OPS

inline float3 cross(float3 a, float3 b) {
  return float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// ---- scalar builtins ----------------------------------------------------------
inline float mad(float a, float b, float c) { return fmaf(a, b, c); }
inline float native_divide(float a, float b) { return a / b; }
inline float native_recip(float a) { return 1.0f / a; }
inline float native_exp(float a) { return expf(a); }
inline float native_powr(float a, float b) { return powf(a, b); }
inline float clamp(float a, float lo, float hi) { return fminf(fmaxf(a, lo), hi); }
inline float max(float a, float b) { return fmaxf(a, b); }
inline float min(float a, float b) { return fminf(a, b); }
inline int max(int a, int b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline float round(float a) { return roundf(a); }
inline float floor(float a) { return floorf(a); }
inline float ceil(float a) { return ceilf(a); }
inline float fabs(float a) { return fabsf(a); }
inline float sqrt(float a) { return sqrtf(a); }
inline float fmod(float a, float b) { return fmodf(a, b); }
inline float tan(float a) { return gbr::gbr_tanf(a); }
// pow with the small integer exponents cl2.cl uses, by repeated multiplication
inline float pow(float x, float y) {
  if (y == 1.0f) return x;
  if (y == 2.0f) return x * x;
  if (y == 3.0f) return (x * x) * x;
  if (y == 4.0f) return (x * x) * (x * x);
  return powf(x, y);
}
inline int mul24(int a, int b) { return a * b; }
inline float as_float(uint u) { float f; memcpy(&f, &u, 4); return f; }
inline int as_int(float f) { int i; memcpy(&i, &f, 4); return i; }

inline int gbr_ref_f2i(float q) { return gbr::f2i_sat(q); }
inline uint gbr_ref_f2u(float q) { return gbr::f2u_sat(q); }
inline int2 convert_int2(float2 a) { return int2(gbr_ref_f2i(a.x), gbr_ref_f2i(a.y)); }
inline uint4 convert_uint4(float4 a) { return uint4(gbr_ref_f2u(a.x), gbr_ref_f2u(a.y), gbr_ref_f2u(a.z), gbr_ref_f2u(a.w)); }
inline uint4 convert_uint4(uchar4 a) { return uint4(a.x, a.y, a.z, a.w); }
inline uchar4 convert_uchar4(uint4 a) { return uchar4{(uchar)a.x, (uchar)a.y, (uchar)a.z, (uchar)a.w}; }
inline float4 convert_float4(uint4 a) { return float4((float)a.x, (float)a.y, (float)a.z, (float)a.w); }
inline float2 convert_float2(int2 a) { return float2((float)a.x, (float)a.y); }
inline float2 convert_float2(ushort2 a) { return float2((float)a.x, (float)a.y); }
inline ushort2 convert_ushort2(float2 a) {
  return ushort2{(ushort)(gbr_ref_f2u(a.x) > 65535u ? 65535u : gbr_ref_f2u(a.x)),
                 (ushort)(gbr_ref_f2u(a.y) > 65535u ? 65535u : gbr_ref_f2u(a.y))};
}

// ---- work items, barriers, atomics -----------------------------------------------
extern thread_local size_t gbr_ref_gid[2];
inline size_t get_global_id(int d) { return gbr_ref_gid[d]; }
#define CLK_GLOBAL_MEM_FENCE 1
#define CLK_LOCAL_MEM_FENCE 2
inline void barrier(int) {}
inline uint atomic_add(uint* p, uint v) { return __atomic_fetch_add(p, v, __ATOMIC_RELAXED); }
inline uint atomic_add(uint* p, int v) { return atomic_add(p, (uint)v); }
inline uint atomic_add(uint* p, float v) { return atomic_add(p, (uint)v); }
inline uint atomic_min(uint* p, uint v) {
  uint cur = __atomic_load_n(p, __ATOMIC_RELAXED);
  while (v < cur && !__atomic_compare_exchange_n(p, &cur, v, true, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
  }
  return cur;
}

// ---- images ---------------------------------------------------------------------
// kind 0: R32UI (the id buffer; writes keep the minimum), kind 1: RGBA UNORM8
// (read_imagef returns c/255), kind 2: RGBA float written by write_imagef.
struct image2d_t {
  void* data;
  int w, h;
  int kind;
};
typedef int sampler_t;
#define CLK_NORMALIZED_COORDS_FALSE 0
#define CLK_ADDRESS_NONE 0
#define CLK_FILTER_NEAREST 0
#define CLK_ADDRESS_CLAMP_TO_EDGE 2
#define CLK_FILTER_LINEAR 16
inline int2 get_image_dim(image2d_t im) { return int2(im.w, im.h); }
inline uint4 read_imageui(image2d_t im, sampler_t, int2 c) {
  return uint4(static_cast<uint*>(im.data)[(size_t)c.y * im.w + c.x], 0, 0, 1);
}
inline void write_imageui(image2d_t im, int2 c, uint4 v) {
  atomic_min(&static_cast<uint*>(im.data)[(size_t)c.y * im.w + c.x], v.x);
}
inline float4 read_imagef(image2d_t im, sampler_t, int2 c) {
  const uchar* p = static_cast<uchar*>(im.data) + ((size_t)c.y * im.w + c.x) * 4;
  return float4(p[0] / 255.0f, p[1] / 255.0f, p[2] / 255.0f, p[3] / 255.0f);
}
// Unnormalised float coordinates: nearest, or (CLK_FILTER_LINEAR) bilinear
// with clamp-to-edge as OpenCL 1.2 section 8.2 defines it -- i0 = floor(x -
// 0.5), a = frac(x - 0.5) -- with the weights in float (the precision OpenCL
// leaves to the device, pinned).
inline float4 read_imagef(image2d_t im, sampler_t s, float2 c) {
  if (!(s & CLK_FILTER_LINEAR)) return read_imagef(im, s, int2((int)floorf(c.x), (int)floorf(c.y)));
  const float u = c.x - 0.5f, v = c.y - 0.5f;
  const float fi = floorf(u), fj = floorf(v);
  const float a = u - fi, b = v - fj;
  auto cl = [](int i, int n) { return i < 0 ? 0 : (i >= n ? n - 1 : i); };
  const int i0 = cl((int)fi, im.w), i1 = cl((int)fi + 1, im.w), j0 = cl((int)fj, im.h), j1 = cl((int)fj + 1, im.h);
  const float4 t00 = read_imagef(im, s, int2(i0, j0)), t10 = read_imagef(im, s, int2(i1, j0));
  const float4 t01 = read_imagef(im, s, int2(i0, j1)), t11 = read_imagef(im, s, int2(i1, j1));
  float4 r;
  for (int k = 0; k < 4; k++)
    r.s[k] = ((((1.0f - a) * (1.0f - b)) * t00.s[k] + (a * (1.0f - b)) * t10.s[k]) + ((1.0f - a) * b) * t01.s[k]) +
             (a * b) * t11.s[k];
  return r;
}
inline void write_imagef(image2d_t im, int2 c, float4 v) {
  if (!im.data) return;
  memcpy(static_cast<float*>(im.data) + ((size_t)c.y * im.w + c.x) * 4, v.s, 16);
}

// ---- per-render constants (-D SCREENWIDTH / SCREENHEIGHT / FOV_CONST) ----------
extern int gbr_ref_W, gbr_ref_H;
extern float gbr_ref_FOV;

}  // namespace clref
