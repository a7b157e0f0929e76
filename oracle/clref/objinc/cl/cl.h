// cl/cl.h stand-in — TEST INFRASTRUCTURE ONLY: the OpenCL host vector types
// that the reference's vec.hpp, vertex.hpp and obj_load.cpp use, laid out as
// the OpenCL headers lay them out (an array member s first, then x, y, z, w),
// so that the reference's OBJ loader compiles on the host without OpenCL.
#pragma once

#include <cstdint>

typedef float cl_float;
typedef uint32_t cl_uint;
typedef int32_t cl_int;
typedef uint16_t cl_ushort;
typedef uint8_t cl_uchar;

typedef union {
  cl_float s[4];
  struct {
    cl_float x, y, z, w;
  };
} cl_float4;

typedef union {
  cl_float s[2];
  struct {
    cl_float x, y;
  };
} cl_float2;

typedef union {
  cl_ushort s[2];
  struct {
    cl_ushort x, y;
  };
} cl_ushort2;
