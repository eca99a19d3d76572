/*
 * Test infrastructure only (oracle). Maps the OpenCL C dialect used by the
 * reference kernels (bpm/bpm/kernels/bpm_3d_kernels.cl, bpm/psf/kernels/psf_debye.cl,
 * bpm/psf/kernels/bessel.cl) onto host C++ so the kernel bodies compile unchanged
 * from where they lie. Work-item ids come from thread-local variables that the
 * driver loops in ref_*.cpp set before each call. Floating-point contraction is
 * disabled by the build recipe so that every FP32 operation rounds as written.
 */
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>

#include "pyopencl-complex.h"

using std::cos; using std::sin; using std::sqrt; using std::fabs; using std::atan2;
using std::exp; using std::hypot;

#define __kernel
#define __global
#define __constant const
#define __read_only
typedef unsigned int uint;

/* work-item geometry, set by the host-side driver loops */
extern thread_local size_t shim_gid[3];
extern thread_local size_t shim_gsize[3];
static inline size_t get_global_id(int d) { return shim_gid[d]; }
static inline size_t get_global_size(int d) { return shim_gsize[d]; }

static inline int min(int a, int b) { return a < b ? a : b; }

/* binary16 storage with vload_half as in OpenCL */
typedef uint16_t half;
static inline float shim_half_to_float(uint16_t h) {
  uint32_t sign = (uint32_t)(h >> 15) << 31;
  int exp = (h >> 10) & 0x1f;
  uint32_t mant = h & 0x3ff;
  uint32_t bits;
  if (exp == 0) {
    if (mant == 0) {
      bits = sign;
    } else {                       /* subnormal half -> normal float */
      int e = -1;
      do { mant <<= 1; e++; } while ((mant & 0x400) == 0);
      mant &= 0x3ff;
      bits = sign | ((uint32_t)(127 - 15 - e) << 23) | (mant << 13);
    }
  } else if (exp == 31) {
    bits = sign | 0x7f800000u | (mant << 13);
  } else {
    bits = sign | ((uint32_t)(exp - 15 + 127) << 23) | (mant << 13);
  }
  float f;
  std::memcpy(&f, &bits, 4);
  return f;
}
static inline float vload_half(size_t off, const half* p) { return shim_half_to_float(p[off]); }

/* vector types: float4 arithmetic as OpenCL defines it for the kernels the oracle runs
 * (bpm_3d_spheres.cl:fill_dn uses r - r2 and length()); the OpenCL vector literal
 * (float4)(a, b, c, d) is rewritten to make_float4(a, b, c, d) by the build recipe. The
 * scalar-broadcast constructor serves image kernels the oracle never calls. */
struct float2 { float x, y; float2() : x(0), y(0) {} };
struct float4 {
  float x, y, z, w; float2 xy;
  float4() : x(0), y(0), z(0), w(0) {}
  template <typename T> float4(T) : x(0), y(0), z(0), w(0) {}
};
static inline float4 make_float4(float a, float b, float c, float d) {
  float4 r; r.x = a; r.y = b; r.z = c; r.w = d; return r;
}
static inline float4 operator-(const float4& a, const float4& b) {
  return make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w);
}
static inline float length(const float4& a) {
  float s = a.x * a.x;
  s = s + a.y * a.y;
  s = s + a.z * a.z;
  s = s + a.w * a.w;
  return std::sqrt(s);
}
typedef int sampler_t;
struct image3d_t { int unused; };
#define CLK_NORMALIZED_COORDS_FALSE 0
#define CLK_NORMALIZED_COORDS_TRUE 0
#define CLK_ADDRESS_CLAMP_TO_EDGE 0
#define CLK_FILTER_NEAREST 0
#define CLK_FILTER_LINEAR 0
static inline float4 read_imagef(image3d_t, sampler_t, float4) { return float4(0); }
