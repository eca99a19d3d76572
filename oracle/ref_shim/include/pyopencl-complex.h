/*
 * Test infrastructure only (oracle). A minimal, project-written stand-in for the
 * single-precision complex helpers that the reference's OpenCL kernels include as
 * <pyopencl-complex.h>. It lets those kernel sources compile as C++ on the host so
 * that the oracle can run the reference's own arithmetic. The semantics follow the
 * published pyopencl complex API (cfloat_new/add/sub/mul/rmul/mulr/divider/abs/exp/
 * conj); the third-party header itself is not used or copied.
 */
#pragma once
#include <cmath>

typedef struct cfloat_t {
  union { float x; float real; };
  union { float y; float imag; };
} cfloat_t;

static inline cfloat_t cfloat_new(float re, float im) {
  cfloat_t r; r.x = re; r.y = im; return r;
}
static inline cfloat_t cfloat_add(cfloat_t a, cfloat_t b) { return cfloat_new(a.x + b.x, a.y + b.y); }
static inline cfloat_t cfloat_sub(cfloat_t a, cfloat_t b) { return cfloat_new(a.x - b.x, a.y - b.y); }
static inline cfloat_t cfloat_mul(cfloat_t a, cfloat_t b) {
  return cfloat_new(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
static inline cfloat_t cfloat_rmul(float r, cfloat_t a) { return cfloat_new(r * a.x, r * a.y); }
static inline cfloat_t cfloat_mulr(cfloat_t a, float r) { return cfloat_new(a.x * r, a.y * r); }
static inline cfloat_t cfloat_divider(cfloat_t a, float r) { return cfloat_new(a.x / r, a.y / r); }
static inline cfloat_t cfloat_conj(cfloat_t a) { return cfloat_new(a.x, -a.y); }
static inline float cfloat_abs(cfloat_t a) { return std::hypot(a.x, a.y); }
static inline cfloat_t cfloat_exp(cfloat_t a) {
  float e = std::exp(a.x);
  return cfloat_new(e * std::cos(a.y), e * std::sin(a.y));
}
static inline cfloat_t cfloat_divide(cfloat_t a, cfloat_t b) {
  float d = b.x * b.x + b.y * b.y;
  return cfloat_new((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
