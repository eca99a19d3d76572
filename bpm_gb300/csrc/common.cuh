// Shared helpers of the bpm_gb300 CUDA library: error reporting, launch accounting,
// complex arithmetic on float2.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include <atomic>
#include <string>

#include "../../include/bpm_gb300.h"

namespace bpmgb {

// ---- error reporting (thread-local text, returned by bpm_last_error) ------------------
void set_error(const std::string& msg);
void clear_error();
int cuda_fail(cudaError_t e, const char* what);

// number of kernels launched by this library (bpm_launch_count)
extern std::atomic<unsigned long long> g_launches;
inline void count_launch(unsigned long long n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

#define BPM_CUDA_TRY(call)                                   \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return ::bpmgb::cuda_fail(e_, #call); \
  } while (0)

#define BPM_LAUNCH_CHECK(what)                               \
  do {                                                       \
    cudaError_t e_ = cudaGetLastError();                     \
    if (e_ != cudaSuccess) return ::bpmgb::cuda_fail(e_, what); \
    ::bpmgb::count_launch();                                 \
  } while (0)

// ---- complex helpers -------------------------------------------------------------------
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float cabs2(float2 a) { return a.x * a.x + a.y * a.y; }

inline bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

inline size_t align256(size_t n) { return (n + 255) & ~size_t(255); }

}  // namespace bpmgb
