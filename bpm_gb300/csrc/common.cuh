// Shared helpers of the bpm_gb300 CUDA library: error reporting, launch accounting,
// complex arithmetic on float2.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include <atomic>
#include <mutex>
#include <string>
#include <utility>

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
// Every multiply-add is written as an explicit fmaf: left implicit, the compiler may fuse
// either product of a*b - c*d depending on the surrounding code, so the same formula could
// round differently in two kernels. Spelled out, every kernel gets the same bits.
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -(a.y * b.y)), fmaf(a.x, b.y, a.y * b.x));
}
// Complex add and subtract as one packed two-lane FP32 instruction (add/sub.rn.f32x2,
// sm_100 and later): each component is the IEEE single-precision sum, the same bits as two
// scalar adds, in half the issued instructions.
__device__ __forceinline__ unsigned long long f2_pack(float2 a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
__device__ __forceinline__ float2 f2_unpack(unsigned long long r) {
  float2 a;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
  return a;
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(r);
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(r);
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float cabs2(float2 a) { return fmaf(a.x, a.x, a.y * a.y); }

// ---- asynchronous global -> shared copies (cp.async) ------------------------------------
// Each thread's copies complete with cp.async.wait_group, which waits for that thread's own
// copies only (no spin on a flag); a barrier afterwards publishes them to the other threads.
__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem_dst, const void* gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gsrc) : "memory");
}
// copies src_bytes (0 or 16) bytes and zero-fills the rest of the 16-byte piece
__device__ __forceinline__ void cp_async16_zfill(void* smem_dst, const void* gsrc, int src_bytes) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gsrc), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(PENDING) : "memory");
}

// ---- programmatic dependent launch ---------------------------------------------------
// A kernel launched with launch_dep may start while the previous kernel on its stream is
// still running. It loads only plan constants (tables built before any march) until
// dep_wait(), which blocks in hardware until the previous grid has completed and its
// memory is visible; dep_release() then lets the next grid start its own prologue. Both are
// no-ops in a kernel launched without the attribute.
__device__ __forceinline__ void dep_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void dep_release() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_dep(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// One-time setup per device: kernel attributes (dynamic shared-memory limits, cluster
// sizes) and occupancy checks belong to the current device's context, so get(f) runs f the
// first time it is called with each device current, under a lock (no caller on that device
// launches before the setup is complete), and returns what f returned for that device.
struct PerDevice {
  static constexpr int kMax = 64;
  std::mutex m;
  int val[kMax] = {};
  bool done[kMax] = {};
  template <class F>
  int get(F&& f) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMax) return f();
    std::lock_guard<std::mutex> g(m);
    if (!done[dev]) {
      val[dev] = f();
      done[dev] = true;
    }
    return val[dev];
  }
};

inline bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }
inline bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }

inline size_t align256(size_t n) { return (n + 255) & ~size_t(255); }

}  // namespace bpmgb
