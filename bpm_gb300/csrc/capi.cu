// Library-wide C ABI helpers: version, thread-local error text, launch accounting.
#include <string>

#include "common.cuh"

namespace bpmgb {

static thread_local std::string t_error;
std::atomic<unsigned long long> g_launches{0};

void set_error(const std::string& msg) { t_error = msg; }
void clear_error() { t_error.clear(); }

int cuda_fail(cudaError_t e, const char* what) {
  t_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  // leave no sticky error behind for the caller's next runtime call
  cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? BPM_ERR_OOM : BPM_ERR_CUDA;
}

}  // namespace bpmgb

extern "C" int bpm_version(void) { return BPM_GB300_VERSION; }

extern "C" const char* bpm_last_error(void) { return bpmgb::t_error.c_str(); }

extern "C" unsigned long long bpm_launch_count(void) { return bpmgb::g_launches.load(); }

extern "C" int bpm_host_ptr_mapped(const void* p) {
  if (!p) return 0;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return (a.type == cudaMemoryTypeHost && a.devicePointer == p) ? 1 : 0;
}
