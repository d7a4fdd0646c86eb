// Status strings, the thread-local error message and version info of the C ABI.
#include <stdarg.h>
#include <stdio.h>

#include "hm_common.cuh"

static thread_local char g_last_error[512] = "";

void hm_set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

int hm_cuda_status(cudaError_t e, const char* what) {
  hm_set_error("%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? HM_ENOMEM : HM_ECUDA;
}

extern "C" const char* hm_last_error(void) { return g_last_error; }

extern "C" const char* hm_status_string(int s) {
  switch (s) {
    case HM_OK: return "ok";
    case HM_EINVAL: return "invalid argument";
    case HM_ECUDA: return "CUDA error";
    case HM_ECAPACITY: return "capacity exceeded";
    case HM_ETIMEOUT: return "device wait timed out";
    case HM_ENOMEM: return "out of memory";
    case HM_EPARSE: return "parse error";
    case HM_EUNSUPPORTED: return "unsupported";
    default: return "unknown status";
  }
}

extern "C" const char* hm_version(void) { return "hairmsnn-gb300 0.1 sm_103a"; }

extern "C" int hm_copy_to_host(void* host_dst, const void* device_src, int64_t bytes) {
  if (bytes < 0 || (bytes > 0 && (!host_dst || !device_src))) return hm_set_error("hm_copy_to_host: bad args"), HM_EINVAL;
  if (bytes == 0) return HM_OK;
  cudaError_t e = cudaMemcpy(host_dst, device_src, (size_t)bytes, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? HM_OK : hm_cuda_status(e, "hm_copy_to_host");
}
