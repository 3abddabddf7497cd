// Library-level entry points: error strings, version, device queries.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>

#include "gbfoam.h"

namespace gbf {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int reduction_grid() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1216;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
    return 1216;
  int g = sms * 8;
  return g > 4096 ? 4096 : g;
}

}  // namespace gbf

extern "C" const char* gbf_last_error(void) { return gbf::g_err; }

extern "C" int gbf_version(void) { return 1; }

extern "C" int gbf_device_sm_count(int32_t* n_sm) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) {
    gbf::set_error("cuda device query failed: %s", cudaGetErrorString(e));
    return GBF_ERR_CUDA;
  }
  *n_sm = sms;
  return GBF_OK;
}
