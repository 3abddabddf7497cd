// Library-level entry points: error strings, version, device queries.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>

#include <map>
#include <mutex>
#include <utility>

#include "common.cuh"

namespace gbf {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int resident_blocks(const void* kernel, int block) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  const auto key = std::make_pair(kernel, block * 64 + dev);
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, block, 0) != cudaSuccess) n = 0;
  std::lock_guard<std::mutex> lk(mu);
  cache[key] = n;
  return n;
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

extern "C" int gbf_version(void) { return 2; }

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

// --------------------------------------------------------------------------
// Kernel timing probes: event pairs recorded around selected launches.
// --------------------------------------------------------------------------
#include <mutex>
#include <vector>

namespace gbf {

struct Probe {
  std::vector<cudaEvent_t> start, stop;
  int used = 0;
};
static std::mutex g_tmu;
static bool g_timing = false;
static int g_cap = 0;
static Probe g_probes[kNumProbes];

static void clear_probes() {
  for (auto& p : g_probes) {
    for (auto e : p.start) cudaEventDestroy(e);
    for (auto e : p.stop) cudaEventDestroy(e);
    p.start.clear();
    p.stop.clear();
    p.used = 0;
  }
}

bool timing_begin(int probe, cudaStream_t s) {
  if (!g_timing || probe < 0 || probe >= kNumProbes) return false;
  std::lock_guard<std::mutex> lk(g_tmu);
  Probe& p = g_probes[probe];
  if (p.used >= g_cap) return false;
  if ((int)p.start.size() <= p.used) {
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess) return false;
    if (cudaEventCreate(&b) != cudaSuccess) {
      cudaEventDestroy(a);
      return false;
    }
    p.start.push_back(a);
    p.stop.push_back(b);
  }
  return cudaEventRecord(p.start[p.used], s) == cudaSuccess;
}

void timing_end(int probe, cudaStream_t s) {
  std::lock_guard<std::mutex> lk(g_tmu);
  Probe& p = g_probes[probe];
  if (cudaEventRecord(p.stop[p.used], s) == cudaSuccess) p.used++;
}

}  // namespace gbf

extern "C" int gbf_timing_enable(int32_t enable, int32_t max_events) {
  std::lock_guard<std::mutex> lk(gbf::g_tmu);
  gbf::clear_probes();
  gbf::g_timing = enable != 0;
  gbf::g_cap = max_events > 0 ? max_events : 0;
  return GBF_OK;
}

extern "C" int gbf_timing_read(int32_t probe, int32_t* launches, double* total_ms) {
  if (probe < 0 || probe >= gbf::kNumProbes || !launches || !total_ms) {
    gbf::set_error("timing_read: bad probe %d", probe);
    return GBF_ERR_ARG;
  }
  std::lock_guard<std::mutex> lk(gbf::g_tmu);
  gbf::Probe& p = gbf::g_probes[probe];
  double tot = 0.0;
  for (int i = 0; i < p.used; ++i) {
    cudaError_t e = cudaEventSynchronize(p.stop[i]);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, p.start[i], p.stop[i]);
    if (e != cudaSuccess) {
      gbf::set_error("timing_read: %s", cudaGetErrorString(e));
      return GBF_ERR_CUDA;
    }
    tot += ms;
  }
  *launches = p.used;
  *total_ms = tot;
  return GBF_OK;
}
