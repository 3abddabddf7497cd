// Level-scheduled wavefronts in one cooperative launch.
//
// The DIC / DILU factorisations, the apply_full sweeps and the Gauss-Seidel
// sweeps visit the items (cells or faces) of a level schedule level by
// level; items of one level are independent, a level reads what earlier
// levels wrote.  Launching one kernel per level costs a launch and a drain
// per level (767 levels for DIC at 256^3).  Here all blocks are resident
// (cudaLaunchCooperativeKernel) and walk the levels together, separated by
// the bounded software grid barrier of barrier.cuh; values written by other
// blocks are read through L2 (__ldcg) by the item bodies.
//
// A barrier wait that runs out sets the barrier's fault word; every block
// that sees it overwrites the whole output with NaN (an invalid result is
// then visible downstream) and returns.  The host can read the fault word
// with gbf_wavefront_fault.
#pragma once

#include "barrier.cuh"

namespace gbf {

// body(i) for every item i of every level, in level order.  Returns false if
// a barrier wait ran out.
template <typename F>
__device__ __forceinline__ bool run_levels(GridBarrier* bar, const int32_t* __restrict__ level_ptr,
                                           int n_levels, F&& body,
                                           long long max_polls = kBarrierPolls) {
  const int stride = gridDim.x * blockDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  for (int lv = 0; lv < n_levels; ++lv) {
    const int start = __ldg(level_ptr + lv), end = __ldg(level_ptr + lv + 1);
    for (int i = start + tid; i < end; i += stride) body(i);
    if (lv + 1 < n_levels && !grid_barrier(bar, gridDim.x, max_polls)) return false;
  }
  return true;
}

// Every block that observed a barrier fault writes NaN over out[0, n).
__device__ __forceinline__ void poison(double* out, int n) {
  const double nan = __longlong_as_double(0x7ff8000000000000LL);
  for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = nan;
}

// Blocks of a cooperative wavefront launch: resident blocks of `kernel`,
// no more than needed for the largest level and at most `per_sm_max` per SM
// (fewer blocks make a cheaper barrier, more hide more latency of the
// items' dependent loads; a level larger than the grid is looped over).
// Measured on GB300: the Gauss-Seidel cell levels are fastest with two
// blocks per SM, the many small face levels (DILU, sweeps) with one.
// 0 when the device cannot launch cooperatively.
inline int wavefront_grid(const void* kernel, int block, long long max_level_items,
                          int per_sm_max) {
  int dev = 0, coop = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (!coop || sms <= 0) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0) != cudaSuccess ||
      per_sm <= 0)
    return 0;
  long long g = (long long)(per_sm < per_sm_max ? per_sm : per_sm_max) * sms;
  const long long need = (max_level_items + block - 1) / block;
  if (g > need) g = need;
  return g < 1 ? 1 : (int)g;
}

// Zeroes the caller's barrier memory (gbf_wavefront_barrier_bytes) and
// launches `kernel` cooperatively on `grid` blocks of kBlock threads.
inline cudaError_t launch_wavefront(const void* kernel, int grid, void** args, void* barrier,
                                    cudaStream_t s) {
  static_assert(sizeof(GridBarrier) <= 64, "gbf_wavefront_barrier_bytes");
  cudaError_t e = cudaMemsetAsync(barrier, 0, sizeof(GridBarrier), s);
  if (e != cudaSuccess) return e;
  return cudaLaunchCooperativeKernel(kernel, dim3(grid), dim3(kBlock), args, 0, s);
}

// ---- dataflow walks (no barrier between levels) -----------------------------
//
// A step's inputs sit in slots of device memory that hold the empty marker
// until their producer stores them; a step polls only the slots it reads.
// The empty marker is the all-ones bit pattern (a NaN); a NaN result is
// stored as the canonical NaN so that it cannot read as empty.  Every wait
// is bounded: after max_polls passes a warp sets the barrier's fault word
// and returns, and the warps that see the fault word return too; the
// output kernel then writes NaN everywhere.
constexpr long long kFlowEmpty = -1LL;
constexpr long long kFlowPolls = 1LL << 22;  // a few seconds of passes

__device__ __forceinline__ double ld_flow(const double* p) {
  double v;
  asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_flow(double* p, double v) {
  if (v != v) v = __longlong_as_double(0x7ff8000000000000LL);
  asm volatile("st.relaxed.gpu.global.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}

__device__ __forceinline__ bool flow_empty(double v) {
  return __double_as_longlong(v) == kFlowEmpty;
}

// End of one pass over a chunk: true when every lane is done; false with
// *quit set when a wait ran out here or elsewhere.
__device__ __forceinline__ bool flow_pass_end(bool done, long long& polls, long long max_polls,
                                              GridBarrier* bar, bool* quit) {
  if (__all_sync(0xffffffffu, done)) return true;
  ++polls;
  if (polls > max_polls) {
    if ((threadIdx.x & 31) == 0) atomicExch(&bar->fault, 1);
    *quit = true;
    return false;
  }
  // one decision for the whole warp (polls is the same in every lane)
  if ((polls & 63) == 0 && __any_sync(0xffffffffu, *(volatile int*)&bar->fault != 0)) {
    *quit = true;
    return false;
  }
  // the pass is bound by the polls' L2 round trip: 0, 16 or 64 ns of sleep
  // measured the same on GB300 (DILU 128^3 2.61-2.62 ms), 256 ns 2 % slower
  __nanosleep(64);
  return false;
}

}  // namespace gbf
