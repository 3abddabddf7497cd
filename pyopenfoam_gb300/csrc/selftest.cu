// Self-test of the bounded waits (no reference counterpart).
//
// The device-side waits of this library -- the grid barrier of the
// single-launch PCG and the mbarrier waits of the bulk-copy staged Amul --
// give up after a fixed number of polls, record a fault and let the kernel
// return, so that a lost participant turns into an error status instead of a
// hung GPU.  This entry point makes each kind of wait run out on purpose,
// with short poll limits, on a flag that nothing sets:
//   * a two-block cooperative launch in which block 1 never arrives at the
//     grid barrier, so block 0's wait runs out;
//   * one block waiting on an mbarrier on which no copy and no arrival is
//     ever posted.
// Nothing faults, traps or spins without bound; the whole test takes well
// under a millisecond of GPU time.
#include <string.h>

#include "barrier.cuh"
#include "bulk.cuh"
#include "wavefront.cuh"

namespace gbf {

__global__ void barrier_timeout_kernel(GridBarrier* bar, long long polls, int* out) {
  if (blockIdx.x == 1) return;  // the participant that never arrives
  const bool ok = grid_barrier(bar, gridDim.x, polls);
  if (threadIdx.x == 0) out[0] = ok ? 0 : 1;
}

__global__ void mbarrier_timeout_kernel(int polls, int* out) {
  __shared__ unsigned long long bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    bool got = false;
    for (int i = 0; i < polls && !got; ++i) got = mbar_try_wait(&bar, 0);
    out[1] = got ? 0 : 1;
  }
}

// A two-level wavefront whose grid barrier can never complete: block 1
// never arrives.  Block 0's wait runs out, the fault word is set and block 0
// overwrites the whole output with NaN -- the failure path of every
// cooperative wavefront.
__global__ void wavefront_timeout_kernel(const int32_t* level_ptr, GridBarrier* bar,
                                         long long polls, double* out, int n) {
  if (blockIdx.x == 1) return;  // the participant that never arrives
  const bool ok = run_levels(bar, level_ptr, 2, [&](int i) { out[i] = 1.0; }, polls);
  if (!ok) poison(out, n);
}

}  // namespace gbf

using namespace gbf;

extern "C" int gbf_selftest_wavefront_fault(int32_t* result_h) {
  GBF_REQUIRE(result_h, "selftest: NULL pointer");
  int dev = 0, coop = 0;
  GBF_CHECK_CUDA(cudaGetDevice(&dev));
  GBF_CHECK_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  GBF_REQUIRE(coop, "selftest: the device has no cooperative launch");
  constexpr int n = 64;
  struct Buf {
    GridBarrier bar;
    int32_t level_ptr[4];
    double out[n];
  };
  Buf h0;
  memset(&h0, 0, sizeof(h0));
  h0.level_ptr[0] = 0;
  h0.level_ptr[1] = n / 2;
  h0.level_ptr[2] = n;
  Buf* d = nullptr;
  GBF_CHECK_CUDA(cudaMalloc(&d, sizeof(Buf)));
  cudaError_t e = cudaMemcpy(d, &h0, sizeof(Buf), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    const int32_t* lp = d->level_ptr;
    GridBarrier* bar = &d->bar;
    long long polls = 1000;  // ~0.1 ms
    double* out = d->out;
    int nn = n;
    void* args[] = {(void*)&lp, &bar, &polls, &out, &nn};
    e = cudaLaunchCooperativeKernel((const void*)wavefront_timeout_kernel, dim3(2), dim3(32),
                                    args, 0, nullptr);
  }
  Buf h;
  if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(Buf), cudaMemcpyDeviceToHost);
  cudaFree(d);
  GBF_CHECK_CUDA(e);
  int all_nan = 1;
  for (int i = 0; i < n; ++i) all_nan &= (h.out[i] != h.out[i]) ? 1 : 0;
  result_h[0] = h.bar.fault;
  result_h[1] = all_nan;
  return GBF_OK;
}

extern "C" int gbf_selftest_bounded_waits(int32_t* timed_out_h) {
  GBF_REQUIRE(timed_out_h, "selftest: NULL pointer");
  int dev = 0, coop = 0;
  GBF_CHECK_CUDA(cudaGetDevice(&dev));
  GBF_CHECK_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  GBF_REQUIRE(coop, "selftest: the device has no cooperative launch");
  struct Buf {
    GridBarrier bar;
    int out[2];
  };
  Buf* d = nullptr;
  GBF_CHECK_CUDA(cudaMalloc(&d, sizeof(Buf)));
  cudaError_t e = cudaMemset(d, 0, sizeof(Buf));
  if (e == cudaSuccess) {
    GridBarrier* bar = &d->bar;
    long long polls = 1000;  // ~0.1 ms
    int* out = d->out;
    void* args[] = {&bar, &polls, &out};
    e = cudaLaunchCooperativeKernel((const void*)barrier_timeout_kernel, dim3(2), dim3(32), args,
                                    0, nullptr);
  }
  if (e == cudaSuccess) {
    mbarrier_timeout_kernel<<<1, 32>>>(1000, d->out);
    e = cudaGetLastError();
  }
  Buf h;
  if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(Buf), cudaMemcpyDeviceToHost);
  cudaFree(d);
  GBF_CHECK_CUDA(e);
  timed_out_h[0] = h.out[0];
  timed_out_h[1] = h.out[1];
  timed_out_h[2] = h.bar.fault;
  return GBF_OK;
}
