// Shared device helpers of libgbfoam: error reporting, slice addressing,
// deterministic reductions and the last-block ticket.
#pragma once

#include <cuda_runtime.h>
#include <limits.h>
#include <stdint.h>
#include <stdio.h>

#include <utility>

#include <nvtx3/nvToolsExt.h>

#include "gbfoam.h"

namespace gbf {

// NVTX range for the duration of a scope (shows each solve and
// factorisation as one named range in Nsight timelines; free without a
// profiler attached).
struct NvtxScope {
  explicit NvtxScope(const char* name) { nvtxRangePushA(name); }
  ~NvtxScope() { nvtxRangePop(); }
  NvtxScope(const NvtxScope&) = delete;
  NvtxScope& operator=(const NvtxScope&) = delete;
};

// Programmatic dependent launch (sm_90+): a kernel launched with
// launch_pdl may be scheduled while the previous kernel on the stream is
// still finishing; it must call pdl_wait() before it reads anything that
// kernel wrote (the wait returns once the previous grid has completed and
// its memory is visible).  pdl_launch_dependents() lets the next kernel be
// scheduled as this grid's blocks retire.  Both are no-ops for a kernel
// launched without the attribute.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// L2 eviction priority for streams.  Each inner iteration of the mixed
// solvers moves ~20x the L2's size; what pays to keep is the vector one
// kernel writes and the next reads (Ap, z, p).  Loads and stores of data that
// is dead after the access, or not read again until a later iteration, carry
// an evict-first policy so that those hand-over vectors are the lines that
// stay.  Hints only: the values are the same either way.
__device__ __forceinline__ unsigned long long l2_evict_first() {
  unsigned long long policy;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(policy));
  return policy;
}

// Read-only (for this kernel) float4 with an L2 cache policy.
__device__ __forceinline__ float4 ld_nc_hint(const float4* p, unsigned long long policy) {
  float4 v;
  asm("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
      : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
      : "l"(p), "l"(policy));
  return v;
}

// float4 that this thread also writes (after reading it), with an L2 cache
// policy.  The caller's own store of the same address depends on the value,
// so it cannot move before this load.
__device__ __forceinline__ float4 ld_hint(const float4* p, unsigned long long policy) {
  float4 v;
  asm("ld.global.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "l"(p), "l"(policy));
  return v;
}

__device__ __forceinline__ void st_hint(float4* p, float4 v, unsigned long long policy) {
  asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p),
               "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w), "l"(policy));
}

// Scalar forms of the above.
__device__ __forceinline__ float ld_nc_hint(const float* p, unsigned long long policy) {
  float v;
  asm("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(policy));
  return v;
}

__device__ __forceinline__ float ld_hint(const float* p, unsigned long long policy) {
  float v;
  asm("ld.global.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(policy));
  return v;
}

__device__ __forceinline__ void st_hint(float* p, float v, unsigned long long policy) {
  asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(p), "f"(v), "l"(policy));
}

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), int grid, int block, cudaStream_t s,
                              Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Per-thread error message (gbf_last_error()).
void set_error(const char* fmt, ...);

#define GBF_CHECK_CUDA(call)                                                   \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      ::gbf::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                       __FILE__, __LINE__);                                    \
      return GBF_ERR_CUDA;                                                     \
    }                                                                          \
  } while (0)

#define GBF_CHECK_LAUNCH() GBF_CHECK_CUDA(cudaGetLastError())

#define GBF_REQUIRE(cond, ...)                                                 \
  do {                                                                         \
    if (!(cond)) {                                                             \
      ::gbf::set_error(__VA_ARGS__);                                           \
      return GBF_ERR_ARG;                                                      \
    }                                                                          \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Threads per block of the cell kernels.  Must stay a multiple of 32 so that
// a warp covers exactly one 32-cell slice.
constexpr int kBlock = 256;

int check_layout(const gbf_layout* L);  // validates sizes / pointers

// Resident blocks per SM of a kernel at block size `block` (cached per
// kernel and device); 0 on error.
int resident_blocks(const void* kernel, int block);

// Grid of a grid-stride kernel: one full wave of resident blocks, no more
// blocks than there are `block`-sized chunks of work, at most kMaxGrid.
template <typename K>
inline int wave_grid(K kernel, int block, long long work) {
  int per_sm = resident_blocks(reinterpret_cast<const void*>(kernel), block);
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long g = (long long)(per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
  const long long need = (work + block - 1) / block;
  if (g > need) g = need;
  if (g > 4096) g = 4096;
  return g < 1 ? 1 : (int)g;
}

// Kernel timing probes (gbf_timing_enable): timing_begin returns true when
// an event was recorded; the caller then calls timing_end after the launch.
constexpr int kNumProbes = 6;
enum {
  kProbePcgAp = 0,
  kProbeMixedAp = 1,
  kProbeBicgAmul = 2,
  kProbeMixedTrue = 3,
  kProbeMixedBicgAmul = 4,
  kProbeBatchedAp = 5
};
bool timing_begin(int probe, cudaStream_t s);
void timing_end(int probe, cudaStream_t s);
int reduction_grid();  // fixed grid of the reducing kernels (SMs x 8, <= kMaxGrid)
constexpr int kMaxGrid = 4096;

// --------------------------------------------------------------------------
// Slice addressing of one cell.
// --------------------------------------------------------------------------
struct CellSlots {
  int base;  // slot of k = 0 for this lane
  int wo;    // owner-side slot count of the slice
  int wn;    // neighbour-side slot count of the slice
  int e0;    // compressed-offset entry of k = 0 (slice_off / 32)
};

__device__ __forceinline__ CellSlots cell_slots(const gbf_layout& L, int c) {
  const int s = c >> 5;
  CellSlots r;
  if (L.uniform_wo > 0 || L.uniform_wn > 0) {  // fixed widths: no metadata loads
    const int w = L.uniform_wo + L.uniform_wn;
    r.base = 32 * s * w + (c & 31);
    r.wo = L.uniform_wo;
    r.wn = L.uniform_wn;
    r.e0 = s * w;
    return r;
  }
  const int w = __ldg(L.slice_w + s);
  const int off = __ldg(L.slice_off + s);
  r.base = off + (c & 31);
  r.wo = w & 0xffff;
  r.wn = w >> 16;
  r.e0 = off >> 5;
  return r;
}

// Column of slot k (absolute entry index e = e0 + k, slot index i) of cell
// c: from the compressed offset when the slot is uniform across the slice,
// else from slot_col.  -1 marks padding.
__device__ __forceinline__ int slot_column(const gbf_layout& L, int e, int i, int c) {
  if (L.slot_dm != nullptr) {
    const int2 dm = __ldg(reinterpret_cast<const int2*>(L.slot_dm) + e);
    if (dm.x != INT_MIN) return (((unsigned)dm.y >> (c & 31)) & 1u) ? c + dm.x : -1;
  }
  return __ldg(L.slot_col + i);
}

// --------------------------------------------------------------------------
// Deterministic sums: fixed shuffle tree inside a warp, fixed tree over the
// warps of a block, partials reduced by the last block in index order.
// --------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Sum of v over the block; valid in thread 0 only.  `sh` holds blockDim/32.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();  // sh may still be read by a previous call
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  T t = (T)0;
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    t = (lane < nw) ? sh[lane] : (T)0;
    t = warp_sum(t);
  }
  return t;
}

// Returns true in every thread of the block that finished last.  The caller
// wrote its partials (thread 0) before calling; the last block reads only
// partials (and state written by earlier kernels), so only thread 0 fences
// its writes before taking the ticket -- the other threads' stores need no
// ordering here, and a fence in every thread stalls each on its own
// outstanding stores.  The ticket counter is reset by the last block.
__device__ __forceinline__ bool last_block_done(unsigned int* ticket) {
  __shared__ bool am_last;
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned int t = atomicAdd(ticket, 1u);
    am_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (am_last) {
    __threadfence();
    if (threadIdx.x == 0) *ticket = 0u;
  }
  return am_last;
}

// Sum of partials[0..n) in a fixed order, by the whole block; result in
// thread 0.  Reads through L2 (other blocks wrote them).  Thread t adds
// partials t, t + B, t + 2B, ... in that order; the loads of up to eight of
// them are issued before the first add, so a thread waits for one L2 round
// trip instead of one per partial (the grids of one wave leave ~5 partials
// per thread of the reducing block).
template <typename T>
__device__ __forceinline__ T reduce_partials(const T* partials, int n, T* sh) {
  constexpr int U = 8;
  const int B = blockDim.x;
  T v = (T)0;
  for (int i0 = threadIdx.x; i0 < n; i0 += U * B) {
    T q[U];
#pragma unroll
    for (int u = 0; u < U; ++u) q[u] = (i0 + u * B < n) ? __ldcg(partials + i0 + u * B) : (T)0;
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (i0 + u * B < n) v += q[u];
  }
  return block_sum(v, sh);
}

// 0.0 + p without a floating-point add: p itself, except that -0.0 becomes
// +0.0.  The first term of a running sum that starts at 0.0 enters this way,
// which saves one FP64 add per sum (GB300's FP64 rate bounds the bitwise
// FP64 gathers) and gives the same bits as the addition.
__device__ __forceinline__ double first_term(double p) {
  return __double_as_longlong(p) == (long long)0x8000000000000000ULL ? 0.0 : p;
}
__device__ __forceinline__ float first_term(float p) {
  return __float_as_int(p) == (int)0x80000000u ? 0.0f : p;
}

// Canonical IEEE helpers (one rounding each, never contracted to FMA).
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }

// Exact FP64 product of two FP32 values.
__device__ __forceinline__ double dprod(float a, float b) { return (double)a * (double)b; }

// Double-float accumulator: hi + lo carries the running sum of exact FP32
// products.  Every operation is an explicitly rounded intrinsic so that the
// compiler cannot contract or reassociate the error-free transformations.
struct DFAcc {
  float hi = 0.0f, lo = 0.0f;
  __device__ __forceinline__ void add_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    const float e = __fmaf_rn(a, b, -p);  // a*b - p exactly (TwoProduct)
    const float s = __fadd_rn(hi, p);     // TwoSum(hi, p)
    const float bb = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(err, e));
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// (hi, lo) += (bhi, blo) in double-float arithmetic: TwoSum of the high
// parts, low parts and rounding error added into lo.
__device__ __forceinline__ void df_add(float& hi, float& lo, float bhi, float blo) {
  const float s = __fadd_rn(hi, bhi);
  const float bb = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(bhi, bb));
  hi = s;
  lo = __fadd_rn(lo, __fadd_rn(blo, err));
}

__device__ __forceinline__ void df_warp_sum(float& hi, float& lo) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h = __shfl_down_sync(0xffffffffu, hi, o);
    const float l = __shfl_down_sync(0xffffffffu, lo, o);
    df_add(hi, lo, h, l);
  }
}

// Sum over the block of the threads' double-float accumulators, as a double
// in thread 0 (0.0 elsewhere).  The whole tree -- shuffles within each warp,
// then over the warps -- stays in double-float arithmetic on the FP32 pipes
// and only thread 0 converts to FP64: GB300's FP64 rate is a small fraction
// of its FP32 rate, and a per-thread conversion plus an FP64 shuffle tree
// made the reduction, not memory, the bound of the vector kernels when each
// thread holds only a few cells.  Fixed order, so deterministic.  `sh`
// holds blockDim/32 doubles (used as float pairs).
__device__ __forceinline__ double block_sum_df(const DFAcc& a, double* sh) {
  float2* s2 = reinterpret_cast<float2*>(sh);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float hi = a.hi, lo = a.lo;
  df_warp_sum(hi, lo);
  __syncthreads();  // sh may still be read by a previous call
  if (lane == 0) s2[wid] = make_float2(hi, lo);
  __syncthreads();
  double t = 0.0;
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    const float2 e = (lane < nw) ? s2[lane] : make_float2(0.0f, 0.0f);
    hi = e.x;
    lo = e.y;
    df_warp_sum(hi, lo);
    if (lane == 0) t = (double)hi + (double)lo;
  }
  return t;
}

}  // namespace gbf
