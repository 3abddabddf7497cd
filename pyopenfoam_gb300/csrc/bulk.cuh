// Shared-memory staging of the FP32 Amul stream with bulk asynchronous
// copies (cp.async.bulk, completion counted on an mbarrier).
//
// For a layout whose slices all have 3 owner-side and 3 neighbour-side slots,
// every slot offset-uniform (layout_kind == kLayoutHex33), the bytes a block
// of 256 cells streams from HBM are contiguous per 8-slice tile:
//   coefficients 8*6*32 floats (6144 B), x 256 floats (1024 B),
//   diagonal 256 floats (1024 B), {delta, mask} entries 8*6 int2 (384 B).
// One thread of the block issues the four copies of a tile into a ring of
// kStages stage buffers; all threads wait on the stage's mbarrier, compute
// their cell from shared memory (the neighbour x values are gathered from
// global memory through L1/L2) and release the stage with a block barrier,
// after which the issuing thread refills it with the tile kStages ahead.
// The HBM stream therefore stays in flight independently of the registers
// the gather needs.
//
// For a symmetric matrix stored as its owner-side half (SYM), a tile streams
// 8*3*32 owner-side coefficients (3072 B) and the slices' 48 mirror entries
// (48 B) instead of the 6144 B of both sides; a neighbour-side coefficient
// is the owner-side one of the owner cell, read from the stage when that cell
// lies in the tile and from global memory (an L2 hit: its tile streamed
// recently) otherwise.  Neighbour x values of cells inside the tile are read
// from the stage as well.
//
// Every wait is bounded: after kWaitPolls unsuccessful polls the block
// records a fault, drains (again bounded) the copies it has in flight and
// stops streaming; the host turns the fault into GBF_DEVICE_TIMEOUT.
#pragma once

#include <stddef.h>

#include "amul.cuh"

namespace gbf {

// Cells per tile = threads per block of the staged kernels.
#ifndef GBF_TILE_CELLS
#define GBF_TILE_CELLS 256
#endif
constexpr int kTileCells = GBF_TILE_CELLS;
constexpr int kTileSlices = kTileCells / 32;
constexpr int kHexW = 6;
// resident blocks per SM the staged kernels are compiled for (2048 threads)
constexpr int kStreamBlocksPerSM = 2048 / kTileCells;
// the symmetric form copies kTileSlices * kHexW mirror bytes per tile,
// which a bulk copy can move only in multiples of 16 bytes
constexpr bool kSymStaged = (kTileSlices * kHexW) % 16 == 0;
constexpr int kStages = 3;
constexpr int kWaitPolls = 1 << 20;

struct __align__(128) HexStage {
  float coef[kTileSlices * kHexW * 32];
  float x[kTileCells];
  float d[kTileCells];
  int2 dm[kTileSlices * kHexW];
};
static_assert(offsetof(HexStage, dm) % 16 == 0 && (kHexW * sizeof(int2)) % 16 == 0,
              "a slice's offset entries are read as 128-bit words");
constexpr unsigned kStageBytes = sizeof(float) * (kTileSlices * kHexW * 32 + 2 * kTileCells) +
                                 sizeof(int2) * kTileSlices * kHexW;
static_assert(kStageBytes % 16 == 0, "bulk copies move multiples of 16 bytes");

struct __align__(128) HexStageSym {
  float coef[kTileSlices * 3 * 32];
  float x[kTileCells];
  float d[kTileCells];
  int2 dm[kTileSlices * kHexW];
  int8_t mir[kTileSlices * kHexW];
};
constexpr unsigned kStageBytesSym = sizeof(float) * (kTileSlices * 3 * 32 + 2 * kTileCells) +
                                    sizeof(int2) * kTileSlices * kHexW +
                                    sizeof(int8_t) * kTileSlices * kHexW;
static_assert(!kSymStaged || kStageBytesSym % 16 == 0, "bulk copies move multiples of 16 bytes");

template <bool SYM>
struct HexStageOf {
  using type = HexStage;
};
template <>
struct HexStageOf<true> {
  using type = HexStageSym;
};

template <bool SYM>
struct HexRing {
  typename HexStageOf<SYM>::type stage[kStages];
  unsigned long long bar[kStages];
};

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

// Makes initialised barriers visible to the asynchronous proxy.
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
  for (int i = 0; i < kWaitPolls; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// dst and src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes,
                                         unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// bulk_g2s with an L2 evict-first policy: for streams read once per pass
// (coefficients, diagonal), so that their lines are the first to go and the
// vectors the surrounding kernels reuse stay in L2 longer.
__device__ __forceinline__ void bulk_g2s_stream(void* dst, const void* src, unsigned bytes,
                                                unsigned long long* bar) {
  unsigned long long policy;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(policy));
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
      " [%0], [%1], %2, [%3], %4;" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(policy)
      : "memory");
}

// Issues the copies of tile t into stage s (one thread).
__device__ __forceinline__ void hex_issue(HexRing<false>& R, int s, int t, const float* coef,
                                          const float* x, const float* d, const int* slot_dm,
                                          const int8_t*) {
  HexStage& S = R.stage[s];
  mbar_arrive_expect_tx(&R.bar[s], kStageBytes);
  bulk_g2s_stream(S.coef, coef + (size_t)t * (kTileSlices * kHexW * 32), sizeof(S.coef),
                  &R.bar[s]);
  bulk_g2s(S.x, x + (size_t)t * kTileCells, sizeof(S.x), &R.bar[s]);
  bulk_g2s_stream(S.d, d + (size_t)t * kTileCells, sizeof(S.d), &R.bar[s]);
  bulk_g2s(S.dm, slot_dm + (size_t)t * (2 * kTileSlices * kHexW), sizeof(S.dm), &R.bar[s]);
}

__device__ __forceinline__ void hex_issue(HexRing<true>& R, int s, int t, const float* own,
                                          const float* x, const float* d, const int* slot_dm,
                                          const int8_t* slot_mirror) {
  HexStageSym& S = R.stage[s];
  mbar_arrive_expect_tx(&R.bar[s], kStageBytesSym);
  bulk_g2s(S.coef, own + (size_t)t * (kTileSlices * 3 * 32), sizeof(S.coef), &R.bar[s]);
  bulk_g2s(S.x, x + (size_t)t * kTileCells, sizeof(S.x), &R.bar[s]);
  bulk_g2s(S.d, d + (size_t)t * kTileCells, sizeof(S.d), &R.bar[s]);
  bulk_g2s(S.dm, slot_dm + (size_t)t * (2 * kTileSlices * kHexW), sizeof(S.dm), &R.bar[s]);
  bulk_g2s(S.mir, slot_mirror + (size_t)t * (kTileSlices * kHexW), sizeof(S.mir), &R.bar[s]);
}

// (A x)[c] of thread `tid` of the tile in stage S: the products and the
// summation order of cell_amul_fixed<float, A, NEI_FIRST, 3, 3>.
template <typename A, bool NEI_FIRST>
__device__ __forceinline__ A hex_cell_from_stage(const HexStage& S, int tid,
                                                 const float* __restrict__ x, int c) {
  const int sl = tid >> 5, lane = tid & 31;
  float a[kHexW], xv[kHexW];
  bool on[kHexW];
#pragma unroll
  for (int k = 0; k < kHexW; ++k) a[k] = S.coef[(sl * kHexW + k) * 32 + lane];
  // the slice's six {delta, mask} entries: three 128-bit shared loads
  // (48 B per slice, 16-byte aligned in the stage)
  const int4* __restrict__ dm4 = reinterpret_cast<const int4*>(S.dm) + 3 * sl;
#pragma unroll
  for (int q = 0; q < kHexW / 2; ++q) {
    const int4 e = dm4[q];
    on[2 * q] = ((unsigned)e.y >> lane) & 1u;
    on[2 * q + 1] = ((unsigned)e.w >> lane) & 1u;
    xv[2 * q] = on[2 * q] ? __ldg(x + c + e.x) : 0.0f;
    xv[2 * q + 1] = on[2 * q + 1] ? __ldg(x + c + e.z) : 0.0f;
  }
  A so = (A)0, sn = (A)0;
  if (on[0]) so = first_term((A)__fmul_rn(a[0], xv[0]));
#pragma unroll
  for (int k = 1; k < 3; ++k)
    if (on[k]) so = add_rn(so, (A)__fmul_rn(a[k], xv[k]));
  if (on[3]) sn = first_term((A)__fmul_rn(a[3], xv[3]));
#pragma unroll
  for (int k = 4; k < kHexW; ++k)
    if (on[k]) sn = add_rn(sn, (A)__fmul_rn(a[k], xv[k]));
  A y = (A)__fmul_rn(S.d[tid], S.x[tid]);
  if (NEI_FIRST) {
    y = add_rn(y, sn);
    return add_rn(y, so);
  }
  y = add_rn(y, so);
  return add_rn(y, sn);
}

// The symmetric form: (A x)[c] from the owner-side half.  Same products and
// summation order as hex_cell_from_stage<A, false> on the full packing.
template <typename A>
__device__ __forceinline__ A hex_cell_from_stage_sym(const HexStageSym& S, int tid,
                                                     const float* __restrict__ own,
                                                     const float* __restrict__ x, int c) {
  const int sl = tid >> 5, lane = tid & 31;
  const int c0 = c - tid;  // first cell of the tile
  float a[kHexW], xv[kHexW];
  bool on[kHexW];
#pragma unroll
  for (int k = 0; k < 3; ++k) a[k] = S.coef[(sl * 3 + k) * 32 + lane];
#pragma unroll
  for (int k = 0; k < kHexW; ++k) {
    const int2 e = S.dm[sl * kHexW + k];
    on[k] = ((unsigned)e.y >> lane) & 1u;
    const int cn = c + e.x;
    const unsigned in_tile = (unsigned)(cn - c0);
    xv[k] = !on[k] ? 0.0f : (in_tile < (unsigned)kTileCells ? S.x[in_tile] : __ldg(x + cn));
    if (k >= 3) {
      const int j = S.mir[sl * kHexW + k];
      const int i_own = 96 * (cn >> 5) + 32 * j + (cn & 31);
      a[k] = !on[k] ? 0.0f
                    : (in_tile < (unsigned)kTileCells ? S.coef[i_own - 3 * c0] : __ldg(own + i_own));
    }
  }
  A so = (A)0, sn = (A)0;
  if (on[0]) so = first_term((A)__fmul_rn(a[0], xv[0]));
#pragma unroll
  for (int k = 1; k < 3; ++k)
    if (on[k]) so = add_rn(so, (A)__fmul_rn(a[k], xv[k]));
  if (on[3]) sn = first_term((A)__fmul_rn(a[3], xv[3]));
#pragma unroll
  for (int k = 4; k < kHexW; ++k)
    if (on[k]) sn = add_rn(sn, (A)__fmul_rn(a[k], xv[k]));
  A y = (A)__fmul_rn(S.d[tid], S.x[tid]);
  y = add_rn(y, so);
  return add_rn(y, sn);
}

template <typename A, bool NEI_FIRST>
__device__ __forceinline__ A hex_cell(const HexStage& S, int tid, const float*,
                                      const float* __restrict__ x, int c) {
  return hex_cell_from_stage<A, NEI_FIRST>(S, tid, x, c);
}
template <typename A, bool NEI_FIRST>
__device__ __forceinline__ A hex_cell(const HexStageSym& S, int tid,
                                      const float* __restrict__ own,
                                      const float* __restrict__ x, int c) {
  static_assert(!NEI_FIRST, "a symmetric matrix is its own transpose");
  return hex_cell_from_stage_sym<A>(S, tid, own, x, c);
}

// True when the pointers the staged path streams from are 16-byte aligned.
inline bool hex_stream_aligned(const void* coef, const void* x, const void* d,
                               const void* slot_dm) {
  return ((reinterpret_cast<uintptr_t>(coef) | reinterpret_cast<uintptr_t>(x) |
           reinterpret_cast<uintptr_t>(d) | reinterpret_cast<uintptr_t>(slot_dm)) &
          15u) == 0;
}

// Runs f(c, y, xc, pre(c)) for every cell of the full tiles assigned to this
// block (tiles blockIdx.x, blockIdx.x + gridDim.x, ...).  pre(c) -- a load of
// another per-cell operand the epilogue needs -- is issued before the wait
// on the tile's copies, so that its latency overlaps the wait and the
// gather instead of following them.  Returns false if a wait ran out (the
// block then stops streaming after draining its copies).
template <typename A, bool NEI_FIRST, bool SYM, typename PRE, typename F>
__device__ __forceinline__ bool hex_stream_tiles_pre(HexRing<SYM>& R, int n_tiles,
                                                     const float* coef, const float* x,
                                                     const float* d, const int* slot_dm,
                                                     const int8_t* slot_mirror, PRE&& pre,
                                                     F&& f) {
  const int tid = threadIdx.x;
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(&R.bar[s], 1);
    mbar_fence_init();
  }
  __syncthreads();
  int issued = 0;  // tiles issued by thread 0 (valid in thread 0)
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      const int t = blockIdx.x + s * gridDim.x;
      if (t >= n_tiles) break;
      hex_issue(R, s, t, coef, x, d, slot_dm, slot_mirror);
      ++issued;
    }
  }
  bool ok = true;
  int k = 0;
  for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, ++k) {
    const int s = k % kStages;
    const unsigned parity = (unsigned)(k / kStages) & 1u;
    const int c = t * kTileCells + tid;
    const auto aux = pre(c);
    // one thread polls the stage's barrier; the block barrier then orders
    // the completed copies before every thread's reads of the stage
    bool got = true;
    if (tid == 0) got = mbar_wait(&R.bar[s], parity);
    if (__syncthreads_or(!got)) {
      ok = false;
      break;
    }
    f(c, hex_cell<A, NEI_FIRST>(R.stage[s], tid, coef, x, c), R.stage[s].x[tid], aux);
    __syncthreads();  // every thread is done with stage s
    if (tid == 0) {
      const int tn = t + kStages * gridDim.x;
      if (tn < n_tiles) {
        hex_issue(R, s, tn, coef, x, d, slot_dm, slot_mirror);
        ++issued;
      }
    }
  }
  if (!ok && tid == 0) {
    // drain: wait (bounded) for every issued stage not yet consumed
    for (int j = k; j < issued; ++j) mbar_wait(&R.bar[j % kStages], (unsigned)(j / kStages) & 1u);
  }
  __syncthreads();
  return ok;
}

// f(c, y, xc) for every cell of the block's full tiles (no extra operand).
template <typename A, bool NEI_FIRST, bool SYM, typename F>
__device__ __forceinline__ bool hex_stream_tiles(HexRing<SYM>& R, int n_tiles, const float* coef,
                                                 const float* x, const float* d,
                                                 const int* slot_dm, const int8_t* slot_mirror,
                                                 F&& f) {
  return hex_stream_tiles_pre<A, NEI_FIRST, SYM>(
      R, n_tiles, coef, x, d, slot_dm, slot_mirror, [](int) { return 0; },
      [&](int c, A y, float xc, int) { f(c, y, xc); });
}

}  // namespace gbf
