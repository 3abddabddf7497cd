// Batched mixed-precision PCG: many independent systems (of uneven sizes)
// solved together, every kernel covering all systems at once.
//
// No reference counterpart.  The systems are concatenated into one
// block-diagonal LDU layout (each system's cells padded to a multiple of 32,
// so no 32-cell slice straddles two systems).  Work is cut into tiles: a
// tile is a contiguous cell range of ONE system and is processed by one CTA,
// so every CTA reduces into its own system's partial sums; the last tile of
// a system to finish (per-system ticket) reduces that system's partials in
// tile order and advances that system's scalar recurrence.  Systems
// converge independently; tiles of finished systems return at once
// (per-system convergence mask).  The iteration is the reliable-update
// mixed-precision PCG of mixed.cu (FP32 inner iterations, FP64 true
// residuals; x32 += alpha p in the p kernel, the L2 evict-first policies of
// its vector kernels), and a chunk of iterations is captured once into a
// CUDA graph and replayed until every system has finished.
#include <math.h>
#include <string.h>

#include "amul.cuh"
#include "barrier.cuh"

namespace gbf {

struct BState {
  double rz, alpha, beta, res0, res, rmax, target, pAp;
  int inner, status, phase, fold_pending, updates, x_deferred;
  unsigned int ticket[6];
};

// Batch-wide control words, in the last 256 bytes of the workspace: the
// number of systems still iterating, the "some system folds this
// iteration" flag of the persistent form, its tile queue and its grid
// barrier.
struct BCtl {
  int running;
  int fold;
  unsigned int queue;  // tiles taken so far (wraps; only differences are used)
  int pad;
  GridBarrier bar;
};

struct BVecs {
  float *r, *z, *p, *Ap, *xlo, *rD, *d32;
  double* partials;   // [2 * n_tiles]
  BState* st;         // [n_systems]
  int* running;       // systems still iterating
  BCtl* ctl;
};

struct BTiles {
  int n_systems, n_tiles;
  const int32_t* tile_sys;
  const int32_t* tile_begin;
  const int32_t* tile_end;
  const int32_t* sys_tile0;  // [n_systems + 1]
};

using BDFAcc = DFAcc;

// Loads of data another block may have rewritten earlier in the same launch
// (COH: the persistent form, where no kernel boundary separates writer and
// reader) go to L2; the per-phase kernels use the plain or read-only paths.
template <bool COH, typename T>
__device__ __forceinline__ T ldc(const T* p) {
  if constexpr (COH)
    return __ldcg(p);
  else
    return *p;
}

template <bool COH>
__device__ __forceinline__ float ldv_ro(const float* p, unsigned long long ef) {
  if constexpr (COH) {
    float v;
    asm volatile("ld.global.cg.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(ef));
    return v;
  } else {
    return ld_nc_hint(p, ef);
  }
}

template <bool COH>
__device__ __forceinline__ float ldv_rw(const float* p, unsigned long long ef) {
  if constexpr (COH) {
    float v;
    asm volatile("ld.global.cg.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(ef));
    return v;
  } else {
    return ld_hint(p, ef);
  }
}

// The system's status, read once by thread 0 and shared with the block, so
// that every thread of a tile takes the same branch.
template <bool COH>
__device__ __forceinline__ int tile_status(const BState* st) {
  __shared__ int s_status;
  __syncthreads();
  if (threadIdx.x == 0) s_status = ldc<COH>(&st->status);
  __syncthreads();
  return s_status;
}

// True in every thread of the tile that finished last among its system's
// tiles (count = number of tiles of the system); resets the ticket.
__device__ __forceinline__ bool last_tile_of_system(unsigned int* ticket, int count) {
  __shared__ bool am_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) am_last = (atomicAdd(ticket, 1u) == (unsigned)(count - 1));
  __syncthreads();
  if (am_last) {
    __threadfence();
    if (threadIdx.x == 0) *ticket = 0u;
  }
  return am_last;
}

template <int BS>
__device__ __forceinline__ double tile_sum(const double* partials, int t0, int t1, double* sh) {
  double v = 0.0;
  for (int i = t0 + threadIdx.x; i < t1; i += BS) v += __ldcg(partials + i);
  return block_sum(v, sh);
}

__device__ __forceinline__ bool b_converged(double res, double res0, int it,
                                            const gbf_solve_params& P) {
  if (it < P.min_iter) return false;
  if (res < P.tolerance) return true;
  return res0 > 0.0 && res / res0 < P.rel_tol;
}

template <int BS>
__global__ void __launch_bounds__(BS)
    bmp_init_kernel(gbf_layout L, BTiles T, const double* __restrict__ coef64,
                    const double* __restrict__ diag64, const double* __restrict__ pd,
                    const double* __restrict__ b, const double* __restrict__ x, BVecs v,
                    gbf_solve_params P) {
  __shared__ double sh[BS / 32];
  const int tile = blockIdx.x;
  const int s = __ldg(T.tile_sys + tile);
  double rr = 0.0, rz = 0.0;
  for (int c = __ldg(T.tile_begin + tile) + threadIdx.x; c < __ldg(T.tile_end + tile); c += BS) {
    const double y = cell_amul<double, double, false>(L, coef64, diag64, x, c, __ldg(x + c));
    const double rh = __dsub_rn(__ldg(b + c), y);
    const float rD = pd ? (float)(1.0 / __ldg(pd + c)) : 1.0f;
    const float r = (float)rh;
    const float z = rD * r;
    v.rD[c] = rD;
    v.d32[c] = (float)__ldg(diag64 + c);
    v.r[c] = r;
    v.z[c] = z;
    v.p[c] = z;
    v.xlo[c] = 0.0f;
    rr = fma(rh, rh, rr);
    rz += (double)r * (double)z;
  }
  rr = block_sum(rr, sh);
  rz = block_sum(rz, sh);
  if (threadIdx.x == 0) {
    v.partials[tile] = rr;
    v.partials[T.n_tiles + tile] = rz;
  }
  const int t0 = __ldg(T.sys_tile0 + s), t1 = __ldg(T.sys_tile0 + s + 1);
  BState* st = v.st + s;
  if (last_tile_of_system(&st->ticket[0], t1 - t0)) {
    const double trr = tile_sum<BS>(v.partials, t0, t1, sh);
    const double trz = tile_sum<BS>(v.partials + T.n_tiles, t0, t1, sh);
    if (threadIdx.x == 0) {
      const double res = sqrt(trr);
      st->res0 = res;
      st->res = res;
      st->rmax = res;
      st->rz = trz;
      st->target = fmax(P.tolerance, P.rel_tol * res);
      const bool conv = (0 >= P.min_iter) && (res < P.tolerance || (res > 0.0 && 1.0 < P.rel_tol));
      st->status = conv ? GBF_CONVERGED : (P.max_iter < 1 ? GBF_MAX_ITER : GBF_RUNNING);
      if (st->status != GBF_RUNNING) atomicSub(v.running, 1);
    }
  }
}

// ---- one tile of each phase of the iteration --------------------------------
// Ap = A p (FP32), p.Ap; the system's last tile forms alpha (or breakdown).
// TPC threads per cell: 1, or 2 -- the even thread of a pair sums the
// owner-side slots, the odd one the neighbour-side slots, and the even one
// forms (diag * p + owner sum) + neighbour sum, the one-thread order.  A tile
// is a multiple of 32 cells long and a warp covers 16 consecutive cells per
// step, so every lane of a warp runs the same number of steps (the pair
// shuffle takes the full mask).
template <int BS, int KIND, bool COH, int TPC>
__device__ __forceinline__ void bmp_ap_tile(const gbf_layout& L, const BTiles& T, int tile,
                                            const float* __restrict__ coef32, const BVecs& v,
                                            double* sh) {
  static_assert(TPC == 1 || TPC == 2, "one or two threads per cell");
  const int s = __ldg(T.tile_sys + tile);
  BState* st = v.st + s;
  if (tile_status<COH>(st) != GBF_RUNNING) return;
  BDFAcc a;
  const int c_end = __ldg(T.tile_end + tile);
  if constexpr (TPC == 1) {
    for (int c = __ldg(T.tile_begin + tile) + threadIdx.x; c < c_end; c += BS) {
      const float pc = COH ? __ldcg(v.p + c) : __ldg(v.p + c);
      const float y = cell_amul_k<KIND, float, float, false, COH>(L, coef32, v.d32, v.p, c, pc);
      v.Ap[c] = y;
      a.add_prod(pc, y);
    }
  } else {
    const int side = threadIdx.x & 1;
    for (int c = __ldg(T.tile_begin + tile) + (threadIdx.x >> 1); c < c_end; c += BS / 2) {
      const float part = cell_side_sum<KIND, float, float, COH>(L, coef32, v.p, c, side);
      const float sn = __shfl_down_sync(0xffffffffu, part, 1);
      if (side == 0) {
        const float pc = COH ? __ldcg(v.p + c) : __ldg(v.p + c);
        float y = mul_rn(__ldg(v.d32 + c), pc);
        if (L.n_faces > 0) {
          y = add_rn(y, part);
          y = add_rn(y, sn);
        }
        v.Ap[c] = y;
        a.add_prod(pc, y);
      }
    }
  }
  const double acc = block_sum_df(a, sh);
  if (threadIdx.x == 0) v.partials[tile] = acc;
  const int t0 = __ldg(T.sys_tile0 + s), t1 = __ldg(T.sys_tile0 + s + 1);
  if (last_tile_of_system(&st->ticket[1], t1 - t0)) {
    const double pAp = tile_sum<BS>(v.partials, t0, t1, sh);
    if (threadIdx.x == 0) {
      st->pAp = pAp;
      if (fabs(pAp) < 1e-30) {
        st->status = GBF_BREAKDOWN;
        atomicSub(v.running, 1);
      } else {
        st->alpha = ldc<COH>(&st->rz) / pAp;
      }
    }
  }
}

// The cell loop of the batched K_upd for one tile.  FOLD is a template
// parameter, not a branch inside the loop: a branch there is predicated, and
// its FP64 conversion and add then issue on every cell of every iteration.
template <int BS, bool FOLD, bool COH>
__device__ __forceinline__ void bmp_update_cells(const BTiles& T, int tile,
                                                 double* __restrict__ x, const BVecs& v,
                                                 float alpha, BDFAcc& arr, BDFAcc& arz) {
  const unsigned long long ef = l2_evict_first();
  for (int c = __ldg(T.tile_begin + tile) + threadIdx.x; c < __ldg(T.tile_end + tile); c += BS) {
    if constexpr (FOLD) {
      x[c] = ldc<COH>(x + c) + (double)fmaf(alpha, ldc<COH>(v.p + c), ldc<COH>(v.xlo + c));
      v.xlo[c] = 0.0f;
    }
    const float r = fmaf(-alpha, ldv_ro<COH>(v.Ap + c, ef), ldv_rw<COH>(v.r + c, ef));
    const float z = ld_nc_hint(v.rD + c, ef) * r;  // rD: written before this launch
    st_hint(v.r + c, r, ef);
    v.z[c] = z;
    arr.add_prod(r, r);
    arz.add_prod(r, z);
  }
}

// r -= alpha Ap, z = M^-1 r, r.r, r.z; the last tile forms beta or, when a
// reliable update is due, marks the system for the FP64 true residual.
// Returns true in every thread when this tile's system folds.
template <int BS, bool COH>
__device__ __forceinline__ void bmp_update_tile(const BTiles& T, int tile, double* __restrict__ x,
                                                const BVecs& v, double delta,
                                                const gbf_solve_params& P, double* sh) {
  const int s = __ldg(T.tile_sys + tile);
  BState* st = v.st + s;
  if (tile_status<COH>(st) != GBF_RUNNING) return;
  const float alpha = (float)ldc<COH>(&st->alpha);
  const bool fold = ldc<COH>(&st->fold_pending) != 0;
  BDFAcc arr, arz;
  if (fold)
    bmp_update_cells<BS, true, COH>(T, tile, x, v, alpha, arr, arz);
  else
    bmp_update_cells<BS, false, COH>(T, tile, x, v, alpha, arr, arz);
  const double rr = block_sum_df(arr, sh);
  const double rz = block_sum_df(arz, sh);
  if (threadIdx.x == 0) {
    v.partials[tile] = rr;
    v.partials[T.n_tiles + tile] = rz;
  }
  const int t0 = __ldg(T.sys_tile0 + s), t1 = __ldg(T.sys_tile0 + s + 1);
  if (last_tile_of_system(&st->ticket[2], t1 - t0)) {
    const double trr = tile_sum<BS>(v.partials, t0, t1, sh);
    const double trz = tile_sum<BS>(v.partials + T.n_tiles, t0, t1, sh);
    if (threadIdx.x == 0) {
      const int inner = ldc<COH>(&st->inner) + 1;
      st->inner = inner;
      const double res = sqrt(trr);
      st->res = res;
      st->x_deferred = fold ? 0 : 1;  // the p phase adds alpha p to x32
      if (fold) {
        st->fold_pending = 0;
        st->phase = 1;
        if (COH) v.ctl->fold = 1;
      } else {
        st->beta = trz / ldc<COH>(&st->rz);
        st->rz = trz;
        const double rmax = fmax(ldc<COH>(&st->rmax), res);
        st->rmax = rmax;
        if (res < delta * rmax || res < ldc<COH>(&st->target) || inner >= P.max_iter)
          st->fold_pending = 1;
      }
    }
  }
}

// FP64 true residual r = b - A x of a system that has just folded x32 into
// x; the last tile applies the convergence rules to it.
template <int BS, bool COH>
__device__ __forceinline__ void bmp_true_tile(const gbf_layout& L, const BTiles& T, int tile,
                                              const double* __restrict__ coef64,
                                              const double* __restrict__ diag64,
                                              const double* __restrict__ b,
                                              const double* __restrict__ x, const BVecs& v,
                                              const gbf_solve_params& P, double* sh) {
  const int s = __ldg(T.tile_sys + tile);
  BState* st = v.st + s;
  {
    __shared__ int s_go;
    __syncthreads();
    if (threadIdx.x == 0)
      s_go = ldc<COH>(&st->status) == GBF_RUNNING && ldc<COH>(&st->phase) == 1;
    __syncthreads();
    if (!s_go) return;
  }
  double rr = 0.0, rz = 0.0;
  for (int c = __ldg(T.tile_begin + tile) + threadIdx.x; c < __ldg(T.tile_end + tile); c += BS) {
    const double xc = COH ? __ldcg(x + c) : __ldg(x + c);
    const double y = cell_amul<double, double, false, COH>(L, coef64, diag64, x, c, xc);
    const double rh = __dsub_rn(__ldg(b + c), y);
    const float r = (float)rh;
    const float z = __ldg(v.rD + c) * r;
    v.r[c] = r;
    v.z[c] = z;
    rr = fma(rh, rh, rr);
    rz += (double)r * (double)z;
  }
  rr = block_sum(rr, sh);
  rz = block_sum(rz, sh);
  if (threadIdx.x == 0) {
    v.partials[tile] = rr;
    v.partials[T.n_tiles + tile] = rz;
  }
  const int t0 = __ldg(T.sys_tile0 + s), t1 = __ldg(T.sys_tile0 + s + 1);
  if (last_tile_of_system(&st->ticket[3], t1 - t0)) {
    const double trr = tile_sum<BS>(v.partials, t0, t1, sh);
    const double trz = tile_sum<BS>(v.partials + T.n_tiles, t0, t1, sh);
    if (threadIdx.x == 0) {
      const double res = sqrt(trr);
      const int inner = ldc<COH>(&st->inner);
      st->res = res;
      st->updates = ldc<COH>(&st->updates) + 1;
      st->phase = 0;
      if (b_converged(res, ldc<COH>(&st->res0), inner, P)) {
        st->status = GBF_CONVERGED;
        atomicSub(v.running, 1);
      } else if (inner >= P.max_iter) {
        st->status = GBF_MAX_ITER;
        atomicSub(v.running, 1);
      } else {
        st->beta = trz / ldc<COH>(&st->rz);
        st->rz = trz;
        st->rmax = res;
      }
    }
  }
}

// p = z + beta p (and x32 += alpha p when the update phase deferred it).
template <int BS, bool COH>
__device__ __forceinline__ void bmp_p_tile(const BTiles& T, int tile, const BVecs& v) {
  const BState* st = v.st + __ldg(T.tile_sys + tile);
  __shared__ float s_ab[2];
  __shared__ int s_flags[2];
  __syncthreads();
  if (threadIdx.x == 0) {
    s_flags[0] = ldc<COH>(&st->status);
    s_flags[1] = ldc<COH>(&st->x_deferred);
    s_ab[0] = (float)ldc<COH>(&st->beta);
    s_ab[1] = (float)ldc<COH>(&st->alpha);
  }
  __syncthreads();
  if (s_flags[0] != GBF_RUNNING) return;
  const float beta = s_ab[0], alpha = s_ab[1];
  const bool xd = s_flags[1] != 0;
  const unsigned long long ef = l2_evict_first();
  for (int c = __ldg(T.tile_begin + tile) + threadIdx.x; c < __ldg(T.tile_end + tile); c += BS) {
    const float pc = ldc<COH>(v.p + c);
    if (xd) st_hint(v.xlo + c, fmaf(alpha, pc, ldv_rw<COH>(v.xlo + c, ef)), ef);
    v.p[c] = fmaf(beta, pc, ldv_ro<COH>(v.z + c, ef));
  }
}

template <int BS, bool COH>
__device__ __forceinline__ void bmp_fold_tile(const BTiles& T, int tile, double* __restrict__ x,
                                              const BVecs& v) {
  for (int c = __ldg(T.tile_begin + tile) + threadIdx.x; c < __ldg(T.tile_end + tile); c += BS) {
    const float xl = ldc<COH>(v.xlo + c);
    if (xl != 0.0f) x[c] = ldc<COH>(x + c) + (double)xl;
    v.xlo[c] = 0.0f;
  }
}

// ---- the per-phase kernels: one tile per CTA --------------------------------
template <int BS, int KIND, int TPC>
__global__ void __launch_bounds__(BS)
    bmp_ap_kernel(gbf_layout L, BTiles T, const float* __restrict__ coef32, BVecs v) {
  __shared__ double sh[BS / 32];
  bmp_ap_tile<BS, KIND, false, TPC>(L, T, blockIdx.x, coef32, v, sh);
}

template <int BS>
__global__ void __launch_bounds__(BS)
    bmp_update_kernel(BTiles T, double* __restrict__ x, BVecs v, double delta,
                      gbf_solve_params P) {
  __shared__ double sh[BS / 32];
  bmp_update_tile<BS, false>(T, blockIdx.x, x, v, delta, P, sh);
}

template <int BS>
__global__ void __launch_bounds__(BS)
    bmp_true_kernel(gbf_layout L, BTiles T, const double* __restrict__ coef64,
                    const double* __restrict__ diag64, const double* __restrict__ b,
                    const double* __restrict__ x, BVecs v, gbf_solve_params P) {
  __shared__ double sh[BS / 32];
  bmp_true_tile<BS, false>(L, T, blockIdx.x, coef64, diag64, b, x, v, P, sh);
}

template <int BS>
__global__ void __launch_bounds__(BS) bmp_p_kernel(BTiles T, BVecs v) {
  bmp_p_tile<BS, false>(T, blockIdx.x, v);
}

template <int BS>
__global__ void __launch_bounds__(BS) bmp_fold_kernel(BTiles T, double* __restrict__ x, BVecs v) {
  bmp_fold_tile<BS, false>(T, blockIdx.x, x, v);
}

// ---- the persistent form: every iteration of every system in one launch ----
//
// All CTAs are resident (cooperative launch).  Each phase walks the tiles of
// the systems still running: every CTA holds, in shared memory, the prefix
// sums of the running systems' tile counts, takes active tile blockIdx.x
// first and then further active tiles from the batch's tile queue, so that a
// CTA whose tiles ran short takes more (see for_active_tiles).  The phases
// are separated by the bounded grid barrier.  The map of running systems is rebuilt in the p phase, the
// one phase in which no status changes (statuses change only at the end of
// the Amul phase -- breakdown -- and of the true-residual phase), so every
// CTA builds the same map; a system that stops later in the iteration keeps
// its tiles in the map and they return at once.  The true-residual phase and
// its barrier run only in iterations where some system folds (a flag set in
// the update phase, read after its barrier).  The loop ends when the map is
// empty -- a decision every CTA takes from the same map.
constexpr int kPersistentMaxSystems = 4096;

template <int BS>
__device__ __forceinline__ int build_active_map(const BTiles& T, const BVecs& v, int* pref) {
  // pref[i] = tiles of running systems before system i (exclusive scan of
  // per-system counts); returns the total.
  const int S = T.n_systems;
  const int per = (S + BS - 1) / BS;
  const int i0 = threadIdx.x * per;
  int local = 0;
  for (int i = i0; i < i0 + per && i < S; ++i) {
    const int cnt = (__ldcg(&v.st[i].status) == GBF_RUNNING)
                        ? (__ldg(T.sys_tile0 + i + 1) - __ldg(T.sys_tile0 + i))
                        : 0;
    pref[i] = cnt;
    local += cnt;
  }
  // block exclusive scan of the per-thread sums
  __shared__ int wsum[BS / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int incl = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) wsum[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int w = lane < BS / 32 ? wsum[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    if (lane < BS / 32) wsum[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  int run = (wid > 0 ? wsum[wid - 1] : 0) + incl - local;
  for (int i = i0; i < i0 + per && i < S; ++i) {
    const int cnt = pref[i];
    pref[i] = run;
    run += cnt;
  }
  const int total = wsum[BS / 32 - 1];
  if (threadIdx.x == 0) pref[S] = total;
  __syncthreads();
  return total;
}

// Active tile t -> tile index (pref as built above; systems with no active
// tiles have pref[i] == pref[i+1]).
__device__ __forceinline__ int active_tile(const BTiles& T, const int* pref, int t) {
  int lo = 0, hi = T.n_systems - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (pref[mid + 1] > t)
      hi = mid;
    else
      lo = mid + 1;
  }
  return __ldg(T.sys_tile0 + lo) + (t - pref[lo]);
}

// Runs body(t) for the active tiles t < nact of one phase on this CTA: tile
// blockIdx.x, then the tiles G + k that the queue hands out, k counted from
// the queue's value when the phase began (base).  Thread 0 takes the next
// ticket before the current tile starts, so the atomic's round trip hides
// behind the tile.  Every CTA that ran a tile takes exactly one ticket that
// comes back >= nact, and one that did not run any takes none, so a phase
// takes exactly nact tickets whatever the timing: every CTA advances base by
// nact and the next phase starts from the same value without a reset.  The
// grid barrier between phases orders one phase's tickets before the next's.
// Which CTA runs a tile never changes its result: the tile's partial sums
// and the per-system scalars that the last tile of a system forms are
// summed in a fixed order.
template <typename Body>
__device__ __forceinline__ void for_active_tiles(unsigned int* queue, unsigned int& base, int nact,
                                                 Body&& body) {
  __shared__ int s_next[2];  // double-buffered: one barrier per tile
  const int G = (int)gridDim.x;
  int t = (int)blockIdx.x, k = 0;
  while (t < nact) {
    unsigned int ticket = 0u;
    if (threadIdx.x == 0) ticket = atomicAdd(queue, 1u);
    body(t);
    if (threadIdx.x == 0) s_next[k] = G + (int)(ticket - base);
    __syncthreads();
    t = s_next[k];
    k ^= 1;
  }
  base += (unsigned int)nact;
}

// Compiled for 1536 resident threads per SM (40 registers): with every
// phase's registers in one kernel it would otherwise hold 62 and run 1024.
template <int BS, int KIND, int TPC>
__global__ void __launch_bounds__(BS, 1536 / BS)
    bmp_persistent_kernel(gbf_layout L, BTiles T, const double* __restrict__ coef64,
                          const double* __restrict__ diag64, const float* __restrict__ coef32,
                          const double* __restrict__ b, double* __restrict__ x, BVecs v,
                          double delta, gbf_solve_params P) {
  extern __shared__ int pref[];  // [n_systems + 1]
  __shared__ double sh[BS / 32];
  const unsigned G = gridDim.x;
  GridBarrier* bar = &v.ctl->bar;
  // statuses were set by the init kernel (a separate launch); the barrier
  // keeps them unchanged until every CTA has built the same first map
  int nact = build_active_map<BS>(T, v, pref);
  if (!grid_barrier(bar, G)) return;
  unsigned int* queue = &v.ctl->queue;
  unsigned int base = 0u;  // the init kernel zeroed the queue
  const long long cap = (long long)P.max_iter + 4;
  for (long long it = 0; nact > 0 && it < cap; ++it) {
    for_active_tiles(queue, base, nact, [&](int t) {
      bmp_ap_tile<BS, KIND, true, TPC>(L, T, active_tile(T, pref, t), coef32, v, sh);
    });
    if (!grid_barrier(bar, G)) return;
    for_active_tiles(queue, base, nact, [&](int t) {
      bmp_update_tile<BS, true>(T, active_tile(T, pref, t), x, v, delta, P, sh);
    });
    if (!grid_barrier(bar, G)) return;
    if (__ldcg(&v.ctl->fold) != 0) {
      for_active_tiles(queue, base, nact, [&](int t) {
        bmp_true_tile<BS, true>(L, T, active_tile(T, pref, t), coef64, diag64, b, x, v, P, sh);
      });
      if (!grid_barrier(bar, G)) return;
    }
    // p phase: no status changes here, so every CTA rebuilds the same map
    nact = build_active_map<BS>(T, v, pref);
    if (blockIdx.x == 0 && threadIdx.x == 0) v.ctl->fold = 0;  // read by all before this phase
    for_active_tiles(queue, base, nact,
                     [&](int t) { bmp_p_tile<BS, true>(T, active_tile(T, pref, t), v); });
    if (!grid_barrier(bar, G)) return;
  }
  // fold the FP32 corrections left in x32 into x (every tile once)
  for (int t = blockIdx.x; t < T.n_tiles; t += G) bmp_fold_tile<BS, true>(T, t, x, v);
}

static size_t b256(size_t b) { return (b + 255) & ~(size_t)255; }

// Control words at the start of a solve: every system running, no fold
// flag, the grid barrier's counter and fault word at zero.
__global__ void bmp_ctl_init_kernel(BCtl* ctl, int n_systems) {
  ctl->running = n_systems;
  ctl->fold = 0;
  ctl->queue = 0u;
  ctl->pad = 0;
  ctl->bar.count = 0ull;
  ctl->bar.fault = 0;
  ctl->bar.pad = 0;
}

template <int BS, int TPC>
static int launch_iteration(cudaStream_t s, int nt, const gbf_layout& L, const BTiles& T,
                            const double* coef64, const double* diag64, const float* coef32,
                            const double* b, double* x, const BVecs& v, double delta,
                            const gbf_solve_params& P, bool probe) {
  const bool tb = probe && timing_begin(kProbeBatchedAp, s);
  GBF_LAYOUT_DISPATCH(L, K, bmp_ap_kernel<BS, K, TPC><<<nt, BS, 0, s>>>(L, T, coef32, v));
  if (tb) timing_end(kProbeBatchedAp, s);
  bmp_update_kernel<BS><<<nt, BS, 0, s>>>(T, x, v, delta, P);
  bmp_true_kernel<BS><<<nt, BS, 0, s>>>(L, T, coef64, diag64, b, x, v, P);
  bmp_p_kernel<BS><<<nt, BS, 0, s>>>(T, v);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

// Resident CTAs of the persistent kernel (occupancy x SMs, at most one per
// tile); 0 when it cannot be launched cooperatively.
template <int BS, int KIND, int TPC>
static int persistent_grid(int n_systems, int n_tiles) {
  int dev = 0, sms = 0, coop = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop)
    return 0;
  const size_t shm = sizeof(int) * (size_t)(n_systems + 1);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bmp_persistent_kernel<BS, KIND, TPC>,
                                                    BS, shm) != cudaSuccess ||
      per_sm <= 0)
    return 0;
  long long g = (long long)per_sm * sms;
  if (g > n_tiles) g = n_tiles;
  return g < 1 ? 1 : (int)g;
}

template <int BS, int KIND, int TPC>
static cudaError_t launch_persistent(int grid, cudaStream_t s, const gbf_layout& L,
                                     const BTiles& T, const double* coef64, const double* diag64,
                                     const float* coef32, const double* b, double* x,
                                     const BVecs& v, double delta, const gbf_solve_params& P) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(BS);
  cfg.dynamicSmemBytes = sizeof(int) * (size_t)(T.n_systems + 1);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, bmp_persistent_kernel<BS, KIND, TPC>, L, T, coef64, diag64,
                            coef32, b, x, v, delta, P);
}

// Per-system results from the state blocks.
static int read_results(const BVecs& v, int S, int launches, gbf_solve_result* R,
                        cudaStream_t s) {
  BState* hs = new BState[S];
  cudaError_t e = cudaMemcpyAsync(hs, v.st, sizeof(BState) * (size_t)S, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    delete[] hs;
    set_error("batched_pcg: %s", cudaGetErrorString(e));
    return GBF_ERR_CUDA;
  }
  for (int i = 0; i < S; ++i) {
    memset(R + i, 0, sizeof(gbf_solve_result));
    R[i].iterations = hs[i].inner + 1;
    R[i].status = hs[i].status == GBF_RUNNING ? GBF_MAX_ITER : hs[i].status;
    R[i].final_residual = hs[i].res;
    R[i].initial_residual = hs[i].res0;
    R[i].inner_iterations = hs[i].inner;
    R[i].outer_updates = hs[i].updates;
    R[i].launches = launches;
  }
  delete[] hs;
  return GBF_OK;
}

// The persistent form: control words, the init kernel and one cooperative
// launch for every iteration of every system (optionally captured together
// in a CUDA graph and replayed once).
template <int BS, int KIND, int TPC>
static int batched_solve_persistent(const gbf_layout* L, const BTiles& T, const double* coef64,
                                    const double* diag64, const float* coef32, const double* pd,
                                    const double* b, double* x, double delta,
                                    const gbf_solve_params* P, bool graph_capture,
                                    gbf_solve_result* R, const BVecs& v, cudaStream_t s) {
  const int S = T.n_systems, nt = T.n_tiles;
  GBF_REQUIRE(S <= kPersistentMaxSystems,
              "batched_pcg: the persistent form takes at most %d systems (got %d)",
              kPersistentMaxSystems, S);
  const int G = persistent_grid<BS, KIND, TPC>(S, nt);
  GBF_REQUIRE(G > 0, "batched_pcg: the device cannot run the persistent form");
  auto enqueue = [&](cudaStream_t q) -> cudaError_t {
    cudaError_t e = cudaMemsetAsync(v.st, 0, sizeof(BState) * (size_t)S, q);
    if (e != cudaSuccess) return e;
    bmp_ctl_init_kernel<<<1, 1, 0, q>>>(v.ctl, S);
    bmp_init_kernel<BS><<<nt, BS, 0, q>>>(*L, T, coef64, diag64, pd, b, x, v, *P);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_persistent<BS, KIND, TPC>(G, q, *L, T, coef64, diag64, coef32, b, x, v, delta,
                                            *P);
  };
  if (graph_capture) {
    cudaStream_t cap = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    GBF_CHECK_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    cudaError_t e1 = (e == cudaSuccess) ? enqueue(cap) : e;
    cudaError_t e2 = cudaStreamEndCapture(cap, &graph);
    if (e == cudaSuccess) e = e1 != cudaSuccess ? e1 : e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (e == cudaSuccess) e = cudaGraphLaunch(exec, s);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cap);
    if (e != cudaSuccess) {
      set_error("batched_pcg: persistent graph: %s", cudaGetErrorString(e));
      return GBF_ERR_CUDA;
    }
  } else {
    cudaError_t e = enqueue(s);
    if (e != cudaSuccess) {
      set_error("batched_pcg: persistent launch: %s", cudaGetErrorString(e));
      return GBF_ERR_CUDA;
    }
  }
  BCtl hc;
  GBF_CHECK_CUDA(cudaMemcpyAsync(&hc, v.ctl, sizeof(hc), cudaMemcpyDeviceToHost, s));
  int rc = read_results(v, S, 3, R, s);
  if (rc) return rc;
  if (hc.bar.fault) {
    // a barrier wait ran out: the iterations stopped where they were
    for (int i = 0; i < S; ++i) R[i].status = GBF_DEVICE_TIMEOUT;
  }
  return GBF_OK;
}

template <int BS, int TPC>
static int batched_solve(const gbf_layout* L, const BTiles& T, const double* coef64,
                         const double* diag64, const float* coef32, const double* pd,
                         const double* b, double* x, double delta, const gbf_solve_params* P,
                         int form, gbf_solve_result* R, const BVecs& v, cudaStream_t s) {
  const bool use_graph = (form & 1) != 0;
  if (form & 2) {
    if (layout_kind(*L) == kLayoutHex33)
      return batched_solve_persistent<BS, kLayoutHex33, TPC>(L, T, coef64, diag64, coef32, pd, b,
                                                             x, delta, P, use_graph, R, v, s);
    return batched_solve_persistent<BS, kLayoutGeneric, TPC>(L, T, coef64, diag64, coef32, pd, b,
                                                             x, delta, P, use_graph, R, v, s);
  }
  const int nt = T.n_tiles;
  const int S = T.n_systems;
  GBF_CHECK_CUDA(cudaMemsetAsync(v.st, 0, sizeof(BState) * (size_t)S, s));
  bmp_ctl_init_kernel<<<1, 1, 0, s>>>(v.ctl, S);
  bmp_init_kernel<BS><<<nt, BS, 0, s>>>(*L, T, coef64, diag64, pd, b, x, v, *P);
  GBF_CHECK_LAUNCH();
  const int chunk = P->check_every > 0 ? P->check_every : 16;
  const int limit = P->max_iter + 2;
  int launched = 0, running = S, launches = 2;
  GBF_CHECK_CUDA(cudaMemcpyAsync(&running, v.running, sizeof(int), cudaMemcpyDeviceToHost, s));
  GBF_CHECK_CUDA(cudaStreamSynchronize(s));

  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  cudaStream_t cap = nullptr;
  if (use_graph && running > 0) {
    // capture one chunk on a private stream; launches then go to `s`
    GBF_CHECK_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    int rc = GBF_OK;
    for (int j = 0; j < chunk && e == cudaSuccess && rc == GBF_OK; ++j)
      rc = launch_iteration<BS, TPC>(cap, nt, *L, T, coef64, diag64, coef32, b, x, v, delta, *P,
                                     false);
    cudaError_t e2 = cudaStreamEndCapture(cap, &graph);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess && rc == GBF_OK) e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess || rc != GBF_OK) {
      if (graph) cudaGraphDestroy(graph);
      cudaStreamDestroy(cap);
      set_error("batched_pcg: graph capture failed: %s", cudaGetErrorString(e));
      return GBF_ERR_CUDA;
    }
  }
  int rc = GBF_OK;
  while (running > 0 && launched < limit) {
    if (exec) {
      cudaError_t e = cudaGraphLaunch(exec, s);
      if (e != cudaSuccess) {
        set_error("batched_pcg: graph launch failed: %s", cudaGetErrorString(e));
        rc = GBF_ERR_CUDA;
        break;
      }
    } else {
      for (int j = 0; j < chunk; ++j) {
        rc = launch_iteration<BS, TPC>(s, nt, *L, T, coef64, diag64, coef32, b, x, v, delta, *P,
                                       true);
        if (rc) break;
      }
      if (rc) {
        set_error("batched_pcg: launch failed");
        break;
      }
    }
    launched += chunk;
    launches += 4 * chunk;
    cudaError_t e = cudaMemcpyAsync(&running, v.running, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      set_error("batched_pcg: %s", cudaGetErrorString(e));
      rc = GBF_ERR_CUDA;
      break;
    }
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (cap) cudaStreamDestroy(cap);
  if (rc) return rc;
  bmp_fold_kernel<BS><<<nt, BS, 0, s>>>(T, x, v);
  GBF_CHECK_LAUNCH();
  launches += 1;
  return read_results(v, S, launches, R, s);
}

}  // namespace gbf

using namespace gbf;

extern "C" size_t gbf_batched_mixed_pcg_workspace_bytes(int32_t n, int32_t n_systems,
                                                        int32_t n_tiles) {
  if (n < 0 || n_systems < 0 || n_tiles < 0) return 0;
  return 7 * b256(sizeof(float) * (size_t)n) + b256(sizeof(double) * 2 * (size_t)n_tiles) +
         b256(sizeof(BState) * (size_t)n_systems) + b256(sizeof(BCtl));
}

extern "C" int gbf_batched_mixed_pcg_solve(const gbf_layout* L, const gbf_batch* B,
                                           const double* coef64, const double* diag64,
                                           const float* coef32, const double* pd,
                                           const double* b, double* x, double delta,
                                           const gbf_solve_params* P, int32_t block_size,
                                           int32_t form, gbf_solve_result* R, void* ws,
                                           size_t ws_bytes, void* stream) {
  ::gbf::NvtxScope nvtx_("gbf_batched_mixed_pcg_solve");
  int rc = check_layout(L);
  if (rc) return rc;
  GBF_REQUIRE(B && P && R, "batched_pcg: NULL batch/params/result");
  GBF_REQUIRE(B->n_systems >= 1 && B->n_tiles >= B->n_systems, "batched_pcg: bad batch sizes");
  GBF_REQUIRE(B->tile_sys && B->tile_begin && B->tile_end && B->sys_tile0,
              "batched_pcg: NULL tile arrays");
  GBF_REQUIRE(delta > 0.0 && delta < 1.0, "batched_pcg: delta must be in (0, 1)");
  GBF_REQUIRE(P->max_iter >= 0, "batched_pcg: negative max_iter");
  GBF_REQUIRE(block_size == 128 || block_size == 256 || block_size == 512,
              "batched_pcg: block_size must be 128, 256 or 512 (got %d)", block_size);
  GBF_REQUIRE(form >= 0 && form <= 7,
              "batched_pcg: form must be 0..7 (bits 0-1 the launch form, bit 2 two threads "
              "per cell; got %d)", form);
  const int n = L->n_cells;
  GBF_REQUIRE(diag64 && b && x && ws && (L->n_faces == 0 || (coef64 && coef32)),
              "batched_pcg: NULL pointer");
  GBF_REQUIRE(ws_bytes >= gbf_batched_mixed_pcg_workspace_bytes(n, B->n_systems, B->n_tiles),
              "batched_pcg: workspace too small");
  char* w = static_cast<char*>(ws);
  const size_t vb = b256(sizeof(float) * (size_t)n);
  BVecs v;
  float** vecs[7] = {&v.r, &v.z, &v.p, &v.Ap, &v.xlo, &v.rD, &v.d32};
  for (int i = 0; i < 7; ++i) *vecs[i] = reinterpret_cast<float*>(w + i * vb);
  size_t off = 7 * vb;
  v.partials = reinterpret_cast<double*>(w + off);
  off += b256(sizeof(double) * 2 * (size_t)B->n_tiles);
  v.st = reinterpret_cast<BState*>(w + off);
  off += b256(sizeof(BState) * (size_t)B->n_systems);
  v.ctl = reinterpret_cast<BCtl*>(w + off);
  v.running = &v.ctl->running;
  BTiles T{B->n_systems, B->n_tiles, B->tile_sys, B->tile_begin, B->tile_end, B->sys_tile0};
  cudaStream_t s = as_stream(stream);
  const int f = form & 3;
  const bool pair = (form & 4) != 0;
#define GBF_BATCHED_CASE(BSZ)                                                                  \
  return pair ? batched_solve<BSZ, 2>(L, T, coef64, diag64, coef32, pd, b, x, delta, P, f, R, \
                                      v, s)                                                    \
              : batched_solve<BSZ, 1>(L, T, coef64, diag64, coef32, pd, b, x, delta, P, f, R, \
                                      v, s)
  switch (block_size) {
    case 128:
      GBF_BATCHED_CASE(128);
    case 512:
      GBF_BATCHED_CASE(512);
    default:
      GBF_BATCHED_CASE(256);
  }
#undef GBF_BATCHED_CASE
}
