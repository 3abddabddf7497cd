// Mixed-precision PCG: FP32 inner iterations with FP64 reliable updates.
//
// No reference counterpart: the precision pattern of this solver is FP32
// Amul / preconditioner / vectors, with an FP64 outer residual r = b - A x,
// FP64 solution update and FP64 dot-product reductions.  It follows the
// reliable-update scheme of Sleijpen & van der Vorst ("Reliable updated
// residuals in hybrid Bi-CG methods", Computing 56, 1996), in the mixed
// precision form of Clark et al. (2010): the Krylov recurrence runs in
// FP32; whenever the iterated residual has dropped by `delta` since the last
// update (or below the target), the FP32 correction is folded into the FP64
// solution and the FP32 residual is replaced by the true FP64 residual
// b - A x.  The search direction p is kept, so -- unlike restarted defect
// correction -- no Krylov information is lost.  Convergence is only ever
// declared on a true FP64 residual.
//
// Per inner iteration (four launches; K_true returns at once unless an
// update is due):
//   K_ap   : Ap = A32 p, p.Ap                       -> alpha
//   K_upd  : r -= alpha Ap, z = rD r, r.r, r.z      -> beta, update decision
//            (when an update is due, also fold x64 += x32 + alpha p, x32 = 0)
//   K_true : r64 = b - A64 x64 (reference-order Amul), r = (float) r64,
//            z = rD r, |r64|, r.z                   -> convergence, beta
//   K_p    : x32 += alpha p (unless K_upd folded), p = z + beta p
// The FP32 solution update sits in K_p, which reads p anyway, so K_upd reads
// neither p nor x32 on the iterations without an update (4 bytes per cell
// per iteration less); each x32 element sees the same fmaf sequence as it
// would in K_upd.
// Dot products of FP32 vectors are accumulated per thread in double-float
// arithmetic on the FP32 pipes -- each product split exactly into p + e with
// a fused multiply-add (Dekker's TwoProduct), summed with Knuth's TwoSum --
// and the per-thread (hi, lo) pairs are combined in FP64.  This keeps ~48
// significant bits without issuing FP64 instructions per element (GB300's
// FP64 rate is a small fraction of its FP32 rate).
#include <math.h>
#include <string.h>

#include "bulk.cuh"

namespace gbf {

enum { MP_NORMAL = 0, MP_TRUE_RESIDUAL = 1 };

struct MixedState {
  double rz, alpha, beta, res0, res, rmax, target, pAp;
  int inner, status, n_hist, phase, fold_pending, updates, fault, x_deferred;
  unsigned int ticket[8];
};

struct MixedVecs {
  float *r, *z, *p, *Ap, *xlo, *rD, *d32;
  double* partials;
  MixedState* st;
};

// r64 = b - A64 x64 for cell c; writes r, z; returns r64.
__device__ __forceinline__ double true_residual_cell(const gbf_layout& L,
                                                     const double* __restrict__ coef64,
                                                     const double* __restrict__ diag64,
                                                     const double* __restrict__ b,
                                                     const double* __restrict__ x, int c) {
  const double y = cell_amul<double, double, false>(L, coef64, diag64, x, c, __ldg(x + c));
  return __dsub_rn(__ldg(b + c), y);
}

__global__ void __launch_bounds__(kBlock)
    mp_init_kernel(gbf_layout L, const double* __restrict__ coef64,
                   const double* __restrict__ diag64, const double* __restrict__ pd,
                   const double* __restrict__ b, const double* __restrict__ x, MixedVecs v,
                   double* hist, gbf_solve_params P) {
  __shared__ double sh[kBlock / 32];
  const int G = gridDim.x;
  double rr = 0.0, rz = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < L.n_cells; c += G * blockDim.x) {
    const double rh = true_residual_cell(L, coef64, diag64, b, x, c);
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
    rz += dprod(r, z);
  }
  rr = block_sum(rr, sh);
  rz = block_sum(rz, sh);
  if (threadIdx.x == 0) {
    v.partials[blockIdx.x] = rr;
    v.partials[G + blockIdx.x] = rz;
  }
  if (last_block_done(&v.st->ticket[0])) {
    const double trr = reduce_partials(v.partials, G, sh);
    const double trz = reduce_partials(v.partials + G, G, sh);
    if (threadIdx.x == 0) {
      MixedState* st = v.st;
      const double res = sqrt(trr);
      hist[0] = res;
      st->n_hist = 1;
      st->res0 = res;
      st->res = res;
      st->rmax = res;
      st->rz = trz;
      st->inner = 0;
      st->target = fmax(P.tolerance, P.rel_tol * res);
      const bool conv = (0 >= P.min_iter) &&
                        (res < P.tolerance || (res > 0.0 && res / res < P.rel_tol));
      st->status = conv ? GBF_CONVERGED : (P.max_iter < 1 ? GBF_MAX_ITER : GBF_RUNNING);
    }
  }
}

template <int KIND>
__global__ void __launch_bounds__(kBlock)
    mp_ap_kernel(gbf_layout L, const float* __restrict__ coef32, MixedVecs v) {
  pdl_wait();
  pdl_launch_dependents();
  if (v.st->status != GBF_RUNNING) return;
  __shared__ double sh[kBlock / 32];
  const int G = gridDim.x;
  DFAcc a;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < L.n_cells; c += G * blockDim.x) {
    const float pc = __ldg(v.p + c);
    const float y = cell_amul_k<KIND, float, float, false>(L, coef32, v.d32, v.p, c, pc);
    v.Ap[c] = y;
    a.add_prod(pc, y);
  }
  const double acc = block_sum_df(a, sh);
  if (threadIdx.x == 0) v.partials[blockIdx.x] = acc;
  if (last_block_done(&v.st->ticket[1])) {
    const double pAp = reduce_partials(v.partials, G, sh);
    if (threadIdx.x == 0) {
      MixedState* st = v.st;
      st->pAp = pAp;
      if (fabs(pAp) < 1e-30)
        st->status = GBF_BREAKDOWN;
      else
        st->alpha = st->rz / pAp;
    }
  }
}

// K_ap for a hex 3+3 layout: the coefficient / p / diagonal stream of each
// 256-cell tile is staged in shared memory by bulk asynchronous copies
// (bulk.cuh); the cells of the last, partial tile come from global memory.
// A wait that runs out records st->fault, which the last block turns into
// GBF_DEVICE_TIMEOUT once every block has arrived.
template <bool SYM>
__global__ void __launch_bounds__(kTileCells, kStreamBlocksPerSM)
    mp_ap_stream_kernel(gbf_layout L, const float* __restrict__ coef32, MixedVecs v,
                        int n_tiles) {
  pdl_wait();
  pdl_launch_dependents();
  if (v.st->status != GBF_RUNNING) return;
  __shared__ HexRing<SYM> ring;
  __shared__ double sh[kTileCells / 32];
  const int G = gridDim.x;
  DFAcc a;
  const bool ok = hex_stream_tiles<float, false, SYM>(ring, n_tiles, coef32, v.p, v.d32,
                                                      L.slot_dm, L.slot_mirror,
                                                      [&](int c, float y, float pc) {
                                                   v.Ap[c] = y;
                                                   a.add_prod(pc, y);
                                                 });
  if (blockIdx.x == n_tiles % G) {
    const int c = n_tiles * kTileCells + threadIdx.x;
    if (c < L.n_cells) {
      const float pc = __ldg(v.p + c);
      const float y = SYM ? cell_amul_sym33<float>(L, coef32, v.d32, v.p, c, pc)
                          : cell_amul_fixed<float, float, false, 3, 3>(L, coef32, v.d32, v.p,
                                                                       c, pc);
      v.Ap[c] = y;
      a.add_prod(pc, y);
    }
  }
  if (!ok && threadIdx.x == 0) atomicExch(&v.st->fault, 1);
  const double acc = block_sum_df(a, sh);
  if (threadIdx.x == 0) v.partials[blockIdx.x] = acc;
  if (last_block_done(&v.st->ticket[1])) {
    const double pAp = reduce_partials(v.partials, G, sh);
    if (threadIdx.x == 0) {
      MixedState* st = v.st;
      st->pAp = pAp;
      if (__ldcg(&st->fault))
        st->status = GBF_DEVICE_TIMEOUT;
      else if (fabs(pAp) < 1e-30)
        st->status = GBF_BREAKDOWN;
      else
        st->alpha = st->rz / pAp;
    }
  }
}

// The cell loop of K_upd.  Four cells per thread with 128-bit loads and
// stores of the FP32 vectors (the workspace vectors are 256-byte aligned);
// the n % 4 tail cells one per thread.  FOLD is a template parameter, not a
// branch inside the loop: a branch there is predicated, and its FP64
// conversions and adds then issue on every cell of every iteration (GB300's
// FP64 rate made that the kernel's bound).
template <bool FOLD>
__device__ __forceinline__ void mp_update_cells(int n, double* __restrict__ x, const MixedVecs& v,
                                                float alpha, DFAcc& arr, DFAcc& arz) {
  const int n4 = n >> 2;
  const int stride = gridDim.x * blockDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  float4* __restrict__ xlo4 = reinterpret_cast<float4*>(v.xlo);
  float4* __restrict__ r4 = reinterpret_cast<float4*>(v.r);
  float4* __restrict__ z4 = reinterpret_cast<float4*>(v.z);
  const float4* __restrict__ p4 = reinterpret_cast<const float4*>(v.p);
  const float4* __restrict__ ap4 = reinterpret_cast<const float4*>(v.Ap);
  const float4* __restrict__ rd4 = reinterpret_cast<const float4*>(v.rD);
  const unsigned long long ef = l2_evict_first();
#pragma unroll 2
  for (int q = tid; q < n4; q += stride) {
    // Ap and rD are dead until a later kernel or iteration, r is next read
    // by the next iteration: evict first, keep z (read by K_p next)
    const float4 ap = ld_nc_hint(ap4 + q, ef), rd = ld_nc_hint(rd4 + q, ef);
    float4 r = ld_hint(r4 + q, ef), z;
    if constexpr (FOLD) {
      const float4 pp = p4[q];
      float4 xl = xlo4[q];
      xl.x = fmaf(alpha, pp.x, xl.x);
      xl.y = fmaf(alpha, pp.y, xl.y);
      xl.z = fmaf(alpha, pp.z, xl.z);
      xl.w = fmaf(alpha, pp.w, xl.w);
      const int c = 4 * q;
      x[c] += (double)xl.x;
      x[c + 1] += (double)xl.y;
      x[c + 2] += (double)xl.z;
      x[c + 3] += (double)xl.w;
      xlo4[q] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    r.x = fmaf(-alpha, ap.x, r.x);
    r.y = fmaf(-alpha, ap.y, r.y);
    r.z = fmaf(-alpha, ap.z, r.z);
    r.w = fmaf(-alpha, ap.w, r.w);
    z.x = rd.x * r.x;
    z.y = rd.y * r.y;
    z.z = rd.z * r.z;
    z.w = rd.w * r.w;
    st_hint(r4 + q, r, ef);
    z4[q] = z;
    arr.add_prod(r.x, r.x);
    arr.add_prod(r.y, r.y);
    arr.add_prod(r.z, r.z);
    arr.add_prod(r.w, r.w);
    arz.add_prod(r.x, z.x);
    arz.add_prod(r.y, z.y);
    arz.add_prod(r.z, z.z);
    arz.add_prod(r.w, z.w);
  }
  for (int c = 4 * n4 + tid; c < n; c += stride) {
    if constexpr (FOLD) {
      x[c] += (double)fmaf(alpha, v.p[c], v.xlo[c]);
      v.xlo[c] = 0.0f;
    }
    const float r = fmaf(-alpha, v.Ap[c], v.r[c]);
    const float z = __ldg(v.rD + c) * r;
    v.r[c] = r;
    v.z[c] = z;
    arr.add_prod(r, r);
    arz.add_prod(r, z);
  }
}

__global__ void __launch_bounds__(kBlock)
    mp_update_kernel(int n, double* __restrict__ x, MixedVecs v, double delta,
                     gbf_solve_params P) {
  pdl_wait();
  pdl_launch_dependents();
  if (v.st->status != GBF_RUNNING) return;
  __shared__ double sh[kBlock / 32];
  const int G = gridDim.x;
  const float alpha = (float)v.st->alpha;
  const bool fold = v.st->fold_pending != 0;
  DFAcc arr, arz;
  if (fold)
    mp_update_cells<true>(n, x, v, alpha, arr, arz);
  else
    mp_update_cells<false>(n, x, v, alpha, arr, arz);
  const double rr = block_sum_df(arr, sh);
  const double rz = block_sum_df(arz, sh);
  if (threadIdx.x == 0) {
    v.partials[blockIdx.x] = rr;
    v.partials[G + blockIdx.x] = rz;
  }
  if (last_block_done(&v.st->ticket[2])) {
    const double trr = reduce_partials(v.partials, G, sh);
    const double trz = reduce_partials(v.partials + G, G, sh);
    if (threadIdx.x == 0) {
      MixedState* st = v.st;
      st->inner += 1;
      const double res = sqrt(trr);
      st->res = res;
      st->x_deferred = fold ? 0 : 1;  // K_p adds alpha p to x32
      if (fold) {
        st->fold_pending = 0;
        st->phase = MP_TRUE_RESIDUAL;  // K_true replaces r and sets beta
      } else {
        st->beta = trz / st->rz;
        st->rz = trz;
        st->rmax = fmax(st->rmax, res);
        if (res < delta * st->rmax || res < st->target || st->inner >= P.max_iter)
          st->fold_pending = 1;
      }
    }
  }
}

__global__ void __launch_bounds__(kBlock)
    mp_true_kernel(gbf_layout L, const double* __restrict__ coef64,
                   const double* __restrict__ diag64, const double* __restrict__ b,
                   const double* __restrict__ x, MixedVecs v, double* hist, int hist_cap,
                   gbf_solve_params P) {
  pdl_wait();
  pdl_launch_dependents();
  if (v.st->status != GBF_RUNNING || v.st->phase != MP_TRUE_RESIDUAL) return;
  __shared__ double sh[kBlock / 32];
  const int G = gridDim.x;
  double rr = 0.0, rz = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < L.n_cells; c += G * blockDim.x) {
    const double rh = true_residual_cell(L, coef64, diag64, b, x, c);
    const float r = (float)rh;
    const float z = __ldg(v.rD + c) * r;
    v.r[c] = r;
    v.z[c] = z;
    rr = fma(rh, rh, rr);
    rz += dprod(r, z);
  }
  rr = block_sum(rr, sh);
  rz = block_sum(rz, sh);
  if (threadIdx.x == 0) {
    v.partials[blockIdx.x] = rr;
    v.partials[G + blockIdx.x] = rz;
  }
  if (last_block_done(&v.st->ticket[3])) {
    const double trr = reduce_partials(v.partials, G, sh);
    const double trz = reduce_partials(v.partials + G, G, sh);
    if (threadIdx.x == 0) {
      MixedState* st = v.st;
      const double res = sqrt(trr);
      st->res = res;
      st->updates += 1;
      if (st->n_hist < hist_cap) hist[st->n_hist] = res;
      st->n_hist += 1;
      st->phase = MP_NORMAL;
      const bool conv = st->inner >= P.min_iter &&
                        (res < P.tolerance || (st->res0 > 0.0 && res / st->res0 < P.rel_tol));
      if (conv) {
        st->status = GBF_CONVERGED;
      } else if (st->inner >= P.max_iter) {
        st->status = GBF_MAX_ITER;
      } else {
        st->beta = trz / st->rz;
        st->rz = trz;
        st->rmax = res;
      }
    }
  }
}

// p = z + beta p, after x32 += alpha p with the old p when X (the update
// K_upd left to this kernel).
template <bool X>
__device__ __forceinline__ void mp_p_cells(int n, const MixedVecs& v) {
  const float beta = (float)v.st->beta;
  const float alpha = (float)v.st->alpha;
  const int n4 = n >> 2;
  const int stride = gridDim.x * blockDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  float4* __restrict__ p4 = reinterpret_cast<float4*>(v.p);
  float4* __restrict__ xlo4 = reinterpret_cast<float4*>(v.xlo);
  const float4* __restrict__ z4 = reinterpret_cast<const float4*>(v.z);
  const unsigned long long ef = l2_evict_first();
#pragma unroll 2
  for (int q = tid; q < n4; q += stride) {
    // z is dead after this kernel and x32 is next touched by the next
    // iteration: evict first, keep p (read by the next K_ap)
    float4 p = p4[q];
    const float4 z = ld_nc_hint(z4 + q, ef);
    if constexpr (X) {
      float4 xl = ld_hint(xlo4 + q, ef);
      xl.x = fmaf(alpha, p.x, xl.x);
      xl.y = fmaf(alpha, p.y, xl.y);
      xl.z = fmaf(alpha, p.z, xl.z);
      xl.w = fmaf(alpha, p.w, xl.w);
      st_hint(xlo4 + q, xl, ef);
    }
    p.x = fmaf(beta, p.x, z.x);
    p.y = fmaf(beta, p.y, z.y);
    p.z = fmaf(beta, p.z, z.z);
    p.w = fmaf(beta, p.w, z.w);
    p4[q] = p;
  }
  for (int c = 4 * n4 + tid; c < n; c += stride) {
    const float pc = v.p[c];
    if constexpr (X) v.xlo[c] = fmaf(alpha, pc, v.xlo[c]);
    v.p[c] = fmaf(beta, pc, v.z[c]);
  }
}

__global__ void __launch_bounds__(kBlock) mp_p_kernel(int n, MixedVecs v) {
  pdl_wait();
  pdl_launch_dependents();
  if (v.st->status != GBF_RUNNING) return;
  if (v.st->x_deferred)
    mp_p_cells<true>(n, v);
  else
    mp_p_cells<false>(n, v);
}

// Folds any remaining FP32 correction into x (breakdown / iteration limit;
// after convergence x32 is already zero).
__global__ void mp_fold_kernel(int n, double* __restrict__ x, MixedVecs v) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const float xl = v.xlo[c];
    if (xl != 0.0f) x[c] += (double)xl;
    v.xlo[c] = 0.0f;
  }
}

static size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace gbf

using namespace gbf;

extern "C" size_t gbf_mixed_pcg_workspace_bytes(int32_t n) {
  if (n < 0) return 0;
  return 7 * a256(sizeof(float) * (size_t)n) + a256(sizeof(double) * 2 * kMaxGrid) +
         a256(sizeof(MixedState));
}

extern "C" int gbf_mixed_pcg_solve(const gbf_layout* L, const double* coef64,
                                   const double* diag64, const float* coef32,
                                   int32_t coef32_sym, const double* pd, const double* b, double* x, double delta,
                                   double* hist, int32_t hist_cap, const gbf_solve_params* P,
                                   gbf_solve_result* R, void* ws, size_t ws_bytes,
                                   void* stream) {
  ::gbf::NvtxScope nvtx_("gbf_mixed_pcg_solve");
  int rc = check_layout(L);
  if (rc) return rc;
  GBF_REQUIRE(P && R, "mixed_pcg: NULL params/result");
  GBF_REQUIRE(P->max_iter >= 0, "mixed_pcg: negative max_iter");
  GBF_REQUIRE(delta > 0.0 && delta < 1.0, "mixed_pcg: delta must be in (0, 1), got %g", delta);
  const int n = L->n_cells;
  memset(R, 0, sizeof(*R));
  if (n == 0) {
    const bool conv = (0 >= P->min_iter) && (0.0 < P->tolerance);
    R->iterations = 1;
    R->status = conv ? GBF_CONVERGED : (P->max_iter < 1 ? GBF_MAX_ITER : GBF_BREAKDOWN);
    return GBF_OK;
  }
  GBF_REQUIRE(diag64 && b && x && hist && hist_cap >= 1 && ws &&
                  (L->n_faces == 0 || (coef64 && coef32)),
              "mixed_pcg: NULL pointer");
  GBF_REQUIRE(ws_bytes >= gbf_mixed_pcg_workspace_bytes(n), "mixed_pcg: workspace too small");
  const bool sym = coef32_sym != 0 && L->n_faces > 0;
  GBF_REQUIRE(!sym || layout_sym_ok(*L),
              "mixed_pcg: coef32_sym needs a hex 3+3 layout with a mirror table");
  cudaStream_t s = as_stream(stream);
  char* w = static_cast<char*>(ws);
  const size_t vb = a256(sizeof(float) * (size_t)n);
  MixedVecs v;
  float** vecs[7] = {&v.r, &v.z, &v.p, &v.Ap, &v.xlo, &v.rD, &v.d32};
  for (int i = 0; i < 7; ++i) *vecs[i] = reinterpret_cast<float*>(w + i * vb);
  v.partials = reinterpret_cast<double*>(w + 7 * vb);
  v.st = reinterpret_cast<MixedState*>(w + 7 * vb + a256(sizeof(double) * 2 * kMaxGrid));

  // one full wave of resident blocks per kernel (each reduces its own partials)
  const int Gi = wave_grid(mp_init_kernel, kBlock, n);
  const bool hex = layout_kind(*L) == kLayoutHex33;
  // staged K_ap: hex layout, 16-byte aligned coefficient / vector streams
  // (the workspace vectors are 256-byte aligned)
  const bool staged = hex && hex_stream_aligned(coef32, ws, ws, L->slot_dm) &&
                      (!sym || (kSymStaged &&
                                (reinterpret_cast<uintptr_t>(L->slot_mirror) & 15u) == 0));
  const int n_tiles = n / kTileCells;
  const long long tile_work = (long long)(n_tiles > 0 ? n_tiles : 1) * kTileCells;
  const int Ga = staged ? (sym ? wave_grid(mp_ap_stream_kernel<true>, kTileCells, tile_work)
                               : wave_grid(mp_ap_stream_kernel<false>, kTileCells, tile_work))
                 : sym  ? wave_grid(mp_ap_kernel<kLayoutHex33Sym>, kBlock, n)
                 : hex  ? wave_grid(mp_ap_kernel<kLayoutHex33>, kBlock, n)
                        : wave_grid(mp_ap_kernel<kLayoutGeneric>, kBlock, n);
  const int Ba = staged ? kTileCells : kBlock;
  const int Gu = wave_grid(mp_update_kernel, kBlock, (n + 3) / 4);
  const int Gt = wave_grid(mp_true_kernel, kBlock, n);
  const int Gp = wave_grid(mp_p_kernel, kBlock, (n + 3) / 4);
  const int G = wave_grid(mp_fold_kernel, kBlock, n);
  GBF_CHECK_CUDA(cudaMemsetAsync(v.st, 0, sizeof(MixedState), s));
  mp_init_kernel<<<Gi, kBlock, 0, s>>>(*L, coef64, diag64, pd, b, x, v, hist, *P);
  GBF_CHECK_LAUNCH();
  const int chunk = P->check_every > 0 ? P->check_every : 32;
  MixedState hs;
  GBF_CHECK_CUDA(cudaMemcpyAsync(&hs, v.st, sizeof(hs), cudaMemcpyDeviceToHost, s));
  GBF_CHECK_CUDA(cudaStreamSynchronize(s));
  // bounded: every launched iteration advances `inner` until max_iter, where
  // a fold + true residual ends the solve (at most max_iter + 2 iterations)
  int launched = 0;
  const int limit = P->max_iter + 2;
  while (hs.status == GBF_RUNNING && launched < limit) {
    for (int j = 0; j < chunk && launched < limit; ++j, ++launched) {
      // every kernel of the iteration is a programmatic dependent launch of
      // the previous one; one K_ap launch in eight is bracketed by events
      // for the timing probe (an event between two kernels serialises them)
      const bool tb = (launched % 8 == 0) && timing_begin(kProbeMixedAp, s);
      const gbf_layout Lv = *L;
      cudaError_t e;
      if (staged && sym)
        e = launch_pdl(mp_ap_stream_kernel<true>, Ga, Ba, s, Lv, coef32, v, n_tiles);
      else if (staged)
        e = launch_pdl(mp_ap_stream_kernel<false>, Ga, Ba, s, Lv, coef32, v, n_tiles);
      else if (sym)
        e = launch_pdl(mp_ap_kernel<kLayoutHex33Sym>, Ga, Ba, s, Lv, coef32, v);
      else if (hex)
        e = launch_pdl(mp_ap_kernel<kLayoutHex33>, Ga, Ba, s, Lv, coef32, v);
      else
        e = launch_pdl(mp_ap_kernel<kLayoutGeneric>, Ga, Ba, s, Lv, coef32, v);
      if (tb) timing_end(kProbeMixedAp, s);
      if (e == cudaSuccess) e = launch_pdl(mp_update_kernel, Gu, kBlock, s, n, x, v, delta, *P);
      if (e == cudaSuccess)
        e = launch_pdl(mp_true_kernel, Gt, kBlock, s, Lv, coef64, diag64, b,
                       static_cast<const double*>(x), v, hist, hist_cap, *P);
      if (e == cudaSuccess) e = launch_pdl(mp_p_kernel, Gp, kBlock, s, n, v);
      GBF_CHECK_CUDA(e);
    }
    GBF_CHECK_LAUNCH();
    GBF_CHECK_CUDA(cudaMemcpyAsync(&hs, v.st, sizeof(hs), cudaMemcpyDeviceToHost, s));
    GBF_CHECK_CUDA(cudaStreamSynchronize(s));
  }
  mp_fold_kernel<<<G, kBlock, 0, s>>>(n, x, v);
  GBF_CHECK_LAUNCH();
  R->iterations = hs.inner + 1;
  R->status = (hs.status == GBF_RUNNING) ? GBF_MAX_ITER : hs.status;
  R->final_residual = hs.res;
  R->initial_residual = hs.res0;
  R->inner_iterations = hs.inner;
  R->outer_updates = hs.updates;
  R->launches = 2 + 4 * launched;
  return GBF_OK;
}
