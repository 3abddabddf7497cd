// Mixed-precision preconditioned BiCGStab: FP32 inner iterations with FP64
// reliable updates.
//
// No reference counterpart: this is the precision pattern applied to the
// momentum solve of PBiCGSTABSolver (solvers/pbicgstab.py:103-239), whose
// iteration it keeps -- y = p / d_M, v = A y, s = r - alpha v, z = s / d_M,
// t = A z, x += alpha y + omega z, r = s - omega t, p = r + beta (p - omega v),
// with the reference's breakdown tests (rho, r~.v, the t.t branch, omega).
// Vectors, the Amul and the preconditioner apply run in FP32; the solution
// is x64 + x32, where the FP32 correction x32 is folded into the FP64
// solution whenever the iterated residual has dropped by `delta` since the
// last update (or below the target), and the FP32 residual is then replaced
// by the true residual b - A64 x64 (residual replacement with group update,
// van der Vorst & Ye, SIAM J. Sci. Comput. 22, 2000; Sleijpen & van der
// Vorst, Computing 56, 1996).  p, r~ and rho are kept, so the Krylov space
// survives an update.  Convergence is declared on a true FP64 residual
// only; the half-step check on s of the FP64 solver is not taken.
//
// Per inner iteration (six launches, each a programmatic dependent launch
// of the one before; K_true returns at once unless an update is due):
//   K_v    : v = A32 y, r~.v                      -> alpha
//   K_s    : s = r - alpha v, z = s / d_M, x32 += alpha y
//   K_t    : t = A32 z, t.t, t.s (or t.z)         -> omega or the t.t branch
//   K_r    : x32 += omega z (folded into x64 when an update is pending),
//            r = s - omega t, r.r, r~.r           -> beta, update decision
//   K_true : r64 = b - A64 x64 (reference-order Amul), r = (float) r64,
//            |r64|, r~.r                           -> convergence, beta
//   K_p    : p = r + beta (p - omega v), y = p / d_M
// Dot products of FP32 vectors use the double-float accumulator DFAcc
// (error-free products and sums on the FP32 pipes) and FP64 block sums.
#include <math.h>
#include <string.h>

#include "barrier.cuh"
#include "bulk.cuh"

namespace gbf {

enum { MB_NORMAL = 0, MB_TRUE_RESIDUAL = 1 };

struct MbState {
  double rho, alpha, omega, beta, res0, res, rmax, target;
  int inner, status, n_hist, phase, fold_pending, updates, fault, branch;
  unsigned int ticket[8];
};

struct MbVecs {
  float *r, *rt, *p, *v, *y, *s, *z, *t, *xlo, *rD, *d32;
  float *p2, *v2;  // the fused form's second p and v buffers (iteration parity)
  double* partials;
  MbState* st;
};

__device__ __forceinline__ bool mb_converged(double res, double res0, int iter,
                                             const gbf_solve_params& P) {
  if (iter < P.min_iter) return false;
  if (res < P.tolerance) return true;
  return res0 > 0.0 && res / res0 < P.rel_tol;
}

__global__ void __launch_bounds__(kBlock)
    mb_init_kernel(gbf_layout L, const double* __restrict__ coef64,
                   const double* __restrict__ diag64, const double* __restrict__ pd,
                   const double* __restrict__ b, const double* __restrict__ x, MbVecs v,
                   double* hist, gbf_solve_params P) {
  __shared__ double sh[kBlock / 32];
  const int G = gridDim.x;
  double rr = 0.0;
  DFAcc a;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < L.n_cells; c += G * blockDim.x) {
    const double y = cell_amul<double, double, false>(L, coef64, diag64, x, c, __ldg(x + c));
    const double rh = __dsub_rn(__ldg(b + c), y);
    const float rD = pd ? (float)(1.0 / __ldg(pd + c)) : 1.0f;
    const float r = (float)rh;
    v.rD[c] = rD;
    v.d32[c] = (float)__ldg(diag64 + c);
    v.r[c] = r;
    v.rt[c] = r;
    v.p[c] = r;
    v.y[c] = rD * r;
    v.v[c] = 0.0f;
    v.xlo[c] = 0.0f;
    rr = fma(rh, rh, rr);
    a.add_prod(r, r);
  }
  rr = block_sum(rr, sh);
  const double rho = block_sum_df(a, sh);
  if (threadIdx.x == 0) {
    v.partials[blockIdx.x] = rr;
    v.partials[G + blockIdx.x] = rho;
  }
  if (last_block_done(&v.st->ticket[0])) {
    const double trr = reduce_partials(v.partials, G, sh);
    const double trho = reduce_partials(v.partials + G, G, sh);
    if (threadIdx.x == 0) {
      MbState* st = v.st;
      const double res = sqrt(trr);
      hist[0] = res;
      st->n_hist = 1;
      st->res0 = res;
      st->res = res;
      st->rmax = res;
      st->rho = trho;
      st->inner = 0;
      st->target = fmax(P.tolerance, P.rel_tol * res);
      if (mb_converged(res, res, 0, P))
        st->status = GBF_CONVERGED;
      else if (P.max_iter < 1)
        st->status = GBF_MAX_ITER;
      else if (fabs(trho) < 1e-30)
        st->status = GBF_BREAKDOWN;  // pbicgstab.py:154-157
      else
        st->status = GBF_RUNNING;
    }
  }
}

// The second operand of the Amul kernels' dot products for cell c: r~[c]
// (PH 0) or, for the standard omega, s[c] (PH 1; the reference's t.z uses
// the multiplied vector itself).
template <int PH>
__device__ __forceinline__ float mb_amul_aux(const MbVecs& v, int c, int standard_omega) {
  if constexpr (PH == 0)
    return __ldg(v.rt + c);
  else
    return standard_omega ? __ldg(v.s + c) : 0.0f;
}

// Epilogue of the two Amul kernels, cell c: PH 0 stores v and accumulates
// r~.v; PH 1 stores t and accumulates t.t and t.s (standard) or t.z.
template <int PH>
__device__ __forceinline__ void mb_amul_cell(const MbVecs& v, int c, float yv, float xc,
                                             float aux, int standard_omega, DFAcc& a0,
                                             DFAcc& a1) {
  if constexpr (PH == 0) {
    v.v[c] = yv;
    a0.add_prod(aux, yv);
  } else {
    v.t[c] = yv;
    a0.add_prod(yv, yv);
    a1.add_prod(yv, standard_omega ? aux : xc);
  }
}

// Block sums and the last block's scalar step of the two Amul kernels.
template <int PH>
__device__ __forceinline__ void mb_amul_finish(const MbVecs& v, const DFAcc& a0,
                                               const DFAcc& a1, double* sh) {
  const int G = gridDim.x;
  const double s0 = block_sum_df(a0, sh);
  double s1 = 0.0;
  if constexpr (PH == 1) s1 = block_sum_df(a1, sh);
  if (threadIdx.x == 0) {
    v.partials[blockIdx.x] = s0;
    if constexpr (PH == 1) v.partials[G + blockIdx.x] = s1;
  }
  if (last_block_done(&v.st->ticket[1 + PH])) {
    const double t0 = reduce_partials(v.partials, G, sh);
    double t1 = 0.0;
    if constexpr (PH == 1) t1 = reduce_partials(v.partials + G, G, sh);
    if (threadIdx.x == 0) {
      MbState* st = v.st;
      if (__ldcg(&st->fault)) {
        st->status = GBF_DEVICE_TIMEOUT;
      } else if constexpr (PH == 0) {
        if (fabs(t0) < 1e-30)
          st->status = GBF_BREAKDOWN;  // pbicgstab.py:168-171
        else
          st->alpha = st->rho / t0;
      } else {
        if (fabs(t0) < 1e-30) {
          st->branch = 1;  // pbicgstab.py:196-208
        } else {
          st->branch = 0;
          st->omega = t1 / t0;
        }
      }
    }
  }
}

// v = A32 y (PH 0) or t = A32 z (PH 1), generic or hex 3+3 gather.
template <int PH, int KIND>
__global__ void __launch_bounds__(kBlock)
    mb_amul_kernel(gbf_layout L, const float* __restrict__ coef32, MbVecs v, int standard_omega) {
  pdl_wait();
  pdl_launch_dependents();
  if (v.st->status != GBF_RUNNING) return;
  __shared__ double sh[kBlock / 32];
  const float* __restrict__ src = PH == 0 ? v.y : v.z;
  DFAcc a0, a1;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < L.n_cells;
       c += gridDim.x * blockDim.x) {
    const float aux = mb_amul_aux<PH>(v, c, standard_omega);
    const float xc = __ldg(src + c);
    const float yv = cell_amul_k<KIND, float, float, false>(L, coef32, v.d32, src, c, xc);
    mb_amul_cell<PH>(v, c, yv, xc, aux, standard_omega, a0, a1);
  }
  mb_amul_finish<PH>(v, a0, a1, sh);
}

// The same for a hex 3+3 layout with 16-byte aligned streams: each 256-cell
// tile's coefficients, vector and diagonal are staged in shared memory by
// bulk asynchronous copies (bulk.cuh); the cells of the last, partial tile
// come from global memory.  A wait that runs out records st->fault, which
// the last block turns into GBF_DEVICE_TIMEOUT.
template <int PH>
__global__ void __launch_bounds__(kTileCells, kStreamBlocksPerSM)
    mb_amul_stream_kernel(gbf_layout L, const float* __restrict__ coef32, MbVecs v,
                          int n_tiles, int standard_omega) {
  pdl_wait();
  pdl_launch_dependents();
  if (v.st->status != GBF_RUNNING) return;
  __shared__ HexRing<false> ring;
  __shared__ double sh[kTileCells / 32];
  const float* __restrict__ src = PH == 0 ? v.y : v.z;
  DFAcc a0, a1;
  const bool ok = hex_stream_tiles_pre<float, false, false>(
      ring, n_tiles, coef32, src, v.d32, L.slot_dm, nullptr,
      [&](int c) { return mb_amul_aux<PH>(v, c, standard_omega); },
      [&](int c, float yv, float xc, float aux) {
        mb_amul_cell<PH>(v, c, yv, xc, aux, standard_omega, a0, a1);
      });
  if (blockIdx.x == n_tiles % gridDim.x) {
    const int c = n_tiles * kTileCells + threadIdx.x;
    if (c < L.n_cells) {
      const float aux = mb_amul_aux<PH>(v, c, standard_omega);
      const float xc = __ldg(src + c);
      const float yv = cell_amul_fixed<float, float, false, 3, 3>(L, coef32, v.d32, src, c, xc);
      mb_amul_cell<PH>(v, c, yv, xc, aux, standard_omega, a0, a1);
    }
  }
  if (!ok && threadIdx.x == 0) atomicExch(&v.st->fault, 1);
  mb_amul_finish<PH>(v, a0, a1, sh);
}

// s = r - alpha v, z = s / d_M, x32 += alpha y.  Four cells per thread with
// 128-bit accesses (the workspace vectors are 256-byte aligned), then the
// n % 4 tail one cell per thread.
__global__ void __launch_bounds__(kBlock) mb_s_kernel(int n, MbVecs v) {
  pdl_wait();
  pdl_launch_dependents();
  if (v.st->status != GBF_RUNNING) return;
  const float alpha = (float)v.st->alpha;
  const int n4 = n >> 2;
  const int stride = gridDim.x * blockDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const float4* __restrict__ r4 = reinterpret_cast<const float4*>(v.r);
  const float4* __restrict__ v4 = reinterpret_cast<const float4*>(v.v);
  const float4* __restrict__ y4 = reinterpret_cast<const float4*>(v.y);
  const float4* __restrict__ rd4 = reinterpret_cast<const float4*>(v.rD);
  float4* __restrict__ s4 = reinterpret_cast<float4*>(v.s);
  float4* __restrict__ z4 = reinterpret_cast<float4*>(v.z);
  float4* __restrict__ x4 = reinterpret_cast<float4*>(v.xlo);
#pragma unroll 2
  for (int q = tid; q < n4; q += stride) {
    const float4 r = r4[q], vv = v4[q], y = y4[q], rd = __ldg(rd4 + q);
    float4 xl = x4[q], s, z;
    s.x = fmaf(-alpha, vv.x, r.x);
    s.y = fmaf(-alpha, vv.y, r.y);
    s.z = fmaf(-alpha, vv.z, r.z);
    s.w = fmaf(-alpha, vv.w, r.w);
    z.x = rd.x * s.x;
    z.y = rd.y * s.y;
    z.z = rd.z * s.z;
    z.w = rd.w * s.w;
    xl.x = fmaf(alpha, y.x, xl.x);
    xl.y = fmaf(alpha, y.y, xl.y);
    xl.z = fmaf(alpha, y.z, xl.z);
    xl.w = fmaf(alpha, y.w, xl.w);
    s4[q] = s;
    z4[q] = z;
    x4[q] = xl;
  }
  for (int c = 4 * n4 + tid; c < n; c += stride) {
    const float s = fmaf(-alpha, v.v[c], v.r[c]);
    v.s[c] = s;
    v.z[c] = __ldg(v.rD + c) * s;
    v.xlo[c] = fmaf(alpha, v.y[c], v.xlo[c]);
  }
}

// One cell of K_r: the new x32 (folded into x64 when FOLD) and r.
template <bool FOLD>
__device__ __forceinline__ float mb_r_cell(double* __restrict__ x, int c, int branch, float omega,
                                           float s, float t, float z, float& xl) {
  float r = s;
  if (branch == 0) {
    xl = fmaf(omega, z, xl);
    r = fmaf(-omega, t, s);
  }
  if constexpr (FOLD) {
    x[c] += (double)xl;
    xl = 0.0f;
  }
  return r;
}

// The cell loop of K_r, four cells per thread with 128-bit accesses, then
// the n % 4 tail.  FOLD is a template parameter, not a branch inside the
// loop: a branch there is predicated, and its FP64 conversions and adds then
// issue on every cell of every iteration (measured: FP64 pipe 62 % busy).
template <bool FOLD>
__device__ __forceinline__ void mb_r_cells(int n, double* __restrict__ x, const MbVecs& v,
                                           int branch, float omega, DFAcc& arr, DFAcc& artr) {
  const int n4 = n >> 2;
  const int stride = gridDim.x * blockDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const float4* __restrict__ s4 = reinterpret_cast<const float4*>(v.s);
  const float4* __restrict__ t4 = reinterpret_cast<const float4*>(v.t);
  const float4* __restrict__ z4 = reinterpret_cast<const float4*>(v.z);
  const float4* __restrict__ rt4 = reinterpret_cast<const float4*>(v.rt);
  float4* __restrict__ r4 = reinterpret_cast<float4*>(v.r);
  float4* __restrict__ x4 = reinterpret_cast<float4*>(v.xlo);
#pragma unroll 2
  for (int q = tid; q < n4; q += stride) {
    const float4 s = s4[q], t = t4[q], z = z4[q], rt = __ldg(rt4 + q);
    float4 xl = x4[q], r;
    const int c = 4 * q;
    r.x = mb_r_cell<FOLD>(x, c, branch, omega, s.x, t.x, z.x, xl.x);
    r.y = mb_r_cell<FOLD>(x, c + 1, branch, omega, s.y, t.y, z.y, xl.y);
    r.z = mb_r_cell<FOLD>(x, c + 2, branch, omega, s.z, t.z, z.z, xl.z);
    r.w = mb_r_cell<FOLD>(x, c + 3, branch, omega, s.w, t.w, z.w, xl.w);
    r4[q] = r;
    x4[q] = xl;
    arr.add_prod(r.x, r.x);
    arr.add_prod(r.y, r.y);
    arr.add_prod(r.z, r.z);
    arr.add_prod(r.w, r.w);
    artr.add_prod(rt.x, r.x);
    artr.add_prod(rt.y, r.y);
    artr.add_prod(rt.z, r.z);
    artr.add_prod(rt.w, r.w);
  }
  for (int c = 4 * n4 + tid; c < n; c += stride) {
    float xl = v.xlo[c];
    const float r = mb_r_cell<FOLD>(x, c, branch, omega, v.s[c], v.t[c], v.z[c], xl);
    v.r[c] = r;
    v.xlo[c] = xl;
    arr.add_prod(r, r);
    artr.add_prod(__ldg(v.rt + c), r);
  }
}

__global__ void __launch_bounds__(kBlock)
    mb_r_kernel(int n, double* __restrict__ x, MbVecs v, double delta, gbf_solve_params P) {
  pdl_wait();
  pdl_launch_dependents();
  if (v.st->status != GBF_RUNNING) return;
  __shared__ double sh[kBlock / 32];
  const int G = gridDim.x;
  const int branch = v.st->branch;
  const float omega = (float)v.st->omega;
  const bool fold = v.st->fold_pending != 0;
  DFAcc arr, artr;
  if (fold)
    mb_r_cells<true>(n, x, v, branch, omega, arr, artr);
  else
    mb_r_cells<false>(n, x, v, branch, omega, arr, artr);
  const double rr = block_sum_df(arr, sh);
  const double rtr = block_sum_df(artr, sh);
  if (threadIdx.x == 0) {
    v.partials[blockIdx.x] = rr;
    v.partials[G + blockIdx.x] = rtr;
  }
  if (last_block_done(&v.st->ticket[3])) {
    const double trr = reduce_partials(v.partials, G, sh);
    const double trtr = reduce_partials(v.partials + G, G, sh);
    if (threadIdx.x == 0) {
      MbState* st = v.st;
      st->inner += 1;
      const double res = sqrt(trr);
      st->res = res;
      if (branch == 0 && fabs(st->omega) < 1e-30) {
        st->status = GBF_BREAKDOWN;  // pbicgstab.py:227-229
      } else if (fold) {
        st->fold_pending = 0;
        st->phase = MB_TRUE_RESIDUAL;  // K_true replaces r and sets beta
      } else {
        st->beta = branch == 0 ? (trtr / st->rho) * (st->alpha / st->omega)
                               : (trtr / st->rho) * st->alpha;
        st->rho = trtr;
        st->rmax = fmax(st->rmax, res);
        if (res < delta * st->rmax || res < st->target || st->inner >= P.max_iter)
          st->fold_pending = 1;
        else if (fabs(trtr) < 1e-30)
          st->status = GBF_BREAKDOWN;  // the next iteration's rho test
      }
    }
  }
}

__global__ void __launch_bounds__(kBlock)
    mb_true_kernel(gbf_layout L, const double* __restrict__ coef64,
                   const double* __restrict__ diag64, const double* __restrict__ b,
                   const double* __restrict__ x, MbVecs v, double* hist, int hist_cap,
                   gbf_solve_params P) {
  pdl_wait();
  pdl_launch_dependents();
  if (v.st->status != GBF_RUNNING || v.st->phase != MB_TRUE_RESIDUAL) return;
  __shared__ double sh[kBlock / 32];
  const int G = gridDim.x;
  double rr = 0.0;
  DFAcc artr;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < L.n_cells; c += G * blockDim.x) {
    const double y = cell_amul<double, double, false>(L, coef64, diag64, x, c, __ldg(x + c));
    const double rh = __dsub_rn(__ldg(b + c), y);
    const float r = (float)rh;
    v.r[c] = r;
    rr = fma(rh, rh, rr);
    artr.add_prod(__ldg(v.rt + c), r);
  }
  rr = block_sum(rr, sh);
  const double rtr = block_sum_df(artr, sh);
  if (threadIdx.x == 0) {
    v.partials[blockIdx.x] = rr;
    v.partials[G + blockIdx.x] = rtr;
  }
  if (last_block_done(&v.st->ticket[4])) {
    const double trr = reduce_partials(v.partials, G, sh);
    const double trtr = reduce_partials(v.partials + G, G, sh);
    if (threadIdx.x == 0) {
      MbState* st = v.st;
      const double res = sqrt(trr);
      st->res = res;
      st->updates += 1;
      if (st->n_hist < hist_cap) hist[st->n_hist] = res;
      st->n_hist += 1;
      st->phase = MB_NORMAL;
      if (mb_converged(res, st->res0, st->inner, P)) {
        st->status = GBF_CONVERGED;
      } else if (st->inner >= P.max_iter) {
        st->status = GBF_MAX_ITER;
      } else {
        st->beta = st->branch == 0 ? (trtr / st->rho) * (st->alpha / st->omega)
                                   : (trtr / st->rho) * st->alpha;
        st->rho = trtr;
        st->rmax = res;
        if (fabs(trtr) < 1e-30) st->status = GBF_BREAKDOWN;
      }
    }
  }
}

// p = r + beta (p - omega v) (t.t branch: r + beta (p - v)), y = p / d_M.
__global__ void __launch_bounds__(kBlock) mb_p_kernel(int n, MbVecs v) {
  pdl_wait();
  pdl_launch_dependents();
  if (v.st->status != GBF_RUNNING) return;
  const float beta = (float)v.st->beta;
  const float omega = v.st->branch == 0 ? (float)v.st->omega : 1.0f;
  const int n4 = n >> 2;
  const int stride = gridDim.x * blockDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const float4* __restrict__ r4 = reinterpret_cast<const float4*>(v.r);
  const float4* __restrict__ v4 = reinterpret_cast<const float4*>(v.v);
  const float4* __restrict__ rd4 = reinterpret_cast<const float4*>(v.rD);
  float4* __restrict__ p4 = reinterpret_cast<float4*>(v.p);
  float4* __restrict__ y4 = reinterpret_cast<float4*>(v.y);
#pragma unroll 2
  for (int q = tid; q < n4; q += stride) {
    const float4 r = r4[q], vv = v4[q], rd = __ldg(rd4 + q);
    float4 p = p4[q], y;
    p.x = fmaf(beta, fmaf(-omega, vv.x, p.x), r.x);
    p.y = fmaf(beta, fmaf(-omega, vv.y, p.y), r.y);
    p.z = fmaf(beta, fmaf(-omega, vv.z, p.z), r.z);
    p.w = fmaf(beta, fmaf(-omega, vv.w, p.w), r.w);
    y.x = rd.x * p.x;
    y.y = rd.y * p.y;
    y.z = rd.z * p.z;
    y.w = rd.w * p.w;
    p4[q] = p;
    y4[q] = y;
  }
  for (int c = 4 * n4 + tid; c < n; c += stride) {
    const float p = fmaf(beta, fmaf(-omega, v.v[c], v.p[c]), v.r[c]);
    v.p[c] = p;
    v.y[c] = __ldg(v.rD + c) * p;
  }
}

// ---------------------------------------------------------------------------
// The fused form (hex 3+3 layouts): three kernels per iteration, one per
// reduction, instead of five vector and Amul passes.  The p update of an
// iteration moves into the next iteration's v = A y kernel, and the s / z
// update into the t = A z kernel; the multiplied vector's values at
// neighbour cells (y, z) are formed there from the stored vectors instead of
// read -- with the same fmaf sequences as the per-phase kernels, so every
// element has the bits it has there.  p and v are double-buffered by
// iteration parity: the v = A y kernel reads the old p and v at neighbour
// cells while it writes the new ones.
// ---------------------------------------------------------------------------

// (A w)[c] on a hex 3+3 layout for a vector w that is not stored: wq(q)
// forms w at cell q.  The products and summation order of
// cell_amul_fixed<float, float, false, 3, 3>.
template <typename WQ>
__device__ __forceinline__ float hex33_amul_formed(const gbf_layout& L,
                                                   const float* __restrict__ coef,
                                                   const float* __restrict__ diag, int c,
                                                   float wc, WQ&& wq) {
  constexpr int W = 6;
  const int sl = c >> 5, lane = c & 31;
  const int base = 32 * W * sl + lane;
  const int4* __restrict__ dm4 = reinterpret_cast<const int4*>(L.slot_dm) + (W / 2) * sl;
  int d[W];
  unsigned m[W];
#pragma unroll
  for (int q = 0; q < W / 2; ++q) {
    const int4 e = __ldg(dm4 + q);
    d[2 * q] = e.x;
    m[2 * q] = (unsigned)e.y;
    d[2 * q + 1] = e.z;
    m[2 * q + 1] = (unsigned)e.w;
  }
  float a[W], xv[W];
  bool on[W];
  const unsigned long long ef = l2_evict_first();
#pragma unroll
  for (int k = 0; k < W; ++k) a[k] = ld_nc_hint(coef + base + 32 * k, ef);
#pragma unroll
  for (int k = 0; k < W; ++k) {
    on[k] = (m[k] >> lane) & 1u;
    xv[k] = on[k] ? wq(c + d[k]) : 0.0f;
  }
  float so = 0.0f, sn = 0.0f;
  if (on[0]) so = first_term(mul_rn(a[0], xv[0]));
#pragma unroll
  for (int k = 1; k < 3; ++k)
    if (on[k]) so = add_rn(so, mul_rn(a[k], xv[k]));
  if (on[3]) sn = first_term(mul_rn(a[3], xv[3]));
#pragma unroll
  for (int k = 4; k < W; ++k)
    if (on[k]) sn = add_rn(sn, mul_rn(a[k], xv[k]));
  float y = mul_rn(__ldg(diag + c), wc);
  y = add_rn(y, so);
  return add_rn(y, sn);
}

// p = r + beta (p_old - omega v_old) (t.t branch: omega = 1), y = p / d_M,
// v = A32 y, r~.v -> alpha.  In the first iteration beta = 0, so p = r.
__global__ void __launch_bounds__(kBlock)
    mb_pv_kernel(gbf_layout L, const float* __restrict__ coef32, MbVecs v, int parity) {
  pdl_wait();
  pdl_launch_dependents();
  if (v.st->status != GBF_RUNNING) return;
  __shared__ double sh[kBlock / 32];
  const float beta = (float)v.st->beta;
  const float omega = v.st->branch == 0 ? (float)v.st->omega : 1.0f;
  const float* __restrict__ po = parity ? v.p2 : v.p;
  const float* __restrict__ vo = parity ? v.v2 : v.v;
  float* __restrict__ pn = parity ? v.p : v.p2;
  float* __restrict__ vn = parity ? v.v : v.v2;
  const float* __restrict__ r = v.r;
  const float* __restrict__ rD = v.rD;
  auto yq = [&](int q) {
    return __ldg(rD + q) * fmaf(beta, fmaf(-omega, __ldg(vo + q), __ldg(po + q)), __ldg(r + q));
  };
  DFAcc a0, a1;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < L.n_cells;
       c += gridDim.x * blockDim.x) {
    const float pc = fmaf(beta, fmaf(-omega, __ldg(vo + c), __ldg(po + c)), __ldg(r + c));
    const float yc = __ldg(rD + c) * pc;
    pn[c] = pc;
    v.y[c] = yc;
    const float yv = hex33_amul_formed(L, coef32, v.d32, c, yc, yq);
    vn[c] = yv;
    a0.add_prod(__ldg(v.rt + c), yv);
  }
  mb_amul_finish<0>(v, a0, a1, sh);
}

// s = r - alpha v, z = s / d_M, x32 += alpha y, t = A32 z, t.t and t.s (or
// t.z) -> omega or the t.t branch.
__global__ void __launch_bounds__(kBlock)
    mb_st_kernel(gbf_layout L, const float* __restrict__ coef32, MbVecs v, int parity,
                 int standard_omega) {
  pdl_wait();
  pdl_launch_dependents();
  if (v.st->status != GBF_RUNNING) return;
  __shared__ double sh[kBlock / 32];
  const float alpha = (float)v.st->alpha;
  const float* __restrict__ vn = parity ? v.v : v.v2;  // this iteration's v
  const float* __restrict__ r = v.r;
  const float* __restrict__ rD = v.rD;
  auto zq = [&](int q) { return __ldg(rD + q) * fmaf(-alpha, __ldg(vn + q), __ldg(r + q)); };
  DFAcc a0, a1;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < L.n_cells;
       c += gridDim.x * blockDim.x) {
    const float sc = fmaf(-alpha, __ldg(vn + c), __ldg(r + c));
    const float zc = __ldg(rD + c) * sc;
    v.s[c] = sc;
    v.z[c] = zc;
    v.xlo[c] = fmaf(alpha, v.y[c], v.xlo[c]);
    const float tv = hex33_amul_formed(L, coef32, v.d32, c, zc, zq);
    v.t[c] = tv;
    a0.add_prod(tv, tv);
    a1.add_prod(tv, standard_omega ? sc : zc);
  }
  mb_amul_finish<1>(v, a0, a1, sh);
}

// Folds the remaining FP32 correction into x at the end of the solve.
__global__ void mb_fold_kernel(int n, double* __restrict__ x, MbVecs v) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const float xl = v.xlo[c];
    if (xl != 0.0f) x[c] += (double)xl;
    v.xlo[c] = 0.0f;
  }
}

// ---------------------------------------------------------------------------
// The whole inner loop in one cooperative launch.  The same iteration,
// breakdown tests and reliable updates as the per-phase kernels above; the phases are separated by the
// bounded grid barrier instead of kernel boundaries, and every block reduces
// the per-block partials itself, in the same fixed order, so that all blocks
// hold the same scalars and take the same decisions without a state round
// trip.  Consecutive reductions alternate between two partial buffers: a
// block may write the next reduction's partials while a slower block still
// reads the previous one.  Each block owns a fixed set of cells in every
// phase; data other blocks rewrite inside the launch (y, z, x, the partials)
// is read from L2.  The dot products reduce over this launch's grid, so the
// results agree with the per-phase form to rounding, not bit for bit.
// ---------------------------------------------------------------------------
// Automatic form choice, from a sweep of the forms on GB300 (convection-
// diffusion systems, 16^3 .. 128^3, us per inner iteration): the single
// launch wins while the per-kernel launch gaps dominate (22.7 against 27.8
// fused and 29.5 gather at 32^3), the fused three-kernel form in the middle
// (34.8 against 38.7 gather at 64^3, level at 96^3), the plain L2 gather
// above (81.0 against 92.1 fused and 84.4 staged at 128^3: there the fused
// form's neighbour values, formed from four vectors, cost more than the
// passes it saves), and the staged stream where blocks have many tiles.
constexpr int kMbAutoPersistentCells = 1 << 16;
constexpr int kMbAutoFusedCells = 1 << 19;
constexpr int kMbAutoGatherCells = 1 << 22;

struct MbRegs {
  double rho, alpha, omega, beta, res0, res, rmax, target;
  int inner, status, n_hist, phase, fold_pending, updates, branch;
};

// Sum of this reduction's per-block partials (index `which` of two),
// identical in every block and broadcast to every thread of it (the block
// reduction leaves its result in thread 0 only); `slot` is a shared double.
__device__ __forceinline__ double mb_grid_sum(const double* part, int which, double* sh,
                                              double* slot) {
  const double t = reduce_partials(part + which * gridDim.x, (int)gridDim.x, sh);
  __syncthreads();  // every thread has read the slot's previous value
  if (threadIdx.x == 0) *slot = t;
  __syncthreads();
  return *slot;
}

template <int KIND>
__global__ void __launch_bounds__(kBlock, 3)
    mb_persistent_kernel(gbf_layout L, const double* __restrict__ coef64,
                         const double* __restrict__ diag64, const float* __restrict__ coef32,
                         const double* __restrict__ b, double* __restrict__ x, MbVecs v,
                         double* hist, int hist_cap, double delta, gbf_solve_params P,
                         int standard_omega, GridBarrier* bar) {
  __shared__ double sh[kBlock / 32];
  __shared__ double bc[2];  // the grid sums, broadcast to the block
  const unsigned G = gridDim.x;
  const int n = L.n_cells;
  const int c0 = blockIdx.x * kBlock + threadIdx.x, cs = G * kBlock;
  const bool lead = blockIdx.x == 0 && threadIdx.x == 0;
  // two partial buffers of 2G doubles each
  double* partbuf[2] = {v.partials, v.partials + 2 * G};
  int red = 0;
  MbRegs q;
  {
    const MbState* st = v.st;  // written by mb_init_kernel, a separate launch
    q.rho = st->rho;
    q.alpha = st->alpha;
    q.omega = st->omega;
    q.beta = st->beta;
    q.res0 = st->res0;
    q.res = st->res;
    q.rmax = st->rmax;
    q.target = st->target;
    q.inner = st->inner;
    q.status = st->status;
    q.n_hist = st->n_hist;
    q.phase = MB_NORMAL;
    q.fold_pending = 0;
    q.updates = 0;
    q.branch = 0;
  }
  const long long limit = (long long)P.max_iter + 2;
  bool ok = true;
  for (long long it = 0; q.status == GBF_RUNNING && it < limit; ++it) {
    // v = A32 y, r~.v -> alpha
    {
      double* part = partbuf[red & 1];
      DFAcc a;
      for (int c = c0; c < n; c += cs) {
        const float yc = __ldcg(v.y + c);
        const float yv = cell_amul_k<KIND, float, float, false, true>(L, coef32, v.d32, v.y, c, yc);
        v.v[c] = yv;
        a.add_prod(__ldg(v.rt + c), yv);
      }
      const double s0 = block_sum_df(a, sh);
      if (threadIdx.x == 0) part[blockIdx.x] = s0;
      if (!(ok = grid_barrier(bar, G))) break;
      const double t0 = mb_grid_sum(part, 0, sh, &bc[0]);
      ++red;
      if (fabs(t0) < 1e-30) {
        q.status = GBF_BREAKDOWN;  // pbicgstab.py:168-171
        break;
      }
      q.alpha = q.rho / t0;
    }
    // s = r - alpha v, z = s / d_M, x32 += alpha y
    {
      const float alpha = (float)q.alpha;
      for (int c = c0; c < n; c += cs) {
        const float s = fmaf(-alpha, __ldcg(v.v + c), __ldcg(v.r + c));
        v.s[c] = s;
        v.z[c] = __ldg(v.rD + c) * s;
        v.xlo[c] = fmaf(alpha, __ldcg(v.y + c), __ldcg(v.xlo + c));
      }
      if (!(ok = grid_barrier(bar, G))) break;
    }
    // t = A32 z, t.t, t.s (or t.z) -> omega or the t.t branch
    {
      double* part = partbuf[red & 1];
      DFAcc a0, a1;
      for (int c = c0; c < n; c += cs) {
        const float zc = __ldcg(v.z + c);
        const float tv = cell_amul_k<KIND, float, float, false, true>(L, coef32, v.d32, v.z, c, zc);
        v.t[c] = tv;
        a0.add_prod(tv, tv);
        a1.add_prod(tv, standard_omega ? __ldcg(v.s + c) : zc);
      }
      const double s0 = block_sum_df(a0, sh);
      const double s1 = block_sum_df(a1, sh);
      if (threadIdx.x == 0) {
        part[blockIdx.x] = s0;
        part[G + blockIdx.x] = s1;
      }
      if (!(ok = grid_barrier(bar, G))) break;
      const double t0 = mb_grid_sum(part, 0, sh, &bc[0]);
      const double t1 = mb_grid_sum(part, 1, sh, &bc[1]);
      ++red;
      if (fabs(t0) < 1e-30) {
        q.branch = 1;  // pbicgstab.py:196-208
      } else {
        q.branch = 0;
        q.omega = t1 / t0;
      }
    }
    // x32 += omega z (folded into x64 when an update is pending),
    // r = s - omega t, r.r, r~.r -> beta, update decision
    {
      double* part = partbuf[red & 1];
      const int branch = q.branch;
      const float omega = (float)q.omega;
      const bool fold = q.fold_pending != 0;
      DFAcc arr, artr;
      for (int c = c0; c < n; c += cs) {
        float xl = __ldcg(v.xlo + c);
        const float s = __ldcg(v.s + c);
        float r = s;
        if (branch == 0) {
          xl = fmaf(omega, __ldcg(v.z + c), xl);
          r = fmaf(-omega, __ldcg(v.t + c), s);
        }
        if (fold) {
          x[c] = __ldcg(x + c) + (double)xl;
          xl = 0.0f;
        }
        v.r[c] = r;
        v.xlo[c] = xl;
        arr.add_prod(r, r);
        artr.add_prod(__ldg(v.rt + c), r);
      }
      const double s0 = block_sum_df(arr, sh);
      const double s1 = block_sum_df(artr, sh);
      if (threadIdx.x == 0) {
        part[blockIdx.x] = s0;
        part[G + blockIdx.x] = s1;
      }
      if (!(ok = grid_barrier(bar, G))) break;
      const double trr = mb_grid_sum(part, 0, sh, &bc[0]);
      const double trtr = mb_grid_sum(part, 1, sh, &bc[1]);
      ++red;
      q.inner += 1;
      q.res = sqrt(trr);
      if (branch == 0 && fabs(q.omega) < 1e-30) {
        q.status = GBF_BREAKDOWN;  // pbicgstab.py:227-229
        break;
      } else if (fold) {
        q.fold_pending = 0;
        q.phase = MB_TRUE_RESIDUAL;
      } else {
        q.beta = branch == 0 ? (trtr / q.rho) * (q.alpha / q.omega) : (trtr / q.rho) * q.alpha;
        q.rho = trtr;
        q.rmax = fmax(q.rmax, q.res);
        if (q.res < delta * q.rmax || q.res < q.target || q.inner >= P.max_iter) {
          q.fold_pending = 1;
        } else if (fabs(trtr) < 1e-30) {
          q.status = GBF_BREAKDOWN;  // the next iteration's rho test
          break;
        }
      }
    }
    // r64 = b - A64 x64, r = (float) r64, |r64|, r~.r -> convergence, beta
    if (q.phase == MB_TRUE_RESIDUAL) {
      double* part = partbuf[red & 1];
      double rr = 0.0;
      DFAcc artr;
      for (int c = c0; c < n; c += cs) {
        const double xc = __ldcg(x + c);
        const double y = cell_amul<double, double, false, true>(L, coef64, diag64, x, c, xc);
        const double rh = __dsub_rn(__ldg(b + c), y);
        const float r = (float)rh;
        v.r[c] = r;
        rr = fma(rh, rh, rr);
        artr.add_prod(__ldg(v.rt + c), r);
      }
      rr = block_sum(rr, sh);
      const double rtr = block_sum_df(artr, sh);
      if (threadIdx.x == 0) {
        part[blockIdx.x] = rr;
        part[G + blockIdx.x] = rtr;
      }
      if (!(ok = grid_barrier(bar, G))) break;
      const double trr = mb_grid_sum(part, 0, sh, &bc[0]);
      const double trtr = mb_grid_sum(part, 1, sh, &bc[1]);
      ++red;
      q.res = sqrt(trr);
      q.updates += 1;
      if (lead && q.n_hist < hist_cap) hist[q.n_hist] = q.res;
      q.n_hist += 1;
      q.phase = MB_NORMAL;
      if (mb_converged(q.res, q.res0, q.inner, P)) {
        q.status = GBF_CONVERGED;
        break;
      } else if (q.inner >= P.max_iter) {
        q.status = GBF_MAX_ITER;
        break;
      }
      q.beta = q.branch == 0 ? (trtr / q.rho) * (q.alpha / q.omega) : (trtr / q.rho) * q.alpha;
      q.rho = trtr;
      q.rmax = q.res;
      if (fabs(trtr) < 1e-30) {
        q.status = GBF_BREAKDOWN;
        break;
      }
    }
    // p = r + beta (p - omega v), y = p / d_M
    {
      const float beta = (float)q.beta;
      const float omega = q.branch == 0 ? (float)q.omega : 1.0f;
      for (int c = c0; c < n; c += cs) {
        const float p = fmaf(beta, fmaf(-omega, __ldcg(v.v + c), __ldcg(v.p + c)),
                             __ldcg(v.r + c));
        v.p[c] = p;
        v.y[c] = __ldg(v.rD + c) * p;
      }
      if (!(ok = grid_barrier(bar, G))) break;
    }
  }
  if (!ok) return;  // the host reads the barrier's fault word
  // fold the remaining FP32 correction of this block's own cells
  for (int c = c0; c < n; c += cs) {
    const float xl = __ldcg(v.xlo + c);
    if (xl != 0.0f) x[c] = __ldcg(x + c) + (double)xl;
    v.xlo[c] = 0.0f;
  }
  if (lead) {
    MbState* st = v.st;
    st->rho = q.rho;
    st->alpha = q.alpha;
    st->omega = q.omega;
    st->beta = q.beta;
    st->res = q.res;
    st->inner = q.inner;
    st->status = q.status;
    st->n_hist = q.n_hist;
    st->updates = q.updates;
  }
}

static size_t mb_a256(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr int kMbVectors = 13;

}  // namespace gbf

using namespace gbf;

extern "C" size_t gbf_mixed_pbicgstab_workspace_bytes(int32_t n) {
  if (n < 0) return 0;
  return kMbVectors * mb_a256(sizeof(float) * (size_t)n) +
         mb_a256(sizeof(double) * 2 * kMaxGrid) + mb_a256(sizeof(MbState)) +
         mb_a256(sizeof(GridBarrier));
}

namespace gbf {
// Resident blocks of the persistent form (occupancy x SMs, at most one per
// 256 cells and kMaxGrid / 2 for the two partial buffers); 0 when the
// device cannot launch it cooperatively.
template <int KIND>
static int mb_persistent_grid(int n) {
  int dev = 0, sms = 0, coop = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mb_persistent_kernel<KIND>, kBlock,
                                                    0) != cudaSuccess ||
      per_sm <= 0)
    return 0;
  long long g = (long long)per_sm * sms;
  const long long need = ((long long)n + kBlock - 1) / kBlock;
  if (g > need) g = need;
  if (g > kMaxGrid / 2) g = kMaxGrid / 2;
  return g < 1 ? 1 : (int)g;
}
}  // namespace gbf

extern "C" int gbf_mixed_pbicgstab_solve(const gbf_layout* L, const double* coef64,
                                         const double* diag64, const float* coef32,
                                         const double* pd, const double* b, double* x,
                                         double delta, double* hist, int32_t hist_cap,
                                         const gbf_solve_params* P, gbf_solve_result* R,
                                         void* ws, size_t ws_bytes, void* stream) {
  ::gbf::NvtxScope nvtx_("gbf_mixed_pbicgstab_solve");
  int rc = check_layout(L);
  if (rc) return rc;
  GBF_REQUIRE(P && R, "mixed_pbicgstab: NULL params/result");
  GBF_REQUIRE(P->max_iter >= 0, "mixed_pbicgstab: negative max_iter");
  GBF_REQUIRE(delta > 0.0 && delta < 1.0, "mixed_pbicgstab: delta must be in (0, 1), got %g",
              delta);
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
              "mixed_pbicgstab: NULL pointer");
  GBF_REQUIRE(ws_bytes >= gbf_mixed_pbicgstab_workspace_bytes(n),
              "mixed_pbicgstab: workspace too small");
  cudaStream_t s = as_stream(stream);
  char* w = static_cast<char*>(ws);
  const size_t vb = mb_a256(sizeof(float) * (size_t)n);
  MbVecs v;
  float** vecs[kMbVectors] = {&v.r, &v.rt, &v.p,  &v.v,   &v.y, &v.s, &v.z,
                              &v.t, &v.xlo, &v.rD, &v.d32, &v.p2, &v.v2};
  for (int i = 0; i < kMbVectors; ++i) *vecs[i] = reinterpret_cast<float*>(w + i * vb);
  v.partials = reinterpret_cast<double*>(w + kMbVectors * vb);
  v.st = reinterpret_cast<MbState*>(w + kMbVectors * vb +
                                    mb_a256(sizeof(double) * 2 * kMaxGrid));
  GridBarrier* bar = reinterpret_cast<GridBarrier*>(
      w + kMbVectors * vb + mb_a256(sizeof(double) * 2 * kMaxGrid) + mb_a256(sizeof(MbState)));
  GBF_REQUIRE(P->variant >= 0 && P->variant <= 9, "mixed_pbicgstab: variant must be 0..9");
  const int standard_omega = P->variant & 1;
  // 0 auto, 1 kernels (staged Amul), 2 kernels + gather, 3 persistent, 4 fused
  const int form = P->variant >> 1;

  const int Gi = wave_grid(mb_init_kernel, kBlock, n);
  const bool hex = layout_kind(*L) == kLayoutHex33;
  // the whole inner loop in one cooperative launch (auto: up to 2^16 cells)
  if (form == 3 || (form == 0 && n <= kMbAutoPersistentCells)) {
    const int Gq = hex ? mb_persistent_grid<kLayoutHex33>(n) : mb_persistent_grid<kLayoutGeneric>(n);
    GBF_REQUIRE(Gq > 0 || form != 3, "mixed_pbicgstab: the device cannot run the persistent form");
    if (Gq > 0) {
      GBF_CHECK_CUDA(cudaMemsetAsync(v.st, 0, sizeof(MbState), s));
      GBF_CHECK_CUDA(cudaMemsetAsync(bar, 0, sizeof(GridBarrier), s));
      mb_init_kernel<<<Gi, kBlock, 0, s>>>(*L, coef64, diag64, pd, b, x, v, hist, *P);
      GBF_CHECK_LAUNCH();
      gbf_layout Lc = *L;
      gbf_solve_params Pc = *P;
      int so = standard_omega, hc = hist_cap;
      double dl = delta;
      void* args[] = {&Lc, (void*)&coef64, (void*)&diag64, (void*)&coef32, (void*)&b, &x, &v,
                      &hist, &hc, &dl, &Pc, &so, &bar};
      GBF_CHECK_CUDA(cudaLaunchCooperativeKernel(
          hex ? (const void*)mb_persistent_kernel<kLayoutHex33>
              : (const void*)mb_persistent_kernel<kLayoutGeneric>,
          dim3(Gq), dim3(kBlock), args, 0, s));
      MbState hs;
      GridBarrier hb;
      GBF_CHECK_CUDA(cudaMemcpyAsync(&hs, v.st, sizeof(hs), cudaMemcpyDeviceToHost, s));
      GBF_CHECK_CUDA(cudaMemcpyAsync(&hb, bar, sizeof(hb), cudaMemcpyDeviceToHost, s));
      GBF_CHECK_CUDA(cudaStreamSynchronize(s));
      R->iterations = hs.inner + 1;
      R->status = hb.fault ? GBF_DEVICE_TIMEOUT
                           : (hs.status == GBF_RUNNING ? GBF_MAX_ITER : hs.status);
      R->final_residual = hs.res;
      R->initial_residual = hs.res0;
      R->inner_iterations = hs.inner;
      R->outer_updates = hs.updates;
      R->launches = 2;
      return GBF_OK;
    }
  }
  // staged Amul: hex layout, 16-byte aligned coefficient / vector streams
  // the fused form needs the hex 3+3 gather; on other layouts it runs as the
  // gather kernels
  const bool fused = hex && (form == 4 || (form == 0 && n <= kMbAutoFusedCells));
  const bool gather = form == 2 || form == 4 || (form == 0 && n <= kMbAutoGatherCells);
  const bool staged = !gather && hex && hex_stream_aligned(coef32, ws, ws, L->slot_dm);
  const int n_tiles = n / kTileCells;
  const long long tile_work = (long long)(n_tiles > 0 ? n_tiles : 1) * kTileCells;
  const int Ga = staged ? wave_grid(mb_amul_stream_kernel<0>, kTileCells, tile_work)
                 : hex  ? wave_grid(mb_amul_kernel<0, kLayoutHex33>, kBlock, n)
                        : wave_grid(mb_amul_kernel<0, kLayoutGeneric>, kBlock, n);
  const int Gb = staged ? wave_grid(mb_amul_stream_kernel<1>, kTileCells, tile_work)
                 : hex  ? wave_grid(mb_amul_kernel<1, kLayoutHex33>, kBlock, n)
                        : wave_grid(mb_amul_kernel<1, kLayoutGeneric>, kBlock, n);
  const int Ba = staged ? kTileCells : kBlock;
  const int Gs = wave_grid(mb_s_kernel, kBlock, (n + 3) / 4);
  const int Gr = wave_grid(mb_r_kernel, kBlock, (n + 3) / 4);
  const int Gt = wave_grid(mb_true_kernel, kBlock, n);
  const int Gp = wave_grid(mb_p_kernel, kBlock, (n + 3) / 4);
  const int Gf = wave_grid(mb_fold_kernel, kBlock, n);
  GBF_CHECK_CUDA(cudaMemsetAsync(v.st, 0, sizeof(MbState), s));
  mb_init_kernel<<<Gi, kBlock, 0, s>>>(*L, coef64, diag64, pd, b, x, v, hist, *P);
  GBF_CHECK_LAUNCH();
  const int chunk = P->check_every > 0 ? P->check_every : 32;
  MbState hs;
  GBF_CHECK_CUDA(cudaMemcpyAsync(&hs, v.st, sizeof(hs), cudaMemcpyDeviceToHost, s));
  GBF_CHECK_CUDA(cudaStreamSynchronize(s));
  // bounded: every launched iteration advances `inner` until max_iter, where
  // a fold + true residual ends the solve (at most max_iter + 2 iterations)
  int launched = 0;
  const int limit = P->max_iter + 2;
  const int Gpv = fused ? wave_grid(mb_pv_kernel, kBlock, n) : 0;
  const int Gst = fused ? wave_grid(mb_st_kernel, kBlock, n) : 0;
  while (hs.status == GBF_RUNNING && launched < limit) {
    for (int j = 0; j < chunk && launched < limit; ++j, ++launched) {
      const gbf_layout Lv = *L;
      const bool tb = (launched % 8 == 0) && timing_begin(kProbeMixedBicgAmul, s);
      cudaError_t e;
      if (fused) {
        const int parity = launched & 1;
        e = launch_pdl(mb_pv_kernel, Gpv, kBlock, s, Lv, coef32, v, parity);
        if (tb) timing_end(kProbeMixedBicgAmul, s);
        if (e == cudaSuccess)
          e = launch_pdl(mb_st_kernel, Gst, kBlock, s, Lv, coef32, v, parity, standard_omega);
        if (e == cudaSuccess) e = launch_pdl(mb_r_kernel, Gr, kBlock, s, n, x, v, delta, *P);
        if (e == cudaSuccess)
          e = launch_pdl(mb_true_kernel, Gt, kBlock, s, Lv, coef64, diag64, b,
                         static_cast<const double*>(x), v, hist, hist_cap, *P);
        GBF_CHECK_CUDA(e);
        continue;
      }
      if (staged)
        e = launch_pdl(mb_amul_stream_kernel<0>, Ga, Ba, s, Lv, coef32, v, n_tiles,
                       standard_omega);
      else if (hex)
        e = launch_pdl(mb_amul_kernel<0, kLayoutHex33>, Ga, Ba, s, Lv, coef32, v, standard_omega);
      else
        e = launch_pdl(mb_amul_kernel<0, kLayoutGeneric>, Ga, Ba, s, Lv, coef32, v,
                       standard_omega);
      if (tb) timing_end(kProbeMixedBicgAmul, s);
      if (e == cudaSuccess) e = launch_pdl(mb_s_kernel, Gs, kBlock, s, n, v);
      if (e == cudaSuccess) {
        if (staged)
          e = launch_pdl(mb_amul_stream_kernel<1>, Gb, Ba, s, Lv, coef32, v, n_tiles,
                         standard_omega);
        else if (hex)
          e = launch_pdl(mb_amul_kernel<1, kLayoutHex33>, Gb, Ba, s, Lv, coef32, v,
                         standard_omega);
        else
          e = launch_pdl(mb_amul_kernel<1, kLayoutGeneric>, Gb, Ba, s, Lv, coef32, v,
                         standard_omega);
      }
      if (e == cudaSuccess) e = launch_pdl(mb_r_kernel, Gr, kBlock, s, n, x, v, delta, *P);
      if (e == cudaSuccess)
        e = launch_pdl(mb_true_kernel, Gt, kBlock, s, Lv, coef64, diag64, b,
                       static_cast<const double*>(x), v, hist, hist_cap, *P);
      if (e == cudaSuccess) e = launch_pdl(mb_p_kernel, Gp, kBlock, s, n, v);
      GBF_CHECK_CUDA(e);
    }
    GBF_CHECK_LAUNCH();
    GBF_CHECK_CUDA(cudaMemcpyAsync(&hs, v.st, sizeof(hs), cudaMemcpyDeviceToHost, s));
    GBF_CHECK_CUDA(cudaStreamSynchronize(s));
  }
  mb_fold_kernel<<<Gf, kBlock, 0, s>>>(n, x, v);
  GBF_CHECK_LAUNCH();
  R->iterations = hs.inner + 1;
  R->status = (hs.status == GBF_RUNNING) ? GBF_MAX_ITER : hs.status;
  R->final_residual = hs.res;
  R->initial_residual = hs.res0;
  R->inner_iterations = hs.inner;
  R->outer_updates = hs.updates;
  R->launches = 2 + (fused ? 4 : 6) * launched;
  return GBF_OK;
}
