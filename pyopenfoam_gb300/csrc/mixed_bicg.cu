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

// Folds the remaining FP32 correction into x at the end of the solve.
__global__ void mb_fold_kernel(int n, double* __restrict__ x, MbVecs v) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const float xl = v.xlo[c];
    if (xl != 0.0f) x[c] += (double)xl;
    v.xlo[c] = 0.0f;
  }
}

static size_t mb_a256(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr int kMbVectors = 11;

}  // namespace gbf

using namespace gbf;

extern "C" size_t gbf_mixed_pbicgstab_workspace_bytes(int32_t n) {
  if (n < 0) return 0;
  return kMbVectors * mb_a256(sizeof(float) * (size_t)n) +
         mb_a256(sizeof(double) * 2 * kMaxGrid) + mb_a256(sizeof(MbState));
}

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
  float** vecs[kMbVectors] = {&v.r, &v.rt, &v.p, &v.v,   &v.y,  &v.s,
                              &v.z, &v.t,  &v.xlo, &v.rD, &v.d32};
  for (int i = 0; i < kMbVectors; ++i) *vecs[i] = reinterpret_cast<float*>(w + i * vb);
  v.partials = reinterpret_cast<double*>(w + kMbVectors * vb);
  v.st = reinterpret_cast<MbState*>(w + kMbVectors * vb +
                                    mb_a256(sizeof(double) * 2 * kMaxGrid));
  const int standard_omega = P->variant == 1 ? 1 : 0;

  const int Gi = wave_grid(mb_init_kernel, kBlock, n);
  const bool hex = layout_kind(*L) == kLayoutHex33;
  // staged Amul: hex layout, 16-byte aligned coefficient / vector streams
  const bool staged = hex && hex_stream_aligned(coef32, ws, ws, L->slot_dm);
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
  while (hs.status == GBF_RUNNING && launched < limit) {
    for (int j = 0; j < chunk && launched < limit; ++j, ++launched) {
      const gbf_layout Lv = *L;
      const bool tb = (launched % 8 == 0) && timing_begin(kProbeMixedBicgAmul, s);
      cudaError_t e;
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
  R->launches = 2 + 6 * launched;
  return GBF_OK;
}
