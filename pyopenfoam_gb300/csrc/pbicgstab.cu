// FP64 preconditioned BiCGStab, PBiCGSTABSolver._solve
// (solvers/pbicgstab.py:103-239), with two residual checks per iteration
// (on the half-step s and on r) as ResidualMonitor counts them.
//
// Five kernels per iteration; all scalars and the branch taken live in
// device memory, decided by the last block of the reducing kernels:
//   K_v  : v = A y (y = p / d), partial rt.v    -> alpha, breakdown |rt.v|
//   K_s  : s = r - alpha v, z = s / d, x = x + alpha y, partial s.s
//                                               -> |s| check (half step)
//   K_t  : t = A z, partials t.t, t.z          -> omega or the t.t branch
//   K_r  : x = x + omega z, r = s - omega t    (t.t branch: r = s),
//          partials r.r, rt.r                   -> |r| check, beta, rho
//   K_p  : p = r + beta (p - omega v)          (t.t branch: r + beta (p - v)),
//          y = p / d
// x + alpha*y + omega*z is formed as (x + alpha*y) + omega*z, the reference's
// left-to-right evaluation, so storing x + alpha*y in K_s changes nothing.
#include <math.h>
#include <string.h>

#include "amul.cuh"

namespace gbf {

struct BicgState {
  double rho, alpha, omega, beta, res0, res, rtv, tt;
  int iter, status, n_hist, branch;  // branch: 0 regular, 1 t.t breakdown path
  unsigned int ticket[8];
};

struct BicgVecs {
  double *r, *rt, *p, *v, *y, *s, *z, *t, *partials;
  BicgState* st;
};

__device__ __forceinline__ bool bicg_converged(double res, double res0, int iter,
                                               const gbf_solve_params& P) {
  if (iter < P.min_iter) return false;
  if (res < P.tolerance) return true;
  if (res0 > 0.0 && res / res0 < P.rel_tol) return true;
  return false;
}

template <bool PREC>
__global__ void __launch_bounds__(kBlock)
    bicg_init_kernel(gbf_layout L, const double* __restrict__ coef, const double* __restrict__ diag,
                     const double* __restrict__ pd, const double* __restrict__ b,
                     const double* __restrict__ x, BicgVecs v, double* hist, gbf_solve_params P) {
  __shared__ double sh[kBlock / 32];
  const int G = gridDim.x;
  double rr = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < L.n_cells; c += G * blockDim.x) {
    const double y = cell_amul<double, double, false>(L, coef, diag, x, c, __ldg(x + c));
    const double rc = __dsub_rn(__ldg(b + c), y);
    v.r[c] = rc;
    v.rt[c] = rc;
    v.p[c] = rc;
    v.y[c] = PREC ? __ddiv_rn(rc, __ldg(pd + c)) : rc;
    v.v[c] = 0.0;
    rr = fma(rc, rc, rr);
  }
  rr = block_sum(rr, sh);
  if (threadIdx.x == 0) v.partials[blockIdx.x] = rr;
  if (last_block_done(&v.st->ticket[0])) {
    const double trr = reduce_partials(v.partials, G, sh);
    if (threadIdx.x == 0) {
      BicgState* st = v.st;
      const double res = sqrt(trr);
      hist[0] = res;
      st->res0 = res;
      st->res = res;
      st->n_hist = 1;
      st->rho = trr;  // rt = r: rt.r is the same fixed-order sum
      st->iter = 1;
      if (bicg_converged(res, res, 0, P))
        st->status = GBF_CONVERGED;
      else if (P.max_iter < 1)
        st->status = GBF_MAX_ITER;
      else if (fabs(trr) < 1e-30)
        st->status = GBF_BREAKDOWN;  // pbicgstab.py:154-157
      else
        st->status = GBF_RUNNING;
    }
  }
}

template <int KIND>
__global__ void __launch_bounds__(kBlock)
    bicg_v_kernel(gbf_layout L, const double* __restrict__ coef, const double* __restrict__ diag,
                  BicgVecs v) {
  if (v.st->status != GBF_RUNNING) return;
  __shared__ double sh[kBlock / 32];
  const int G = gridDim.x;
  double acc = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < L.n_cells; c += G * blockDim.x) {
    const double yv =
        cell_amul_k<KIND, double, double, false>(L, coef, diag, v.y, c, __ldg(v.y + c));
    v.v[c] = yv;
    acc = fma(__ldg(v.rt + c), yv, acc);
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) v.partials[blockIdx.x] = acc;
  if (last_block_done(&v.st->ticket[1])) {
    const double rtv = reduce_partials(v.partials, G, sh);
    if (threadIdx.x == 0) {
      BicgState* st = v.st;
      st->rtv = rtv;
      if (fabs(rtv) < 1e-30)
        st->status = GBF_BREAKDOWN;  // pbicgstab.py:168-171
      else
        st->alpha = st->rho / rtv;
    }
  }
}

template <bool PREC>
__global__ void __launch_bounds__(kBlock)
    bicg_s_kernel(int n, const double* __restrict__ pd, double* __restrict__ x, BicgVecs v,
                  double* hist, gbf_solve_params P) {
  if (v.st->status != GBF_RUNNING) return;
  __shared__ double sh[kBlock / 32];
  const int G = gridDim.x;
  const double alpha = v.st->alpha;
  double ss = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += G * blockDim.x) {
    const double sc = __dsub_rn(v.r[c], __dmul_rn(alpha, v.v[c]));
    v.s[c] = sc;
    v.z[c] = PREC ? __ddiv_rn(sc, __ldg(pd + c)) : sc;
    x[c] = __dadd_rn(x[c], __dmul_rn(alpha, v.y[c]));
    ss = fma(sc, sc, ss);
  }
  ss = block_sum(ss, sh);
  if (threadIdx.x == 0) v.partials[blockIdx.x] = ss;
  if (last_block_done(&v.st->ticket[2])) {
    const double tss = reduce_partials(v.partials, G, sh);
    if (threadIdx.x == 0) {
      BicgState* st = v.st;
      const double res = sqrt(tss);
      hist[st->n_hist] = res;
      st->n_hist += 1;
      st->res = res;
      // pbicgstab.py:179-183: converged on s, x = x + alpha*y already stored
      if (bicg_converged(res, st->res0, st->iter, P)) st->status = GBF_CONVERGED;
    }
  }
}

template <int KIND>
__global__ void __launch_bounds__(kBlock)
    bicg_t_kernel(gbf_layout L, const double* __restrict__ coef, const double* __restrict__ diag,
                  BicgVecs v, int standard_omega) {
  if (v.st->status != GBF_RUNNING) return;
  __shared__ double sh[kBlock / 32];
  const int G = gridDim.x;
  double tt = 0.0, tz = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < L.n_cells; c += G * blockDim.x) {
    const double zc = __ldg(v.z + c);
    const double tc = cell_amul_k<KIND, double, double, false>(L, coef, diag, v.z, c, zc);
    v.t[c] = tc;
    tt = fma(tc, tc, tt);
    // reference: omega = (t.z)/(t.t); standard BiCGStab: (t.s)/(t.t)
    tz = fma(tc, standard_omega ? v.s[c] : zc, tz);
  }
  tt = block_sum(tt, sh);
  tz = block_sum(tz, sh);
  if (threadIdx.x == 0) {
    v.partials[blockIdx.x] = tt;
    v.partials[G + blockIdx.x] = tz;
  }
  if (last_block_done(&v.st->ticket[3])) {
    const double ttt = reduce_partials(v.partials, G, sh);
    const double ttz = reduce_partials(v.partials + G, G, sh);
    if (threadIdx.x == 0) {
      BicgState* st = v.st;
      st->tt = ttt;
      if (fabs(ttt) < 1e-30) {
        st->branch = 1;  // pbicgstab.py:196-208
      } else {
        st->branch = 0;
        st->omega = ttz / ttt;
      }
    }
  }
}

__global__ void __launch_bounds__(kBlock)
    bicg_r_kernel(int n, double* __restrict__ x, BicgVecs v, double* hist, gbf_solve_params P) {
  if (v.st->status != GBF_RUNNING) return;
  __shared__ double sh[kBlock / 32];
  const int G = gridDim.x;
  const int branch = v.st->branch;
  const double omega = v.st->omega;
  double rr = 0.0, rtr = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += G * blockDim.x) {
    double rc;
    if (branch == 0) {
      x[c] = __dadd_rn(x[c], __dmul_rn(omega, v.z[c]));
      rc = __dsub_rn(v.s[c], __dmul_rn(omega, v.t[c]));
    } else {
      rc = v.s[c];
    }
    v.r[c] = rc;
    rr = fma(rc, rc, rr);
    rtr = fma(__ldg(v.rt + c), rc, rtr);
  }
  rr = block_sum(rr, sh);
  rtr = block_sum(rtr, sh);
  if (threadIdx.x == 0) {
    v.partials[blockIdx.x] = rr;
    v.partials[G + blockIdx.x] = rtr;
  }
  if (last_block_done(&v.st->ticket[4])) {
    const double trr = reduce_partials(v.partials, G, sh);
    const double trtr = reduce_partials(v.partials + G, G, sh);
    if (threadIdx.x == 0) {
      BicgState* st = v.st;
      const double res = sqrt(trr);
      hist[st->n_hist] = res;
      st->n_hist += 1;
      st->res = res;
      if (bicg_converged(res, st->res0, st->iter, P)) {
        st->status = GBF_CONVERGED;
      } else {
        const double rho_new = trtr;
        if (branch == 0) {
          if (fabs(st->omega) < 1e-30) {
            st->status = GBF_BREAKDOWN;  // pbicgstab.py:227-229
          } else {
            st->beta = (rho_new / st->rho) * (st->alpha / st->omega);
          }
        } else {
          st->beta = (rho_new / st->rho) * st->alpha;
        }
        st->rho = rho_new;
        if (st->status == GBF_RUNNING) {
          if (st->iter >= P.max_iter)
            st->status = GBF_MAX_ITER;
          else if (fabs(rho_new) < 1e-30)
            st->status = GBF_BREAKDOWN;  // next iteration's top check
          st->iter += 1;
        }
      }
    }
  }
}

template <bool PREC>
__global__ void __launch_bounds__(kBlock)
    bicg_p_kernel(int n, const double* __restrict__ pd, BicgVecs v) {
  if (v.st->status != GBF_RUNNING) return;
  const double beta = v.st->beta;
  const double omega = v.st->omega;
  const int branch = v.st->branch;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const double q = (branch == 0) ? __dsub_rn(v.p[c], __dmul_rn(omega, v.v[c]))
                                   : __dsub_rn(v.p[c], v.v[c]);
    const double pc = __dadd_rn(v.r[c], __dmul_rn(beta, q));
    v.p[c] = pc;
    v.y[c] = PREC ? __ddiv_rn(pc, __ldg(pd + c)) : pc;
  }
}

static size_t align256b(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace gbf

using namespace gbf;

extern "C" size_t gbf_pbicgstab_workspace_bytes(int32_t n) {
  if (n < 0) return 0;
  return 8 * align256b(sizeof(double) * (size_t)n) + align256b(sizeof(double) * 2 * kMaxGrid) +
         align256b(sizeof(BicgState));
}

extern "C" int gbf_pbicgstab_solve_f64(const gbf_layout* L, const double* coef,
                                       const double* diag, const double* pd, const double* b,
                                       double* x, double* hist, const gbf_solve_params* P,
                                       gbf_solve_result* R, void* ws, size_t ws_bytes,
                                       void* stream) {
  ::gbf::NvtxScope nvtx_("gbf_pbicgstab_solve_f64");
  int rc = check_layout(L);
  if (rc) return rc;
  GBF_REQUIRE(P && R, "pbicgstab: NULL params/result");
  GBF_REQUIRE(P->max_iter >= 0, "pbicgstab: negative max_iter");
  const int n = L->n_cells;
  memset(R, 0, sizeof(*R));
  if (n == 0) {
    const bool conv = (0 >= P->min_iter) && (0.0 < P->tolerance);
    R->iterations = 1;
    R->status = conv ? GBF_CONVERGED : (P->max_iter < 1 ? GBF_MAX_ITER : GBF_BREAKDOWN);
    return GBF_OK;
  }
  GBF_REQUIRE(diag && b && x && hist && ws && (L->n_faces == 0 || coef),
              "pbicgstab: NULL pointer");
  GBF_REQUIRE(ws_bytes >= gbf_pbicgstab_workspace_bytes(n), "pbicgstab: workspace too small");
  cudaStream_t s = as_stream(stream);
  char* w = static_cast<char*>(ws);
  const size_t vb = align256b(sizeof(double) * (size_t)n);
  BicgVecs v;
  double** vecs[8] = {&v.r, &v.rt, &v.p, &v.v, &v.y, &v.s, &v.z, &v.t};
  for (int i = 0; i < 8; ++i) *vecs[i] = reinterpret_cast<double*>(w + i * vb);
  v.partials = reinterpret_cast<double*>(w + 8 * vb);
  v.st = reinterpret_cast<BicgState*>(w + 8 * vb + align256b(sizeof(double) * 2 * kMaxGrid));

  int G = reduction_grid();
  const int need = (n + kBlock - 1) / kBlock;
  if (G > need) G = need;
  GBF_CHECK_CUDA(cudaMemsetAsync(v.st, 0, sizeof(BicgState), s));
  if (pd)
    bicg_init_kernel<true><<<G, kBlock, 0, s>>>(*L, coef, diag, pd, b, x, v, hist, *P);
  else
    bicg_init_kernel<false><<<G, kBlock, 0, s>>>(*L, coef, diag, pd, b, x, v, hist, *P);
  GBF_CHECK_LAUNCH();

  const int chunk = P->check_every > 0 ? P->check_every : 32;
  BicgState hs;
  GBF_CHECK_CUDA(cudaMemcpyAsync(&hs, v.st, sizeof(hs), cudaMemcpyDeviceToHost, s));
  GBF_CHECK_CUDA(cudaStreamSynchronize(s));
  int launched = 0;
  while (hs.status == GBF_RUNNING && launched < P->max_iter) {
    for (int j = 0; j < chunk && launched < P->max_iter; ++j, ++launched) {
      const bool tb = timing_begin(kProbeBicgAmul, s);
      GBF_LAYOUT_DISPATCH(*L, K, bicg_v_kernel<K><<<G, kBlock, 0, s>>>(*L, coef, diag, v));
      if (tb) timing_end(kProbeBicgAmul, s);
      if (pd)
        bicg_s_kernel<true><<<G, kBlock, 0, s>>>(n, pd, x, v, hist, *P);
      else
        bicg_s_kernel<false><<<G, kBlock, 0, s>>>(n, pd, x, v, hist, *P);
      GBF_LAYOUT_DISPATCH(*L, K,
                          bicg_t_kernel<K><<<G, kBlock, 0, s>>>(*L, coef, diag, v,
                                                                P->variant == 1));
      bicg_r_kernel<<<G, kBlock, 0, s>>>(n, x, v, hist, *P);
      if (pd)
        bicg_p_kernel<true><<<G, kBlock, 0, s>>>(n, pd, v);
      else
        bicg_p_kernel<false><<<G, kBlock, 0, s>>>(n, pd, v);
    }
    GBF_CHECK_LAUNCH();
    GBF_CHECK_CUDA(cudaMemcpyAsync(&hs, v.st, sizeof(hs), cudaMemcpyDeviceToHost, s));
    GBF_CHECK_CUDA(cudaStreamSynchronize(s));
  }
  R->iterations = hs.n_hist;
  R->status = (hs.status == GBF_RUNNING) ? GBF_MAX_ITER : hs.status;
  R->final_residual = hs.res;
  R->initial_residual = hs.res0;
  R->launches = 1 + 5 * launched;
  return GBF_OK;
}
