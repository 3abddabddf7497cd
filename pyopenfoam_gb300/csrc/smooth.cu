// Smoothers and the kernels of the host-driven smoothing solvers:
//   Gauss-Seidel sweeps       solvers/smooth_solver.py:134-187 (SmoothSolver,
//                             smoother "GaussSeidel"), solvers/smoothers.py:
//                             63-149 (GaussSeidelSmoother, forward+backward,
//                             relaxed)
//   residual r = b - A x      every smoother's and solver's residual
//   relaxation x += w s z     JacobiSmoother (smoothers.py:152-200), the
//                             DIC/DILU Richardson smoothers
//                             (smooth_solver.py:189-232, smoothers.py:203-260)
//   |r|_2                     the residual norm of the convergence checks
//
// Gauss-Seidel runs as a level-scheduled wavefront (one launch per level,
// gbf_gs_schedule): a cell's update reads the already-updated values of its
// lower-numbered neighbours (forward) and the old values of the others, as
// the reference's sequential cell loop does; no two neighbours share a level.
// Each row sum follows the reference's loop over faces in ascending face
// order (owner-side and neighbour-side slots merged by face index), one
// rounding per operation, so the sweep is bitwise the reference's.
#include <limits.h>
#include <math.h>

#include "amul.cuh"
#include "wavefront.cuh"

namespace gbf {

// The row sum of cell c's update: dc * xc, then coef * x[col] over the
// cell's slots in ascending face order (owner-side and neighbour-side slots
// merged by face index), one rounding per operation.  fetch(col) gives the
// x value the update reads at col.
template <typename FETCH>
__device__ __forceinline__ double gs_row(const gbf_layout& L, const double* __restrict__ coef,
                                         double dc, double xc, int c, FETCH&& fetch) {
  double row = __dmul_rn(dc, xc);
  bool merged = false;
  if (L.n_faces > 0) {
    const CellSlots cs = cell_slots(L, c);
    if (cs.wo <= 4 && cs.wn <= 4) {
      // Every slot's face, coefficient and x value loaded at once; when the
      // cell's neighbour-side faces all precede its owner-side faces (always
      // on a mesh in upper-triangular face order), ascending face order is
      // the neighbour-side slots followed by the owner-side slots.
      int fk[8];
      double a[8], xv[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const bool use = k < 4 ? k < cs.wo : (k - 4) < cs.wn;
        const int slot_k = k < 4 ? k : cs.wo + (k - 4);
        const int slot = cs.base + 32 * slot_k;
        fk[k] = use ? __ldg(L.slot_face + slot) : -1;
        const int col = use ? slot_column(L, cs.e0 + slot_k, slot, c) : -1;
        a[k] = use ? __ldg(coef + slot) : 0.0;
        xv[k] = (use && col >= 0) ? fetch(col) : 0.0;
      }
      int max_nei = -1, min_own = INT_MAX;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (fk[k] >= 0 && fk[k] < min_own) min_own = fk[k];
        if (fk[4 + k] > max_nei) max_nei = fk[4 + k];
      }
      if (max_nei < min_own) {
#pragma unroll
        for (int k = 4; k < 8; ++k)
          if (fk[k] >= 0) row = __dadd_rn(row, __dmul_rn(a[k], xv[k]));
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (fk[k] >= 0) row = __dadd_rn(row, __dmul_rn(a[k], xv[k]));
        merged = true;
      }
    }
  }
  if (L.n_faces > 0 && !merged) {
    const CellSlots cs = cell_slots(L, c);
    int i = 0, j = 0;
    while (true) {
      int fi = INT_MAX, fj = INT_MAX;
      while (i < cs.wo && (fi = __ldg(L.slot_face + cs.base + 32 * i)) < 0) ++i;
      if (i >= cs.wo) fi = INT_MAX;
      while (j < cs.wn && (fj = __ldg(L.slot_face + cs.base + 32 * (cs.wo + j))) < 0) ++j;
      if (j >= cs.wn) fj = INT_MAX;
      if (fi == INT_MAX && fj == INT_MAX) break;
      const int k = fi < fj ? i : cs.wo + j;
      const int slot = cs.base + 32 * k;
      const int col = slot_column(L, cs.e0 + k, slot, c);
      row = __dadd_rn(row, __dmul_rn(__ldg(coef + slot), fetch(col)));
      if (fi < fj)
        ++i;
      else
        ++j;
    }
  }
  return row;
}

// The updated value of cell c from its row sum (the value itself when the
// diagonal is too small to divide by, as in the reference).
template <bool RELAX>
__device__ __forceinline__ double gs_update(double row, double dc, double xc, double bc,
                                            double omega) {
  const double off = __dsub_rn(row, __dmul_rn(dc, xc));
  if (!(fabs(dc) > 1e-30)) return xc;
  const double nv = __ddiv_rn(__dsub_rn(bc, off), dc);
  return RELAX ? __dadd_rn(xc, __dmul_rn(omega, __dsub_rn(nv, xc))) : nv;
}

template <bool RELAX>
__device__ __forceinline__ void gs_cell(const gbf_layout& L, const double* __restrict__ coef,
                                        const double* __restrict__ diag,
                                        const double* __restrict__ b, int c, double omega,
                                        double* x) {
  const double dc = __ldg(diag + c);
  const double xc = __ldcg(x + c);
  const double row = gs_row(L, coef, dc, xc, c, [&](int col) { return __ldcg(x + col); });
  if (fabs(dc) > 1e-30) x[c] = gs_update<RELAX>(row, dc, xc, __ldg(b + c), omega);
}

template <bool RELAX>
__global__ void __launch_bounds__(kBlock)
    gs_level_kernel(gbf_layout L, const double* __restrict__ coef, const double* __restrict__ diag,
                    const double* __restrict__ b, const int32_t* __restrict__ level_ptr,
                    const int32_t* __restrict__ level_cells, int level, double omega,
                    double* x) {
  const int start = __ldg(level_ptr + level);
  const int count = __ldg(level_ptr + level + 1) - start;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < count) gs_cell<RELAX>(L, coef, diag, b, __ldg(level_cells + start + t), omega, x);
}

// A whole Gauss-Seidel sweep in one cooperative launch (wavefront.cuh).
template <bool RELAX>
__global__ void __launch_bounds__(kBlock)
    gs_coop_kernel(gbf_layout L, const double* __restrict__ coef, const double* __restrict__ diag,
                   const double* __restrict__ b, const int32_t* __restrict__ level_ptr,
                   const int32_t* __restrict__ level_cells, int n_levels, double omega,
                   double* x, GridBarrier* bar) {
  if (!run_levels(bar, level_ptr, n_levels, [&](int i) {
        gs_cell<RELAX>(L, coef, diag, b, __ldg(level_cells + i), omega, x);
      }))
    poison(x, L.n_cells);
}

// A whole Gauss-Seidel sweep as a dataflow walk (wavefront.cuh): the cells
// of the level schedule in level order, dealt 32 at a time round-robin to
// the warps of one block per SM.  The sweep reads the old values from x_old
// (never written during the walk) and writes the new ones into the slots
// x_new (initialised to the empty marker); a cell polls only the new values
// it reads -- its neighbours swept before it (lower-numbered forward,
// higher-numbered backward), which are at earlier levels -- so the warp
// holding the earliest unfinished cell always finds its inputs.  The row sum
// and the update are gs_cell's (gs_row, gs_update): the same bits.
template <bool RELAX>
__global__ void __launch_bounds__(kBlock)
    gs_flow_kernel(gbf_layout L, const double* __restrict__ coef, const double* __restrict__ diag,
                   const double* __restrict__ b, const int32_t* __restrict__ cells, int reverse,
                   double omega, const double* __restrict__ x_old, double* x_new,
                   GridBarrier* bar, long long max_polls) {
  const int n = L.n_cells;
  const int lane = threadIdx.x & 31;
  const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long chunks = ((long long)n + 31) >> 5;
  long long polls = 0;
  for (long long ch = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; ch < chunks;
       ch += warps) {
    const long long i = ch * 32 + lane;
    bool done = i >= n;
    int c = 0;
    double dc = 0.0, xc = 0.0, bc = 0.0;
    if (!done) {
      c = __ldg(cells + i);
      dc = __ldg(diag + c);
      xc = __ldg(x_old + c);
      bc = __ldg(b + c);
    }
    bool quit = false;
    for (;;) {
      if (!done) {
        bool missing = false;
        const double row = gs_row(L, coef, dc, xc, c, [&](int col) {
          if (reverse ? col > c : col < c) {
            const double v = ld_flow(x_new + col);
            missing |= flow_empty(v);
            return v;
          }
          return __ldg(x_old + col);
        });
        if (!missing) {
          st_flow(x_new + c, gs_update<RELAX>(row, dc, xc, bc, omega));
          done = true;
        }
      }
      if (flow_pass_end(done, polls, max_polls, bar, &quit)) break;
      if (quit) return;
    }
  }
}

// x = the new values, or NaN everywhere if a wait of the walk ran out.
__global__ void gs_flow_out_kernel(int n, const GridBarrier* bar, const double* __restrict__ x_new,
                                   double* __restrict__ x) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) x[c] = bar->fault != 0 ? __longlong_as_double(0x7ff8000000000000LL) : x_new[c];
}

// r = b - A x with A x in the reference's order (cell_amul).
template <int KIND>
__global__ void __launch_bounds__(kBlock)
    residual_kernel(gbf_layout L, const double* __restrict__ coef, const double* __restrict__ diag,
                    const double* __restrict__ b, const double* __restrict__ x,
                    double* __restrict__ r) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < L.n_cells; c += gridDim.x * blockDim.x)
    r[c] = __dsub_rn(__ldg(b + c),
                     cell_amul_k<KIND, double, double, false>(L, coef, diag, x, c, __ldg(x + c)));
}

// x += (omega * s_c) * z with s_c = 1 / max(|diag_c|, 1e-30), or
// x += omega * z without a diagonal.
__global__ void __launch_bounds__(kBlock)
    relax_kernel(int n, double omega, const double* __restrict__ diag,
                 const double* __restrict__ z, double* __restrict__ x) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  double s = omega;
  if (diag) {
    const double a = fabs(__ldg(diag + c));
    s = __dmul_rn(omega, __ddiv_rn(1.0, a > 1e-30 ? a : 1e-30));
  }
  x[c] = __dadd_rn(x[c], __dmul_rn(s, __ldg(z + c)));
}

// out = x + a * y (one rounding each); out may alias x or y.
__global__ void __launch_bounds__(kBlock)
    xpay_kernel(int n, const double* x, double a, const double* y, double* out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) out[c] = __dadd_rn(x[c], __dmul_rn(a, y[c]));
}

// DiagonalSolver: x = b / max(|d|, 1e-30), r = b - d * x.
__global__ void __launch_bounds__(kBlock)
    diagonal_solve_kernel(int n, const double* __restrict__ d, const double* __restrict__ b,
                          double* __restrict__ x, double* __restrict__ r) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const double dc = __ldg(d + c), a = fabs(dc), bc = __ldg(b + c);
  const double xc = __ddiv_rn(bc, a > 1e-30 ? a : 1e-30);
  x[c] = xc;
  r[c] = __dsub_rn(bc, __dmul_rn(dc, xc));
}

// FvMatrix.relax: diag /= a; source += ((1 - a) * diag) * field_old, with
// one_minus_a = 1 - a computed by the caller in double.
__global__ void __launch_bounds__(kBlock)
    fv_relax_kernel(int n, double a, double one_minus_a, double* __restrict__ diag,
                    double* __restrict__ source, const double* __restrict__ old) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const double d = __ddiv_rn(diag[c], a);
  diag[c] = d;
  source[c] = __dadd_rn(source[c], __dmul_rn(__dmul_rn(one_minus_a, d), __ldg(old + c)));
}

constexpr int kNormBlocks = 1024;

__global__ void __launch_bounds__(kBlock)
    dot_partials_kernel(int n, const double* __restrict__ a, const double* __restrict__ b,
                        double* __restrict__ partials) {
  __shared__ double sh[kBlock / 32];
  double s = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
    s = __fma_rn(__ldg(a + c), __ldg(b + c), s);
  s = block_sum(s, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kBlock)
    sum_partials_kernel(int g, const double* __restrict__ partials, double* __restrict__ out) {
  __shared__ double sh[kBlock / 32];
  double s = 0.0;
  for (int i = threadIdx.x; i < g; i += blockDim.x) s = __dadd_rn(s, partials[i]);
  s = block_sum(s, sh);
  if (threadIdx.x == 0) *out = s;
}

__global__ void __launch_bounds__(kBlock)
    sumsq_partials_kernel(int n, const double* __restrict__ r, double* __restrict__ partials) {
  __shared__ double sh[kBlock / 32];
  double s = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const double v = __ldg(r + c);
    s = __fma_rn(v, v, s);
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kBlock)
    sqrt_sum_kernel(int g, const double* __restrict__ partials, double* __restrict__ out) {
  __shared__ double sh[kBlock / 32];
  double s = 0.0;
  for (int i = threadIdx.x; i < g; i += blockDim.x) s = __dadd_rn(s, partials[i]);
  s = block_sum(s, sh);
  if (threadIdx.x == 0) *out = sqrt(s);
}

}  // namespace gbf

using namespace gbf;

extern "C" int gbf_gauss_seidel_f64(const gbf_layout* L, const double* coef, const double* diag,
                                    const double* b, const int32_t* level_ptr,
                                    const int32_t* level_cells, const int32_t* level_ptr_h,
                                    int32_t n_levels, double omega, int32_t relax, double* x,
                                    void* barrier, void* stream) {
  ::gbf::NvtxScope nvtx_("gbf_gauss_seidel_f64");
  int rc = check_layout(L);
  if (rc) return rc;
  if (L->n_cells == 0) return GBF_OK;
  GBF_REQUIRE(diag && b && x && level_ptr && level_cells && level_ptr_h && n_levels >= 0 &&
                  (L->n_faces == 0 || coef),
              "gauss_seidel: NULL pointer or bad level count");
  cudaStream_t s = as_stream(stream);
  int max_level = 0;
  for (int l = 0; l < n_levels; ++l) {
    const int cnt = level_ptr_h[l + 1] - level_ptr_h[l];
    if (cnt > max_level) max_level = cnt;
  }
  const void* coop = relax ? (const void*)gs_coop_kernel<true> : (const void*)gs_coop_kernel<false>;
  const int gc = (barrier && n_levels > 0) ? wavefront_grid(coop, kBlock, max_level, 2) : 0;
  if (gc > 0) {
    gbf_layout Lc = *L;
    int nl = n_levels;
    GridBarrier* bar = static_cast<GridBarrier*>(barrier);
    void* args[] = {&Lc, (void*)&coef, (void*)&diag, (void*)&b, (void*)&level_ptr,
                    (void*)&level_cells, &nl, &omega, &x, &bar};
    GBF_CHECK_CUDA(launch_wavefront(coop, gc, args, barrier, s));
    return GBF_OK;
  }
  for (int l = 0; l < n_levels; ++l) {
    const int cnt = level_ptr_h[l + 1] - level_ptr_h[l];
    if (cnt <= 0) continue;
    const int grid = (cnt + kBlock - 1) / kBlock;
    if (relax)
      gs_level_kernel<true><<<grid, kBlock, 0, s>>>(*L, coef, diag, b, level_ptr, level_cells, l,
                                                    omega, x);
    else
      gs_level_kernel<false><<<grid, kBlock, 0, s>>>(*L, coef, diag, b, level_ptr, level_cells,
                                                     l, omega, x);
  }
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_gauss_seidel_flow_f64(const gbf_layout* L, const double* coef,
                                         const double* diag, const double* b,
                                         const int32_t* level_cells, int32_t reverse,
                                         double omega, int32_t relax, double* x, double* scratch,
                                         void* barrier, void* stream) {
  ::gbf::NvtxScope nvtx_("gbf_gauss_seidel_flow_f64");
  int rc = check_layout(L);
  if (rc) return rc;
  const int n = L->n_cells;
  if (n == 0) return GBF_OK;
  GBF_REQUIRE(diag && b && x && level_cells && scratch && barrier && (L->n_faces == 0 || coef),
              "gauss_seidel_flow: NULL pointer");
  GBF_REQUIRE(scratch != x, "gauss_seidel_flow: scratch must not be x");
  cudaStream_t s = as_stream(stream);
  const void* k = relax ? (const void*)gs_flow_kernel<true> : (const void*)gs_flow_kernel<false>;
  // one block per SM (the polling of warps ahead of the front slows it)
  const int grid = wavefront_grid(k, kBlock, n, 1);
  GBF_REQUIRE(grid > 0, "gauss_seidel_flow: the device cannot launch cooperative kernels");
  GBF_CHECK_CUDA(cudaMemsetAsync(scratch, 0xff, sizeof(double) * (size_t)n, s));
  gbf_layout Lc = *L;
  int rev = reverse != 0;
  long long polls = kFlowPolls;
  GridBarrier* bar = static_cast<GridBarrier*>(barrier);
  const double* xo = x;
  void* args[] = {&Lc, (void*)&coef, (void*)&diag, (void*)&b, (void*)&level_cells, &rev,
                  &omega, (void*)&xo, &scratch, &bar, &polls};
  GBF_CHECK_CUDA(launch_wavefront(k, grid, args, barrier, s));
  gs_flow_out_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, s>>>(n, bar, scratch, x);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_residual_f64(const gbf_layout* L, const double* coef, const double* diag,
                                const double* b, const double* x, double* r, void* stream) {
  int rc = check_layout(L);
  if (rc) return rc;
  if (L->n_cells == 0) return GBF_OK;
  GBF_REQUIRE(diag && b && x && r && (L->n_faces == 0 || coef), "residual: NULL pointer");
  cudaStream_t s = as_stream(stream);
  if (layout_kind(*L) == kLayoutHex33) {
    const int grid = wave_grid(residual_kernel<kLayoutHex33>, kBlock, L->n_cells);
    residual_kernel<kLayoutHex33><<<grid, kBlock, 0, s>>>(*L, coef, diag, b, x, r);
  } else {
    const int grid = wave_grid(residual_kernel<kLayoutGeneric>, kBlock, L->n_cells);
    residual_kernel<kLayoutGeneric><<<grid, kBlock, 0, s>>>(*L, coef, diag, b, x, r);
  }
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_relax_f64(int32_t n, double omega, const double* diag, const double* z,
                             double* x, void* stream) {
  GBF_REQUIRE(n >= 0, "relax: negative n");
  if (n == 0) return GBF_OK;
  GBF_REQUIRE(z && x, "relax: NULL pointer");
  relax_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, as_stream(stream)>>>(n, omega, diag, z, x);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" size_t gbf_norm2_workspace_bytes(void) { return sizeof(double) * kNormBlocks; }

extern "C" int gbf_norm2_f64(int32_t n, const double* r, double* out, void* workspace,
                             void* stream) {
  GBF_REQUIRE(n >= 0 && out && workspace && (n == 0 || r), "norm2: bad arguments");
  cudaStream_t s = as_stream(stream);
  int g = (n + kBlock - 1) / kBlock;
  g = g < 1 ? 1 : (g > kNormBlocks ? kNormBlocks : g);
  double* partials = static_cast<double*>(workspace);
  sumsq_partials_kernel<<<g, kBlock, 0, s>>>(n, r, partials);
  sqrt_sum_kernel<<<1, kBlock, 0, s>>>(g, partials, out);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_xpay_f64(int32_t n, const double* x, double a, const double* y, double* out,
                            void* stream) {
  GBF_REQUIRE(n >= 0, "xpay: negative n");
  if (n == 0) return GBF_OK;
  GBF_REQUIRE(x && y && out, "xpay: NULL pointer");
  xpay_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, as_stream(stream)>>>(n, x, a, y, out);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_dot_f64(int32_t n, const double* a, const double* b, double* out,
                           void* workspace, void* stream) {
  GBF_REQUIRE(n >= 0 && out && workspace && (n == 0 || (a && b)), "dot: bad arguments");
  cudaStream_t s = as_stream(stream);
  int g = (n + kBlock - 1) / kBlock;
  g = g < 1 ? 1 : (g > kNormBlocks ? kNormBlocks : g);
  double* partials = static_cast<double*>(workspace);
  dot_partials_kernel<<<g, kBlock, 0, s>>>(n, a, b, partials);
  sum_partials_kernel<<<1, kBlock, 0, s>>>(g, partials, out);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_diagonal_solve_f64(int32_t n, const double* diag, const double* b, double* x,
                                      double* r, void* stream) {
  GBF_REQUIRE(n >= 0, "diagonal_solve: negative n");
  if (n == 0) return GBF_OK;
  GBF_REQUIRE(diag && b && x && r, "diagonal_solve: NULL pointer");
  diagonal_solve_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, as_stream(stream)>>>(n, diag, b,
                                                                                   x, r);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_fv_relax_f64(int32_t n, double a, double one_minus_a, double* diag,
                                double* source, const double* field_old, void* stream) {
  GBF_REQUIRE(n >= 0, "fv_relax: negative n");
  if (n == 0) return GBF_OK;
  GBF_REQUIRE(diag && source && field_old, "fv_relax: NULL pointer");
  fv_relax_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, as_stream(stream)>>>(
      n, a, one_minus_a, diag, source, field_old);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}
