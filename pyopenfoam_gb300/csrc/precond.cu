// DIC / DILU factorisation (level-scheduled wavefronts) and the diagonal
// preconditioner apply.
#include <math.h>

#include "wavefront.cuh"

namespace gbf {

// d = clamp(|d|, min=1e-30), NaN kept (torch.clamp semantics).
__device__ __forceinline__ void clamp_abs(double* d, int c) {
  const double a = fabs(d[c]);
  d[c] = (a < 1e-30) ? 1e-30 : a;
}

// One launch per level.  Cell c of the level subtracts, in the reference's
// face order, (a*a)/d_j for each neighbour-side face (a = upper[f],
// j = owner[f]) whose |d_j| > 1e-30, reading the factored value for j < c
// (an earlier level) and the unfactored diagonal for j > c
// (solvers/preconditioners.py:124-128).
__device__ __forceinline__ void dic_cell(const gbf_layout& L, const double* __restrict__ coef,
                                         const double* __restrict__ diag, int c, double* d) {
  double dc = __ldg(diag + c);
  if (L.n_faces > 0) {
    const CellSlots cs = cell_slots(L, c);
    if (cs.wn <= 4) {
      // the slots' columns, coefficients and d values loaded at once, then
      // the subtractions in slot (= face) order
      int j[4];
      double a[4], dj[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int i = cs.base + 32 * (cs.wo + k);
        j[k] = k < cs.wn ? __ldg(L.slot_col + i) : -1;
        a[k] = j[k] >= 0 ? __ldg(coef + i) : 0.0;
        dj[k] = j[k] < 0 ? 0.0 : (j[k] < c ? __ldcg(d + j[k]) : __ldg(diag + j[k]));
      }
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (j[k] >= 0 && fabs(dj[k]) > 1e-30)
          dc = __dsub_rn(dc, __ddiv_rn(__dmul_rn(a[k], a[k]), dj[k]));
    } else {
      for (int k = 0; k < cs.wn; ++k) {
        const int i = cs.base + 32 * (cs.wo + k);
        const int jk = __ldg(L.slot_col + i);
        if (jk < 0) continue;
        const double ak = __ldg(coef + i);
        const double djk = (jk < c) ? __ldcg(d + jk) : __ldg(diag + jk);
        if (fabs(djk) > 1e-30) dc = __dsub_rn(dc, __ddiv_rn(__dmul_rn(ak, ak), djk));
      }
    }
  }
  d[c] = dc;
}

__global__ void __launch_bounds__(kBlock)
    dic_level_kernel(gbf_layout L, const double* __restrict__ coef,
                     const double* __restrict__ diag, const int32_t* __restrict__ level_ptr,
                     const int32_t* __restrict__ level_cells, int level, double* d) {
  const int start = __ldg(level_ptr + level);
  const int count = __ldg(level_ptr + level + 1) - start;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < count) dic_cell(L, coef, diag, __ldg(level_cells + start + t), d);
}

// The whole DIC factorisation in one cooperative launch: the cell levels
// separated by the grid barrier, then the clamp.
__global__ void __launch_bounds__(kBlock)
    dic_coop_kernel(gbf_layout L, const double* __restrict__ coef,
                    const double* __restrict__ diag, const int32_t* __restrict__ level_ptr,
                    const int32_t* __restrict__ level_cells, int n_levels, double* d,
                    GridBarrier* bar) {
  const int stride = gridDim.x * blockDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const bool ok =
      run_levels(bar, level_ptr, n_levels,
                 [&](int i) { dic_cell(L, coef, diag, __ldg(level_cells + i), d); }) &&
      grid_barrier(bar, gridDim.x);
  if (!ok) {
    poison(d, L.n_cells);
    return;
  }
  for (int c = tid; c < L.n_cells; c += stride) clamp_abs(d, c);
}

// One launch per face level.  Each cell is touched by at most one face of a
// level, so the two-ended update of preconditioners.py:254-268 (both ends
// read before either is written) runs without conflicts.
__device__ __forceinline__ void dilu_face(const gbf_layout& L, const double* __restrict__ lower,
                                          const double* __restrict__ upper, int f, double* d) {
  const int p = __ldg(L.owner + f), q = __ldg(L.neighbour + f);
  const double l = __ldg(lower + f), u = __ldg(upper + f);
  const double dp = __ldcg(d + p), dn = __ldcg(d + q);
  if (fabs(dn) > 1e-30) d[p] = __dsub_rn(dp, __ddiv_rn(__dmul_rn(l, u), dn));
  if (fabs(dp) > 1e-30) d[q] = __dsub_rn(dn, __ddiv_rn(__dmul_rn(u, l), dp));
}

__global__ void __launch_bounds__(kBlock)
    dilu_level_kernel(gbf_layout L, const double* __restrict__ lower,
                      const double* __restrict__ upper, const int32_t* __restrict__ level_ptr,
                      const int32_t* __restrict__ level_faces, int level, double* d) {
  const int start = __ldg(level_ptr + level);
  const int count = __ldg(level_ptr + level + 1) - start;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < count) dilu_face(L, lower, upper, __ldg(level_faces + start + t), d);
}

__global__ void clamp_abs_kernel(int n, double* d) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) clamp_abs(d, c);
}

// The whole DILU factorisation in one cooperative launch: d = diag, the face
// levels, the clamp.
__global__ void __launch_bounds__(kBlock)
    dilu_coop_kernel(gbf_layout L, const double* __restrict__ lower,
                     const double* __restrict__ upper, const double* __restrict__ diag,
                     const int32_t* __restrict__ level_ptr,
                     const int32_t* __restrict__ level_faces, int n_levels, double* d,
                     GridBarrier* bar) {
  const int stride = gridDim.x * blockDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  for (int c = tid; c < L.n_cells; c += stride) d[c] = __ldg(diag + c);
  bool ok = grid_barrier(bar, gridDim.x);
  if (ok && L.n_faces > 0)
    ok = run_levels(bar, level_ptr, n_levels,
                    [&](int i) { dilu_face(L, lower, upper, __ldg(level_faces + i), d); }) &&
         grid_barrier(bar, gridDim.x);
  if (!ok) {
    poison(d, L.n_cells);
    return;
  }
  for (int c = tid; c < L.n_cells; c += stride) clamp_abs(d, c);
}

__global__ void copy_kernel(int n, const double* __restrict__ s, double* __restrict__ d) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) d[c] = s[c];
}

__global__ void diag_apply_kernel(int n, const double* __restrict__ r,
                                  const double* __restrict__ d, double* __restrict__ z) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) z[c] = __ddiv_rn(r[c], d[c]);
}

}  // namespace gbf

using namespace gbf;

extern "C" size_t gbf_wavefront_barrier_bytes(void) { return 64; }

extern "C" int gbf_wavefront_fault(const void* barrier, int32_t* fault, void* stream) {
  GBF_REQUIRE(barrier && fault, "wavefront_fault: NULL pointer");
  cudaStream_t s = as_stream(stream);
  GBF_CHECK_CUDA(cudaMemcpyAsync(fault, &static_cast<const GridBarrier*>(barrier)->fault,
                                 sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  GBF_CHECK_CUDA(cudaStreamSynchronize(s));
  return GBF_OK;
}

extern "C" int gbf_dic_build_f64(const gbf_layout* L, const double* coef, const double* diag,
                                 const int32_t* level_ptr, const int32_t* level_cells,
                                 int32_t n_levels, int32_t max_level_size, double* d_out,
                                 void* barrier, void* stream) {
  ::gbf::NvtxScope nvtx_("gbf_dic_build_f64");
  int rc = check_layout(L);
  if (rc) return rc;
  const int n = L->n_cells;
  if (n == 0) return GBF_OK;
  GBF_REQUIRE(diag && d_out && level_ptr && level_cells, "dic_build: NULL pointer");
  GBF_REQUIRE(L->n_faces == 0 || coef, "dic_build: NULL coefficients");
  GBF_REQUIRE(n_levels >= 1 && max_level_size >= 1 && max_level_size <= n,
              "dic_build: bad schedule (levels=%d, max size=%d)", n_levels, max_level_size);
  cudaStream_t s = as_stream(stream);
  // One cooperative launch when a barrier is given (measured on GB300: 2.2
  // ms against 3.06 ms of per-level launches at 128^3, 382 levels; 6.73
  // against 6.67 ms at 256^3, 766 levels); else one launch per cell level.
  const int gc =
      barrier ? wavefront_grid((const void*)dic_coop_kernel, kBlock, max_level_size, 2) : 0;
  if (gc > 0) {
    gbf_layout Lc = *L;
    int nl = n_levels;
    GridBarrier* bar = static_cast<GridBarrier*>(barrier);
    void* args[] = {&Lc, (void*)&coef, (void*)&diag, (void*)&level_ptr, (void*)&level_cells,
                    &nl, &d_out, &bar};
    GBF_CHECK_CUDA(launch_wavefront((const void*)dic_coop_kernel, gc, args, barrier, s));
    return GBF_OK;
  }
  const int grid = (max_level_size + kBlock - 1) / kBlock;
  for (int lv = 0; lv < n_levels; ++lv) {
    dic_level_kernel<<<grid, kBlock, 0, s>>>(*L, coef, diag, level_ptr, level_cells, lv, d_out);
  }
  GBF_CHECK_LAUNCH();
  clamp_abs_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, s>>>(n, d_out);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_dilu_build_f64(const gbf_layout* L, const double* lower, const double* upper,
                                  const double* diag, const int32_t* level_ptr,
                                  const int32_t* level_faces, int32_t n_levels,
                                  int32_t max_level_size, double* d_out, void* barrier,
                                  void* stream) {
  ::gbf::NvtxScope nvtx_("gbf_dilu_build_f64");
  int rc = check_layout(L);
  if (rc) return rc;
  const int n = L->n_cells;
  if (n == 0) return GBF_OK;
  GBF_REQUIRE(diag && d_out, "dilu_build: NULL pointer");
  if (L->n_faces > 0) {
    GBF_REQUIRE(lower && upper && level_ptr && level_faces && L->owner && L->neighbour,
                "dilu_build: NULL pointer");
    GBF_REQUIRE(n_levels >= 1 && max_level_size >= 1 && max_level_size <= L->n_faces,
                "dilu_build: bad schedule (levels=%d, max size=%d)", n_levels, max_level_size);
  }
  cudaStream_t s = as_stream(stream);
  const int gc = barrier ? wavefront_grid((const void*)dilu_coop_kernel, kBlock,
                                          max_level_size > n ? max_level_size : n, 1)
                         : 0;
  if (gc > 0) {
    gbf_layout Lc = *L;
    int nl = n_levels;
    GridBarrier* bar = static_cast<GridBarrier*>(barrier);
    void* args[] = {&Lc, (void*)&lower, (void*)&upper, (void*)&diag, (void*)&level_ptr,
                    (void*)&level_faces, &nl, &d_out, &bar};
    GBF_CHECK_CUDA(launch_wavefront((const void*)dilu_coop_kernel, gc, args, barrier, s));
    return GBF_OK;
  }
  copy_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, s>>>(n, diag, d_out);
  GBF_CHECK_LAUNCH();
  if (L->n_faces > 0) {
    const int grid = (max_level_size + kBlock - 1) / kBlock;
    for (int lv = 0; lv < n_levels; ++lv)
      dilu_level_kernel<<<grid, kBlock, 0, s>>>(*L, lower, upper, level_ptr, level_faces, lv,
                                                d_out);
    GBF_CHECK_LAUNCH();
  }
  clamp_abs_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, s>>>(n, d_out);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_diag_apply_f64(int32_t n, const double* r, const double* d, double* z,
                                  void* stream) {
  GBF_REQUIRE(n >= 0, "diag_apply: negative size");
  if (n == 0) return GBF_OK;
  GBF_REQUIRE(r && d && z, "diag_apply: NULL pointer");
  diag_apply_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, as_stream(stream)>>>(n, r, d, z);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

// ---------------------------------------------------------------------------
// Triangular sweeps of the full DIC / DILU solves, one launch per level of
// gbf_sweep_schedule: res[W] = res[W] - (coef[f] * res[R]) / d[R] when
// |d[R]| > 1e-30, rounded as the reference's
// `result[n] - upper[f] * result[p] / d_p` (preconditioners.py:176-182).
// ---------------------------------------------------------------------------
namespace gbf {
__device__ __forceinline__ void sweep_face(const int32_t* __restrict__ own,
                                           const int32_t* __restrict__ nei,
                                           const double* __restrict__ coef,
                                           const double* __restrict__ d, int f, int reverse,
                                           double* res) {
  const int R = reverse ? __ldg(nei + f) : __ldg(own + f);
  const int W = reverse ? __ldg(own + f) : __ldg(nei + f);
  const double dr = __ldg(d + R);
  if (fabs(dr) > 1e-30) {
    const double u = __ddiv_rn(__dmul_rn(__ldg(coef + f), __ldcg(res + R)), dr);
    res[W] = __dsub_rn(__ldcg(res + W), u);
  }
}

__global__ void __launch_bounds__(kBlock)
    sweep_level_kernel(const int32_t* __restrict__ own, const int32_t* __restrict__ nei,
                       const double* __restrict__ coef, const double* __restrict__ d,
                       const int32_t* __restrict__ level_ptr,
                       const int32_t* __restrict__ level_faces, int level, int reverse,
                       double* res) {
  const int start = __ldg(level_ptr + level);
  const int count = __ldg(level_ptr + level + 1) - start;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < count) sweep_face(own, nei, coef, d, __ldg(level_faces + start + t), reverse, res);
}

// A whole sweep in one cooperative launch.
__global__ void __launch_bounds__(kBlock)
    sweep_coop_kernel(const int32_t* __restrict__ own, const int32_t* __restrict__ nei,
                      const double* __restrict__ coef, const double* __restrict__ d,
                      const int32_t* __restrict__ level_ptr,
                      const int32_t* __restrict__ level_faces, int n_levels, int reverse,
                      double* res, int n_cells, GridBarrier* bar) {
  if (!run_levels(bar, level_ptr, n_levels, [&](int i) {
        sweep_face(own, nei, coef, d, __ldg(level_faces + i), reverse, res);
      }))
    poison(res, n_cells);
}
}  // namespace gbf

extern "C" int gbf_sweep_f64(const gbf_layout* L, const double* coef, const double* d,
                             const int32_t* level_ptr, const int32_t* level_faces,
                             int32_t n_levels, int32_t max_level_size, int32_t reverse,
                             double* res, void* barrier, void* stream) {
  int rc = check_layout(L);
  if (rc) return rc;
  if (L->n_faces == 0 || n_levels == 0) return GBF_OK;
  GBF_REQUIRE(coef && d && level_ptr && level_faces && res && L->owner && L->neighbour,
              "sweep: NULL pointer");
  GBF_REQUIRE(n_levels > 0 && max_level_size > 0 && max_level_size <= L->n_faces,
              "sweep: bad schedule (levels=%d, max size=%d)", n_levels, max_level_size);
  cudaStream_t s = as_stream(stream);
  const int gc = barrier ? wavefront_grid((const void*)sweep_coop_kernel, kBlock, max_level_size, 1)
                         : 0;
  if (gc > 0) {
    const int32_t* own = L->owner;
    const int32_t* nei = L->neighbour;
    int nl = n_levels, rev = reverse ? 1 : 0, n = L->n_cells;
    GridBarrier* bar = static_cast<GridBarrier*>(barrier);
    void* args[] = {(void*)&own, (void*)&nei, (void*)&coef, (void*)&d, (void*)&level_ptr,
                    (void*)&level_faces, &nl, &rev, &res, &n, &bar};
    GBF_CHECK_CUDA(launch_wavefront((const void*)sweep_coop_kernel, gc, args, barrier, s));
    return GBF_OK;
  }
  const int grid = (max_level_size + kBlock - 1) / kBlock;
  for (int lv = 0; lv < n_levels; ++lv)
    sweep_level_kernel<<<grid, kBlock, 0, s>>>(L->owner, L->neighbour, coef, d, level_ptr,
                                               level_faces, lv, reverse ? 1 : 0, res);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}
