// DIC / DILU factorisation (level-scheduled wavefronts) and the diagonal
// preconditioner apply.
#include <math.h>
#include <string.h>

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

// ---- dataflow factorisations ------------------------------------------------
//
// The level-scheduled kernels above separate every level by a grid barrier
// and pay an L2 round trip for the level's loads after it: 4-6 us per level
// on GB300.  The dataflow forms below have no barrier: every value that a
// step reads sits in a slot of device memory that holds the empty marker
// until the step producing it stores it, and a step polls only the slots it
// reads.  The steps are the items of the level schedule in level order,
// dealt round-robin to the resident warps in chunks of 32.  A step reads
// only slots of steps at earlier levels, so the warp holding the earliest
// unfinished step always finds its inputs: with every block resident
// (cooperative launch) the walk cannot stall.  A warp loops over its chunk
// until every lane's step has run; a lane whose inputs are not all there
// yet tries again on the next pass, after a short sleep, so no lane spins
// on its own and lanes of one chunk may feed each other.  The arithmetic
// and the order of the subtractions are those of the level-scheduled
// kernels, so the results are the same bits.
//
// The slots, the empty marker and the bounded pass loop: wavefront.cuh.

// DIC: step = one cell of the level schedule; its slot is d[c] itself
// (every cell's factored value is written once, by its own step, and read
// only by cells after it).  The subtractions of dic_cell, in slot order: a
// pass first issues the loads of every slot still pending (they are
// independent, so their round trips overlap), then applies the slots in
// order up to the first one still empty.  Cells with more than four
// neighbour-side slots (polyhedral meshes) walk them one load at a time.
__global__ void __launch_bounds__(kBlock)
    dic_flow_kernel(gbf_layout L, const double* __restrict__ coef,
                    const double* __restrict__ diag, const int32_t* __restrict__ cells,
                    double* d, GridBarrier* bar, long long max_polls) {
  const int n = L.n_cells;
  const int lane = threadIdx.x & 31;
  const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long chunks = ((long long)n + 31) >> 5;
  long long polls = 0;
  for (long long ch = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; ch < chunks;
       ch += warps) {
    const long long i = ch * 32 + lane;
    bool done = i >= n;
    int c = 0, k = 0, wn = 0, base = 0;
    double dc = 0.0;
    int j[4] = {-1, -1, -1, -1};
    double a[4] = {0.0, 0.0, 0.0, 0.0}, dv[4] = {0.0, 0.0, 0.0, 0.0};
    if (!done) {
      c = __ldg(cells + i);
      dc = __ldg(diag + c);
      if (L.n_faces > 0) {
        const CellSlots cs = cell_slots(L, c);
        wn = cs.wn;
        base = cs.base + 32 * cs.wo;
      }
      if (wn <= 4) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          if (q < wn) {
            j[q] = __ldg(L.slot_col + base + 32 * q);
            a[q] = __ldg(coef + base + 32 * q);
            if (j[q] > c) dv[q] = __ldg(diag + j[q]);  // unfactored: read once
          }
        }
      }
    }
    bool quit = false;
    for (;;) {
      if (!done) {
        if (wn <= 4) {
#pragma unroll
          for (int q = 0; q < 4; ++q)
            if (q >= k && j[q] >= 0 && j[q] < c) dv[q] = ld_flow(d + j[q]);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            if (q == k && q < wn) {
              if (j[q] >= 0 && j[q] < c && flow_empty(dv[q])) continue;  // stays at k
              if (j[q] >= 0 && fabs(dv[q]) > 1e-30)
                dc = __dsub_rn(dc, __ddiv_rn(__dmul_rn(a[q], a[q]), dv[q]));
              k = q + 1;
            }
          }
        } else {
          for (; k < wn; ++k) {
            const int s = base + 32 * k;
            const int jk = __ldg(L.slot_col + s);
            if (jk < 0) continue;
            double dj;
            if (jk < c) {
              dj = ld_flow(d + jk);
              if (flow_empty(dj)) break;  // not factored yet: next pass
            } else {
              dj = __ldg(diag + jk);
            }
            if (fabs(dj) > 1e-30) {
              const double ak = __ldg(coef + s);
              dc = __dsub_rn(dc, __ddiv_rn(__dmul_rn(ak, ak), dj));
            }
          }
        }
        if (k >= wn) {
          st_flow(d + c, dc);
          done = true;
        }
      }
      if (flow_pass_end(done, polls, max_polls, bar, &quit)) break;
      if (quit) return;
    }
  }
}

// DILU: step = one face of the level schedule, item i.  slots[2i] and
// slots[2i+1] receive the owner's and the neighbour's value after the face;
// prev[2i], prev[2i+1] name the slots holding their values before it (the
// slot of the cell's previous face in face order), or -1 for the diagonal.
// The update of dilu_face: both ends from the values before the face.
__global__ void __launch_bounds__(kBlock)
    dilu_flow_kernel(gbf_layout L, const double* __restrict__ lower,
                     const double* __restrict__ upper, const double* __restrict__ diag,
                     const int32_t* __restrict__ faces, const int32_t* __restrict__ prev,
                     double* slots, GridBarrier* bar, long long max_polls) {
  const int nf = L.n_faces;
  const int lane = threadIdx.x & 31;
  const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long chunks = ((long long)nf + 31) >> 5;
  long long polls = 0;
  for (long long ch = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; ch < chunks;
       ch += warps) {
    const long long i = ch * 32 + lane;
    bool done = i >= nf;
    int sp = -1, sq = -1;
    double a = 0.0, b = 0.0, l = 0.0, u = 0.0;
    if (!done) {
      const int f = __ldg(faces + i);
      l = __ldg(lower + f);
      u = __ldg(upper + f);
      sp = __ldg(prev + 2 * i);
      sq = __ldg(prev + 2 * i + 1);
      if (sp < 0) a = __ldg(diag + __ldg(L.owner + f));
      if (sq < 0) b = __ldg(diag + __ldg(L.neighbour + f));
    }
    bool quit = false;
    for (;;) {
      if (!done) {
        // both loads issued before either is looked at: one round trip
        const double va = sp >= 0 ? ld_flow(slots + sp) : 0.0;
        const double vb = sq >= 0 ? ld_flow(slots + sq) : 0.0;
        if (sp >= 0 && !flow_empty(va)) {
          a = va;
          sp = -1;
        }
        if (sq >= 0 && !flow_empty(vb)) {
          b = vb;
          sq = -1;
        }
        if (sp < 0 && sq < 0) {
          double na = a, nb = b;
          if (fabs(b) > 1e-30) na = __dsub_rn(a, __ddiv_rn(__dmul_rn(l, u), b));
          if (fabs(a) > 1e-30) nb = __dsub_rn(b, __ddiv_rn(__dmul_rn(u, l), a));
          st_flow(slots + 2 * i, na);
          st_flow(slots + 2 * i + 1, nb);
          done = true;
        }
      }
      if (flow_pass_end(done, polls, max_polls, bar, &quit)) break;
      if (quit) return;
    }
  }
}

// d = clamp(|d|) after the DIC walk; NaN everywhere if a wait ran out.
__global__ void dic_flow_out_kernel(int n, const GridBarrier* bar, double* d) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  if (bar->fault != 0)
    d[c] = __longlong_as_double(0x7ff8000000000000LL);
  else
    clamp_abs(d, c);
}

// d = clamp(|value after the cell's last face|) (the diagonal for a cell on
// no face); NaN everywhere if a wait ran out.
__global__ void dilu_flow_out_kernel(int n, const double* __restrict__ diag,
                                     const int32_t* __restrict__ cell_last,
                                     const double* __restrict__ slots, const GridBarrier* bar,
                                     double* d) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  if (bar->fault != 0) {
    d[c] = __longlong_as_double(0x7ff8000000000000LL);
    return;
  }
  const int s = __ldg(cell_last + c);
  const double a = fabs(s < 0 ? __ldg(diag + c) : slots[s]);
  d[c] = (a < 1e-30) ? 1e-30 : a;
}

// Resident blocks for a dataflow walk over n_items steps: at most
// per_sm_max per SM (the warps beyond the few levels of look-ahead only
// add polling traffic) and no more than the chunks need; 0 when the device
// cannot launch cooperatively.
inline int flow_grid(const void* kernel, long long n_items, int per_sm_max) {
  return wavefront_grid(kernel, kBlock, n_items, per_sm_max);
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

// Blocks per SM of the dataflow walks.  Measured on GB300 (jittered hex
// meshes): one block of 256 threads per SM is fastest -- with 2, 4 and 8
// the polling of the warps waiting ahead of the front slows the front
// (DILU 128^3 2.6 / 3.2 / 3.8 / 3.9 ms); with fewer SMs the look-ahead
// runs short at 256^3 (DIC 3.0 ms on 152 blocks, 3.4 on 114, 4.4 on 76).
static int flow_blocks_per_sm() { return 1; }

extern "C" int gbf_dic_build_flow_f64(const gbf_layout* L, const double* coef, const double* diag,
                                      const int32_t* level_cells, double* d_out, void* barrier,
                                      void* stream) {
  ::gbf::NvtxScope nvtx_("gbf_dic_build_flow_f64");
  int rc = check_layout(L);
  if (rc) return rc;
  const int n = L->n_cells;
  if (n == 0) return GBF_OK;
  GBF_REQUIRE(diag && d_out && level_cells && barrier, "dic_build_flow: NULL pointer");
  GBF_REQUIRE(L->n_faces == 0 || coef, "dic_build_flow: NULL coefficients");
  cudaStream_t s = as_stream(stream);
  const int grid = flow_grid((const void*)dic_flow_kernel, n, flow_blocks_per_sm());
  GBF_REQUIRE(grid > 0, "dic_build_flow: the device cannot launch cooperative kernels");
  GBF_CHECK_CUDA(cudaMemsetAsync(d_out, 0xff, sizeof(double) * (size_t)n, s));
  gbf_layout Lc = *L;
  GridBarrier* bar = static_cast<GridBarrier*>(barrier);
  long long polls = kFlowPolls;
  void* args[] = {&Lc, (void*)&coef, (void*)&diag, (void*)&level_cells, &d_out, &bar, &polls};
  GBF_CHECK_CUDA(launch_wavefront((const void*)dic_flow_kernel, grid, args, barrier, s));
  dic_flow_out_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, s>>>(n, bar, d_out);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" size_t gbf_dilu_flow_slots_bytes(int32_t n_faces) {
  return n_faces > 0 ? 2 * sizeof(double) * (size_t)n_faces : 0;
}

extern "C" int gbf_dilu_build_flow_f64(const gbf_layout* L, const double* lower,
                                       const double* upper, const double* diag,
                                       const int32_t* level_faces, const int32_t* prev,
                                       const int32_t* cell_last, double* slots, double* d_out,
                                       void* barrier, void* stream) {
  ::gbf::NvtxScope nvtx_("gbf_dilu_build_flow_f64");
  int rc = check_layout(L);
  if (rc) return rc;
  const int n = L->n_cells;
  if (n == 0) return GBF_OK;
  GBF_REQUIRE(diag && d_out && barrier && cell_last, "dilu_build_flow: NULL pointer");
  cudaStream_t s = as_stream(stream);
  GridBarrier* bar = static_cast<GridBarrier*>(barrier);
  if (L->n_faces > 0) {
    GBF_REQUIRE(lower && upper && level_faces && prev && slots && L->owner && L->neighbour,
                "dilu_build_flow: NULL pointer");
    GBF_REQUIRE(L->n_faces < (1 << 30), "dilu_build_flow: %d faces (at most 2^30 - 1)",
                L->n_faces);
    const int grid = flow_grid((const void*)dilu_flow_kernel, L->n_faces, flow_blocks_per_sm());
    GBF_REQUIRE(grid > 0, "dilu_build_flow: the device cannot launch cooperative kernels");
    GBF_CHECK_CUDA(cudaMemsetAsync(slots, 0xff, gbf_dilu_flow_slots_bytes(L->n_faces), s));
    gbf_layout Lc = *L;
    long long polls = kFlowPolls;
    void* args[] = {&Lc,          (void*)&lower, (void*)&upper, (void*)&diag,
                    (void*)&level_faces, (void*)&prev, &slots, &bar, &polls};
    GBF_CHECK_CUDA(launch_wavefront((const void*)dilu_flow_kernel, grid, args, barrier, s));
  } else {
    GBF_CHECK_CUDA(cudaMemsetAsync(barrier, 0, sizeof(GridBarrier), s));
  }
  dilu_flow_out_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, s>>>(n, diag, cell_last, slots,
                                                                    bar, d_out);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

// Self-test of the dataflow walk's bounded wait, without a GPU fault: two
// faces whose links point at each other's slots (a cycle that
// gbf_dilu_flow_links never builds), in one chunk of one warp.  Neither
// step ever finds its input; after 1000 passes (well under a millisecond)
// the warp sets the fault word and returns, and the output kernel writes
// NaN.  result_h[0] = the fault word, result_h[1] = 1 if all three outputs
// are NaN.  Every index stays inside the buffers below.
extern "C" int gbf_selftest_flow_fault(int32_t* result_h) {
  GBF_REQUIRE(result_h, "selftest: NULL pointer");
  int dev = 0, coop = 0;
  GBF_CHECK_CUDA(cudaGetDevice(&dev));
  GBF_CHECK_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  GBF_REQUIRE(coop, "selftest: the device has no cooperative launch");
  struct Buf {
    GridBarrier bar;
    int32_t own[2], nei[2], faces[2], prev[4], last[3], pad;
    double lower[2], upper[2], diag[3], slots[4], out[3];
  };
  Buf h0;
  memset(&h0, 0, sizeof(h0));
  h0.own[0] = 0, h0.own[1] = 1;
  h0.nei[0] = 1, h0.nei[1] = 2;
  h0.faces[0] = 0, h0.faces[1] = 1;
  // item 0 reads its neighbour from slot 2 (item 1's), item 1 its owner
  // from slot 1 (item 0's): each waits for the other
  h0.prev[0] = -1, h0.prev[1] = 2, h0.prev[2] = 1, h0.prev[3] = -1;
  h0.last[0] = 0, h0.last[1] = 2, h0.last[2] = 3;
  for (int i = 0; i < 2; ++i) h0.lower[i] = h0.upper[i] = -1.0;
  for (int i = 0; i < 3; ++i) h0.diag[i] = 4.0;
  memset(h0.slots, 0xff, sizeof(h0.slots));
  Buf* d = nullptr;
  GBF_CHECK_CUDA(cudaMalloc(&d, sizeof(Buf)));
  cudaError_t e = cudaMemcpy(d, &h0, sizeof(Buf), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    gbf_layout L;
    memset(&L, 0, sizeof(L));
    L.n_cells = 3;
    L.n_faces = 2;
    L.owner = d->own;
    L.neighbour = d->nei;
    const double *lo = d->lower, *up = d->upper, *dg = d->diag;
    const int32_t *fc = d->faces, *pv = d->prev;
    double* sl = d->slots;
    GridBarrier* bar = &d->bar;
    long long polls = 1000;
    void* args[] = {&L, (void*)&lo, (void*)&up, (void*)&dg, (void*)&fc, (void*)&pv, &sl, &bar,
                    &polls};
    e = cudaLaunchCooperativeKernel((const void*)dilu_flow_kernel, dim3(1), dim3(32), args, 0,
                                    nullptr);
    if (e == cudaSuccess) {
      dilu_flow_out_kernel<<<1, 32>>>(3, d->diag, d->last, d->slots, &d->bar, d->out);
      e = cudaGetLastError();
    }
  }
  Buf h;
  if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(Buf), cudaMemcpyDeviceToHost);
  cudaFree(d);
  GBF_CHECK_CUDA(e);
  int all_nan = 1;
  for (int i = 0; i < 3; ++i) all_nan &= (h.out[i] != h.out[i]) ? 1 : 0;
  result_h[0] = h.bar.fault;
  result_h[1] = all_nan;
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

namespace gbf {
// The sweep as a dataflow walk: item i (face f of the schedule, in level
// order) writes slot i = W's value after the face; prev[2i] / prev[2i+1]
// name the slots holding W's value before the face and R's value at it (-1:
// the entry value in res, which the walk never writes).  sweep_face's
// arithmetic, so the same bits.
__global__ void __launch_bounds__(kBlock)
    sweep_flow_kernel(const int32_t* __restrict__ own, const int32_t* __restrict__ nei,
                      const double* __restrict__ coef, const double* __restrict__ d,
                      const int32_t* __restrict__ items, const int32_t* __restrict__ prev,
                      int n_items, int reverse, const double* __restrict__ res, double* slots,
                      GridBarrier* bar, long long max_polls) {
  const int lane = threadIdx.x & 31;
  const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long chunks = ((long long)n_items + 31) >> 5;
  long long polls = 0;
  for (long long ch = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; ch < chunks;
       ch += warps) {
    const long long i = ch * 32 + lane;
    bool done = i >= n_items;
    int sw = -1, sr = -1;
    double w = 0.0, r = 0.0, dr = 0.0, cf = 0.0;
    if (!done) {
      const int f = __ldg(items + i);
      const int R = reverse ? __ldg(nei + f) : __ldg(own + f);
      const int W = reverse ? __ldg(own + f) : __ldg(nei + f);
      cf = __ldg(coef + f);
      dr = __ldg(d + R);
      sw = __ldg(prev + 2 * i);
      sr = __ldg(prev + 2 * i + 1);
      if (sw < 0) w = __ldg(res + W);
      if (sr < 0) r = __ldg(res + R);
    }
    bool quit = false;
    for (;;) {
      if (!done) {
        const double vw = sw >= 0 ? ld_flow(slots + sw) : 0.0;
        const double vr = sr >= 0 ? ld_flow(slots + sr) : 0.0;
        if (sw >= 0 && !flow_empty(vw)) {
          w = vw;
          sw = -1;
        }
        if (sr >= 0 && !flow_empty(vr)) {
          r = vr;
          sr = -1;
        }
        if (sw < 0 && sr < 0) {
          st_flow(slots + i,
                  fabs(dr) > 1e-30 ? __dsub_rn(w, __ddiv_rn(__dmul_rn(cf, r), dr)) : w);
          done = true;
        }
      }
      if (flow_pass_end(done, polls, max_polls, bar, &quit)) break;
      if (quit) return;
    }
  }
}

// res[c] = c's last written value (unchanged if none), or NaN everywhere if
// a wait of the walk ran out.
__global__ void sweep_flow_out_kernel(int n, const int32_t* __restrict__ cell_last,
                                      const double* __restrict__ slots, const GridBarrier* bar,
                                      double* res) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  if (bar->fault != 0) {
    res[c] = __longlong_as_double(0x7ff8000000000000LL);
    return;
  }
  const int s = __ldg(cell_last + c);
  if (s >= 0) res[c] = slots[s];
}
}  // namespace gbf

extern "C" int gbf_sweep_flow_f64(const gbf_layout* L, const double* coef, const double* d,
                                  const int32_t* items, int32_t n_items, const int32_t* prev,
                                  const int32_t* cell_last, int32_t reverse, double* res,
                                  double* slots, void* barrier, void* stream) {
  int rc = check_layout(L);
  if (rc) return rc;
  const int n = L->n_cells;
  if (n == 0 || n_items == 0) return GBF_OK;
  GBF_REQUIRE(coef && d && items && prev && cell_last && res && slots && barrier && L->owner &&
                  L->neighbour && n_items > 0 && n_items <= L->n_faces,
              "sweep_flow: NULL pointer or bad item count");
  cudaStream_t s = as_stream(stream);
  const int grid = wavefront_grid((const void*)sweep_flow_kernel, kBlock, n_items, 1);
  GBF_REQUIRE(grid > 0, "sweep_flow: the device cannot launch cooperative kernels");
  GBF_CHECK_CUDA(cudaMemsetAsync(slots, 0xff, sizeof(double) * (size_t)n_items, s));
  const int32_t* own = L->owner;
  const int32_t* nei = L->neighbour;
  int ni = n_items, rev = reverse ? 1 : 0;
  long long polls = kFlowPolls;
  GridBarrier* bar = static_cast<GridBarrier*>(barrier);
  const double* r0 = res;
  void* args[] = {(void*)&own, (void*)&nei, (void*)&coef, (void*)&d, (void*)&items,
                  (void*)&prev, &ni, &rev, (void*)&r0, &slots, &bar, &polls};
  GBF_CHECK_CUDA(launch_wavefront((const void*)sweep_flow_kernel, grid, args, barrier, s));
  sweep_flow_out_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, s>>>(n, cell_last, slots, bar,
                                                                     res);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

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
