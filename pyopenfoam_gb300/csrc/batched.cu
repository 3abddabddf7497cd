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

namespace gbf {

struct BState {
  double rz, alpha, beta, res0, res, rmax, target, pAp;
  int inner, status, phase, fold_pending, updates, x_deferred;
  unsigned int ticket[6];
};

struct BVecs {
  float *r, *z, *p, *Ap, *xlo, *rD, *d32;
  double* partials;   // [2 * n_tiles]
  BState* st;         // [n_systems]
  int* running;       // systems still iterating
};

struct BTiles {
  int n_systems, n_tiles;
  const int32_t* tile_sys;
  const int32_t* tile_begin;
  const int32_t* tile_end;
  const int32_t* sys_tile0;  // [n_systems + 1]
};

using BDFAcc = DFAcc;

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

template <int BS, int KIND>
__global__ void __launch_bounds__(BS)
    bmp_ap_kernel(gbf_layout L, BTiles T, const float* __restrict__ coef32, BVecs v) {
  const int tile = blockIdx.x;
  const int s = __ldg(T.tile_sys + tile);
  BState* st = v.st + s;
  if (st->status != GBF_RUNNING) return;
  __shared__ double sh[BS / 32];
  BDFAcc a;
  for (int c = __ldg(T.tile_begin + tile) + threadIdx.x; c < __ldg(T.tile_end + tile); c += BS) {
    const float pc = __ldg(v.p + c);
    const float y = cell_amul_k<KIND, float, float, false>(L, coef32, v.d32, v.p, c, pc);
    v.Ap[c] = y;
    a.add_prod(pc, y);
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
        st->alpha = st->rz / pAp;
      }
    }
  }
}

// The cell loop of the batched K_upd for one tile.  FOLD is a template
// parameter, not a branch inside the loop: a branch there is predicated, and
// its FP64 conversion and add then issue on every cell of every iteration.
template <int BS, bool FOLD>
__device__ __forceinline__ void bmp_update_cells(const BTiles& T, int tile,
                                                 double* __restrict__ x, const BVecs& v,
                                                 float alpha, BDFAcc& arr, BDFAcc& arz) {
  const unsigned long long ef = l2_evict_first();
  for (int c = __ldg(T.tile_begin + tile) + threadIdx.x; c < __ldg(T.tile_end + tile); c += BS) {
    if constexpr (FOLD) {
      x[c] += (double)fmaf(alpha, v.p[c], v.xlo[c]);
      v.xlo[c] = 0.0f;
    }
    const float r = fmaf(-alpha, ld_nc_hint(v.Ap + c, ef), ld_hint(v.r + c, ef));
    const float z = ld_nc_hint(v.rD + c, ef) * r;
    st_hint(v.r + c, r, ef);
    v.z[c] = z;
    arr.add_prod(r, r);
    arz.add_prod(r, z);
  }
}

template <int BS>
__global__ void __launch_bounds__(BS)
    bmp_update_kernel(BTiles T, double* __restrict__ x, BVecs v, double delta,
                      gbf_solve_params P) {
  const int tile = blockIdx.x;
  const int s = __ldg(T.tile_sys + tile);
  BState* st = v.st + s;
  if (st->status != GBF_RUNNING) return;
  __shared__ double sh[BS / 32];
  const float alpha = (float)st->alpha;
  const bool fold = st->fold_pending != 0;
  BDFAcc arr, arz;
  if (fold)
    bmp_update_cells<BS, true>(T, tile, x, v, alpha, arr, arz);
  else
    bmp_update_cells<BS, false>(T, tile, x, v, alpha, arr, arz);
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
      st->inner += 1;
      const double res = sqrt(trr);
      st->res = res;
      st->x_deferred = fold ? 0 : 1;  // bmp_p_kernel adds alpha p to x32
      if (fold) {
        st->fold_pending = 0;
        st->phase = 1;
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

template <int BS>
__global__ void __launch_bounds__(BS)
    bmp_true_kernel(gbf_layout L, BTiles T, const double* __restrict__ coef64,
                    const double* __restrict__ diag64, const double* __restrict__ b,
                    const double* __restrict__ x, BVecs v, gbf_solve_params P) {
  const int tile = blockIdx.x;
  const int s = __ldg(T.tile_sys + tile);
  BState* st = v.st + s;
  if (st->status != GBF_RUNNING || st->phase != 1) return;
  __shared__ double sh[BS / 32];
  double rr = 0.0, rz = 0.0;
  for (int c = __ldg(T.tile_begin + tile) + threadIdx.x; c < __ldg(T.tile_end + tile); c += BS) {
    const double y = cell_amul<double, double, false>(L, coef64, diag64, x, c, __ldg(x + c));
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
      st->res = res;
      st->updates += 1;
      st->phase = 0;
      if (b_converged(res, st->res0, st->inner, P)) {
        st->status = GBF_CONVERGED;
        atomicSub(v.running, 1);
      } else if (st->inner >= P.max_iter) {
        st->status = GBF_MAX_ITER;
        atomicSub(v.running, 1);
      } else {
        st->beta = trz / st->rz;
        st->rz = trz;
        st->rmax = res;
      }
    }
  }
}

template <int BS>
__global__ void __launch_bounds__(BS) bmp_p_kernel(BTiles T, BVecs v) {
  const int tile = blockIdx.x;
  const BState* st = v.st + __ldg(T.tile_sys + tile);
  if (st->status != GBF_RUNNING) return;
  const float beta = (float)st->beta;
  const float alpha = (float)st->alpha;
  const bool xd = st->x_deferred != 0;
  const unsigned long long ef = l2_evict_first();
  for (int c = __ldg(T.tile_begin + tile) + threadIdx.x; c < __ldg(T.tile_end + tile); c += BS) {
    const float pc = v.p[c];
    if (xd) st_hint(v.xlo + c, fmaf(alpha, pc, ld_hint(v.xlo + c, ef)), ef);
    v.p[c] = fmaf(beta, pc, ld_nc_hint(v.z + c, ef));
  }
}

template <int BS>
__global__ void __launch_bounds__(BS) bmp_fold_kernel(BTiles T, double* __restrict__ x, BVecs v) {
  const int tile = blockIdx.x;
  for (int c = __ldg(T.tile_begin + tile) + threadIdx.x; c < __ldg(T.tile_end + tile); c += BS) {
    const float xl = v.xlo[c];
    if (xl != 0.0f) x[c] += (double)xl;
    v.xlo[c] = 0.0f;
  }
}

static size_t b256(size_t b) { return (b + 255) & ~(size_t)255; }

template <int BS>
static int launch_iteration(cudaStream_t s, int nt, const gbf_layout& L, const BTiles& T,
                            const double* coef64, const double* diag64, const float* coef32,
                            const double* b, double* x, const BVecs& v, double delta,
                            const gbf_solve_params& P) {
  GBF_LAYOUT_DISPATCH(L, K, bmp_ap_kernel<BS, K><<<nt, BS, 0, s>>>(L, T, coef32, v));
  bmp_update_kernel<BS><<<nt, BS, 0, s>>>(T, x, v, delta, P);
  bmp_true_kernel<BS><<<nt, BS, 0, s>>>(L, T, coef64, diag64, b, x, v, P);
  bmp_p_kernel<BS><<<nt, BS, 0, s>>>(T, v);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_ERR_CUDA;
}

template <int BS>
static int batched_solve(const gbf_layout* L, const BTiles& T, const double* coef64,
                         const double* diag64, const float* coef32, const double* pd,
                         const double* b, double* x, double delta, const gbf_solve_params* P,
                         int use_graph, gbf_solve_result* R, const BVecs& v, cudaStream_t s) {
  const int nt = T.n_tiles;
  const int S = T.n_systems;
  GBF_CHECK_CUDA(cudaMemsetAsync(v.st, 0, sizeof(BState) * (size_t)S, s));
  GBF_CHECK_CUDA(cudaMemcpyAsync(v.running, &S, sizeof(int), cudaMemcpyHostToDevice, s));
  bmp_init_kernel<BS><<<nt, BS, 0, s>>>(*L, T, coef64, diag64, pd, b, x, v, *P);
  GBF_CHECK_LAUNCH();
  const int chunk = P->check_every > 0 ? P->check_every : 16;
  const int limit = P->max_iter + 2;
  int launched = 0, running = S, launches = 1;
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
      rc = launch_iteration<BS>(cap, nt, *L, T, coef64, diag64, coef32, b, x, v, delta, *P);
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
        rc = launch_iteration<BS>(s, nt, *L, T, coef64, diag64, coef32, b, x, v, delta, *P);
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
  // per-system results
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

}  // namespace gbf

using namespace gbf;

extern "C" size_t gbf_batched_mixed_pcg_workspace_bytes(int32_t n, int32_t n_systems,
                                                        int32_t n_tiles) {
  if (n < 0 || n_systems < 0 || n_tiles < 0) return 0;
  return 7 * b256(sizeof(float) * (size_t)n) + b256(sizeof(double) * 2 * (size_t)n_tiles) +
         b256(sizeof(BState) * (size_t)n_systems) + 256;
}

extern "C" int gbf_batched_mixed_pcg_solve(const gbf_layout* L, const gbf_batch* B,
                                           const double* coef64, const double* diag64,
                                           const float* coef32, const double* pd,
                                           const double* b, double* x, double delta,
                                           const gbf_solve_params* P, int32_t block_size,
                                           int32_t use_graph, gbf_solve_result* R, void* ws,
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
  v.running = reinterpret_cast<int*>(w + off);
  BTiles T{B->n_systems, B->n_tiles, B->tile_sys, B->tile_begin, B->tile_end, B->sys_tile0};
  cudaStream_t s = as_stream(stream);
  switch (block_size) {
    case 128:
      return batched_solve<128>(L, T, coef64, diag64, coef32, pd, b, x, delta, P, use_graph, R,
                                v, s);
    case 512:
      return batched_solve<512>(L, T, coef64, diag64, coef32, pd, b, x, delta, P, use_graph, R,
                                v, s);
    default:
      return batched_solve<256>(L, T, coef64, diag64, coef32, pd, b, x, delta, P, use_graph, R,
                                v, s);
  }
}
