// FP64 preconditioned conjugate gradient, PCGSolver._solve
// (solvers/pcg.py:97-187) with ResidualMonitor's convergence rules
// (solvers/residual.py:112-145).
//
// One iteration = three kernels; the scalars (alpha, beta, r.z, status,
// iteration, residual history) live in device memory and are produced by the
// last block of the reducing kernels, so the host never waits inside an
// iteration.  It reads the 64-byte status block every `check_every`
// iterations; kernels launched after convergence return immediately.
//
//   K_ap     : Ap = A p (bitwise reference Amul), partial p.Ap
//              last block: breakdown test |pAp| < 1e-30, alpha = rz / pAp
//   K_update : x = x + alpha p, r = r - alpha Ap, z = r / d,
//              partials r.r and r.z
//              last block: |r|, history, convergence, beta = rz'/rz
//   K_p      : p = z + beta p
//
// Element-wise arithmetic rounds exactly as the reference's torch ops
// (alpha*p rounded, then added; r / d by IEEE division); dot products are
// deterministic fixed-order trees with fused multiply-add accumulation.
#include <math.h>
#include <string.h>

#include "amul.cuh"

namespace gbf {

struct PcgState {
  double rz, alpha, beta, res0, res, pAp;
  int iter, status, n_hist, pad;
  unsigned int ticket[4];
};

struct PcgVecs {
  double *r, *z, *p, *Ap, *partials;
  PcgState* st;
};

__device__ __forceinline__ bool monitor_converged(double res, double res0, int iter,
                                                  const gbf_solve_params& P) {
  if (iter < P.min_iter) return false;
  if (res < P.tolerance) return true;
  if (res0 > 0.0 && res / res0 < P.rel_tol) return true;
  return false;
}

template <bool PREC>
__global__ void __launch_bounds__(kBlock)
    pcg_init_kernel(gbf_layout L, const double* __restrict__ coef, const double* __restrict__ diag,
                    const double* __restrict__ pd, const double* __restrict__ b,
                    const double* __restrict__ x, PcgVecs v, double* hist, gbf_solve_params P) {
  __shared__ double sh[kBlock / 32];
  const int G = gridDim.x;
  double rr = 0.0, rz = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < L.n_cells; c += G * blockDim.x) {
    const double y = cell_amul<double, double, false>(L, coef, diag, x, c, __ldg(x + c));
    const double rc = __dsub_rn(__ldg(b + c), y);
    const double zc = PREC ? __ddiv_rn(rc, __ldg(pd + c)) : rc;
    v.r[c] = rc;
    v.z[c] = zc;
    v.p[c] = zc;
    rr = fma(rc, rc, rr);
    rz = fma(rc, zc, rz);
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
      PcgState* st = v.st;
      const double res = sqrt(trr);
      hist[0] = res;
      st->res0 = res;
      st->res = res;
      st->n_hist = 1;
      st->rz = trz;
      st->iter = 1;
      if (monitor_converged(res, res, 0, P))
        st->status = GBF_CONVERGED;
      else
        st->status = (P.max_iter < 1) ? GBF_MAX_ITER : GBF_RUNNING;
    }
  }
}

template <int KIND>
__global__ void __launch_bounds__(kBlock)
    pcg_ap_kernel(gbf_layout L, const double* __restrict__ coef, const double* __restrict__ diag,
                  PcgVecs v) {
  if (v.st->status != GBF_RUNNING) return;
  __shared__ double sh[kBlock / 32];
  const int G = gridDim.x;
  const double* p = v.p;
  double acc = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < L.n_cells; c += G * blockDim.x) {
    const double pc = __ldg(p + c);
    const double y = cell_amul_k<KIND, double, double, false>(L, coef, diag, p, c, pc);
    v.Ap[c] = y;
    acc = fma(pc, y, acc);
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) v.partials[blockIdx.x] = acc;
  if (last_block_done(&v.st->ticket[1])) {
    const double pAp = reduce_partials(v.partials, G, sh);
    if (threadIdx.x == 0) {
      PcgState* st = v.st;
      st->pAp = pAp;
      if (fabs(pAp) < 1e-30)
        st->status = GBF_BREAKDOWN;  // pcg.py:153-156: x returned as is
      else
        st->alpha = st->rz / pAp;
    }
  }
}

template <bool PREC>
__global__ void __launch_bounds__(kBlock)
    pcg_update_kernel(int n, const double* __restrict__ pd, double* __restrict__ x, PcgVecs v,
                      double* hist, gbf_solve_params P) {
  if (v.st->status != GBF_RUNNING) return;
  __shared__ double sh[kBlock / 32];
  const int G = gridDim.x;
  const double alpha = v.st->alpha;
  double rr = 0.0, rz = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += G * blockDim.x) {
    const double xc = __dadd_rn(x[c], __dmul_rn(alpha, v.p[c]));
    const double rc = __dsub_rn(v.r[c], __dmul_rn(alpha, v.Ap[c]));
    const double zc = PREC ? __ddiv_rn(rc, __ldg(pd + c)) : rc;
    x[c] = xc;
    v.r[c] = rc;
    v.z[c] = zc;
    rr = fma(rc, rc, rr);
    rz = fma(rc, zc, rz);
  }
  rr = block_sum(rr, sh);
  rz = block_sum(rz, sh);
  if (threadIdx.x == 0) {
    v.partials[blockIdx.x] = rr;
    v.partials[G + blockIdx.x] = rz;
  }
  if (last_block_done(&v.st->ticket[2])) {
    const double trr = reduce_partials(v.partials, G, sh);
    const double trz = reduce_partials(v.partials + G, G, sh);
    if (threadIdx.x == 0) {
      PcgState* st = v.st;
      const int it = st->iter;
      const double res = sqrt(trr);
      hist[it] = res;
      st->res = res;
      st->n_hist = it + 1;
      if (monitor_converged(res, st->res0, it, P)) {
        st->status = GBF_CONVERGED;
      } else {
        st->beta = trz / st->rz;
        st->rz = trz;
        st->iter = it + 1;
        if (it >= P.max_iter) st->status = GBF_MAX_ITER;
      }
    }
  }
}

__global__ void __launch_bounds__(kBlock) pcg_p_kernel(int n, PcgVecs v) {
  if (v.st->status != GBF_RUNNING) return;
  const double beta = v.st->beta;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
    v.p[c] = __dadd_rn(v.z[c], __dmul_rn(beta, v.p[c]));
}

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace gbf

using namespace gbf;

extern "C" size_t gbf_pcg_workspace_bytes(int32_t n) {
  if (n < 0) return 0;
  return 4 * align256(sizeof(double) * (size_t)n) + align256(sizeof(double) * 2 * kMaxGrid) +
         align256(sizeof(PcgState));
}

extern "C" int gbf_pcg_solve_f64(const gbf_layout* L, const double* coef, const double* diag,
                                 const double* pd, const double* b, double* x, double* hist,
                                 const gbf_solve_params* P, gbf_solve_result* R, void* ws,
                                 size_t ws_bytes, void* stream) {
  int rc = check_layout(L);
  if (rc) return rc;
  GBF_REQUIRE(P && R, "pcg: NULL params/result");
  GBF_REQUIRE(P->max_iter >= 0, "pcg: negative max_iter");
  const int n = L->n_cells;
  memset(R, 0, sizeof(*R));
  if (n == 0) {
    // empty system: |r| = 0; converged iff 0 < tolerance (residual.py:137-140),
    // otherwise the first p.Ap = 0 is a breakdown (pcg.py:153)
    const bool conv = (0 >= P->min_iter) && (0.0 < P->tolerance);
    R->iterations = 1;
    R->status = conv ? GBF_CONVERGED : (P->max_iter < 1 ? GBF_MAX_ITER : GBF_BREAKDOWN);
    return GBF_OK;
  }
  GBF_REQUIRE(diag && b && x && hist && ws && (L->n_faces == 0 || coef), "pcg: NULL pointer");
  GBF_REQUIRE(ws_bytes >= gbf_pcg_workspace_bytes(n), "pcg: workspace too small");
  cudaStream_t s = as_stream(stream);

  char* w = static_cast<char*>(ws);
  const size_t vb = align256(sizeof(double) * (size_t)n);
  PcgVecs v;
  v.r = reinterpret_cast<double*>(w);
  v.z = reinterpret_cast<double*>(w + vb);
  v.p = reinterpret_cast<double*>(w + 2 * vb);
  v.Ap = reinterpret_cast<double*>(w + 3 * vb);
  v.partials = reinterpret_cast<double*>(w + 4 * vb);
  v.st = reinterpret_cast<PcgState*>(w + 4 * vb + align256(sizeof(double) * 2 * kMaxGrid));

  int G = reduction_grid();
  const int need = (n + kBlock - 1) / kBlock;
  if (G > need) G = need;
  GBF_CHECK_CUDA(cudaMemsetAsync(v.st, 0, sizeof(PcgState), s));
  if (pd)
    pcg_init_kernel<true><<<G, kBlock, 0, s>>>(*L, coef, diag, pd, b, x, v, hist, *P);
  else
    pcg_init_kernel<false><<<G, kBlock, 0, s>>>(*L, coef, diag, pd, b, x, v, hist, *P);
  GBF_CHECK_LAUNCH();

  const int chunk = P->check_every > 0 ? P->check_every : 32;
  PcgState hs;
  GBF_CHECK_CUDA(cudaMemcpyAsync(&hs, v.st, sizeof(hs), cudaMemcpyDeviceToHost, s));
  GBF_CHECK_CUDA(cudaStreamSynchronize(s));
  int launched = 0;
  while (hs.status == GBF_RUNNING && launched < P->max_iter) {
    for (int j = 0; j < chunk && launched < P->max_iter; ++j, ++launched) {
      const bool tb = timing_begin(kProbePcgAp, s);
      if (layout_kind(*L) == kLayoutHex33)
        pcg_ap_kernel<kLayoutHex33><<<G, kBlock, 0, s>>>(*L, coef, diag, v);
      else
        pcg_ap_kernel<kLayoutGeneric><<<G, kBlock, 0, s>>>(*L, coef, diag, v);
      if (tb) timing_end(kProbePcgAp, s);
      if (pd)
        pcg_update_kernel<true><<<G, kBlock, 0, s>>>(n, pd, x, v, hist, *P);
      else
        pcg_update_kernel<false><<<G, kBlock, 0, s>>>(n, pd, x, v, hist, *P);
      pcg_p_kernel<<<G, kBlock, 0, s>>>(n, v);
    }
    GBF_CHECK_LAUNCH();
    GBF_CHECK_CUDA(cudaMemcpyAsync(&hs, v.st, sizeof(hs), cudaMemcpyDeviceToHost, s));
    GBF_CHECK_CUDA(cudaStreamSynchronize(s));
  }
  R->iterations = hs.n_hist;
  R->status = (hs.status == GBF_RUNNING) ? GBF_MAX_ITER : hs.status;
  R->final_residual = hs.res;
  R->initial_residual = hs.res0;
  R->launches = 1 + 3 * launched;
  return GBF_OK;
}

// ---------------------------------------------------------------------------
// gbf_pcg_solve_f64_noalloc: the FP64 PCG solve without a caller workspace.
//
// Who needs it: callers that cannot allocate device memory at the moment they
// solve.  Examples are code that records its work into a CUDA stream capture
// (cudaMalloc and cudaFree are not allowed there, and cudaFree synchronises
// the whole device), real-time or embedded time loops that must never wait
// on the allocator or handle an out-of-memory error mid-step, and host
// programs that run under a fixed device-memory budget and pass the solver
// only their own input and output buffers.  Such a caller keeps x, b, the
// matrix and the history buffer; everything else the solve needs (the four
// iteration vectors r, z, p, Ap, the per-block partial sums and the state
// block) lives in one file-scope device array of fixed size.
//
// Limits and rules:
//   * at most kNoAllocMaxCells (1,048,576) cells; larger systems are refused
//     with GBF_ERR_ARG -- use gbf_pcg_solve_f64 with a workspace for them;
//   * the array occupies 32.1 MiB on every GPU that loads the library, until
//     the process exits;
//   * the first call on a device looks up the array's device address on that
//     device (cudaGetSymbolAddress, with the device current) and caches it;
//     make that first call before any stream capture that includes this
//     entry point;
//   * all calls share the one array, which keeps the previous call's
//     contents: the state block is cleared at the start of every call, and
//     calls whose work overlaps on the GPU (different streams, or different
//     host threads on one device) race on the array and must be serialised
//     by the caller;
//   * nothing here calls cudaMalloc, cudaFree or any allocating routine.
// ---------------------------------------------------------------------------
#include <mutex>

namespace gbf {

constexpr int kNoAllocMaxCells = 1 << 20;
constexpr size_t kNoAllocVecBytes = sizeof(double) * (size_t)kNoAllocMaxCells;  // 256-aligned
constexpr size_t kNoAllocPartialBytes = ((sizeof(double) * 2 * kMaxGrid) + 255) & ~(size_t)255;
constexpr size_t kNoAllocStateBytes = (sizeof(PcgState) + 255) & ~(size_t)255;
constexpr size_t kNoAllocBytes = 4 * kNoAllocVecBytes + kNoAllocPartialBytes + kNoAllocStateBytes;

static __device__ __align__(256) unsigned char g_pcg_noalloc_scratch[kNoAllocBytes];

constexpr int kNoAllocMaxDevices = 64;
static std::mutex g_noalloc_mu;
static void* g_noalloc_addr[kNoAllocMaxDevices] = {nullptr};

// Device address of the scratch array on the current device (looked up once
// per device).
static int noalloc_scratch(void** out) {
  int dev = 0;
  GBF_CHECK_CUDA(cudaGetDevice(&dev));
  GBF_REQUIRE(dev >= 0 && dev < kNoAllocMaxDevices, "pcg_noalloc: device %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (g_noalloc_addr[dev] == nullptr) {
    void* p = nullptr;
    GBF_CHECK_CUDA(cudaGetSymbolAddress(&p, g_pcg_noalloc_scratch));
    GBF_REQUIRE(p != nullptr, "pcg_noalloc: scratch address lookup returned NULL");
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return GBF_OK;
}

}  // namespace gbf

extern "C" int gbf_pcg_solve_f64_noalloc(const gbf_layout* L, const double* coef,
                                         const double* diag, const double* pd, const double* b,
                                         double* x, double* hist, const gbf_solve_params* P,
                                         gbf_solve_result* R, void* stream) {
  int rc = check_layout(L);
  if (rc) return rc;
  GBF_REQUIRE(P && R, "pcg_noalloc: NULL params/result");
  GBF_REQUIRE(P->max_iter >= 0, "pcg_noalloc: negative max_iter");
  const int n = L->n_cells;
  GBF_REQUIRE(n <= kNoAllocMaxCells,
              "pcg_noalloc: %d cells exceed the fixed scratch limit of %d cells; use "
              "gbf_pcg_solve_f64 with a workspace",
              n, kNoAllocMaxCells);
  memset(R, 0, sizeof(*R));
  if (n == 0) {
    const bool conv = (0 >= P->min_iter) && (0.0 < P->tolerance);
    R->iterations = 1;
    R->status = conv ? GBF_CONVERGED : (P->max_iter < 1 ? GBF_MAX_ITER : GBF_BREAKDOWN);
    return GBF_OK;
  }
  GBF_REQUIRE(diag && b && x && hist && (L->n_faces == 0 || coef), "pcg_noalloc: NULL pointer");
  void* scratch = nullptr;
  rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  cudaStream_t s = as_stream(stream);

  char* w = static_cast<char*>(scratch);
  PcgVecs v;
  v.r = reinterpret_cast<double*>(w);
  v.z = reinterpret_cast<double*>(w + kNoAllocVecBytes);
  v.p = reinterpret_cast<double*>(w + 2 * kNoAllocVecBytes);
  v.Ap = reinterpret_cast<double*>(w + 3 * kNoAllocVecBytes);
  v.partials = reinterpret_cast<double*>(w + 4 * kNoAllocVecBytes);
  v.st = reinterpret_cast<PcgState*>(w + 4 * kNoAllocVecBytes + kNoAllocPartialBytes);

  int G = reduction_grid();
  const int need = (n + kBlock - 1) / kBlock;
  if (G > need) G = need;
  // the state block (status, scalars, reduction tickets) must start at zero
  GBF_CHECK_CUDA(cudaMemsetAsync(v.st, 0, sizeof(PcgState), s));
  if (pd)
    pcg_init_kernel<true><<<G, kBlock, 0, s>>>(*L, coef, diag, pd, b, x, v, hist, *P);
  else
    pcg_init_kernel<false><<<G, kBlock, 0, s>>>(*L, coef, diag, pd, b, x, v, hist, *P);
  GBF_CHECK_LAUNCH();

  const int chunk = P->check_every > 0 ? P->check_every : 32;
  PcgState hs;
  GBF_CHECK_CUDA(cudaMemcpyAsync(&hs, v.st, sizeof(hs), cudaMemcpyDeviceToHost, s));
  GBF_CHECK_CUDA(cudaStreamSynchronize(s));
  int launched = 0;
  while (hs.status == GBF_RUNNING && launched < P->max_iter) {
    for (int j = 0; j < chunk && launched < P->max_iter; ++j, ++launched) {
      pcg_ap_kernel<kLayoutGeneric><<<G, kBlock, 0, s>>>(*L, coef, diag, v);
      if (pd)
        pcg_update_kernel<true><<<G, kBlock, 0, s>>>(n, pd, x, v, hist, *P);
      else
        pcg_update_kernel<false><<<G, kBlock, 0, s>>>(n, pd, x, v, hist, *P);
      pcg_p_kernel<<<G, kBlock, 0, s>>>(n, v);
    }
    GBF_CHECK_LAUNCH();
    GBF_CHECK_CUDA(cudaMemcpyAsync(&hs, v.st, sizeof(hs), cudaMemcpyDeviceToHost, s));
    GBF_CHECK_CUDA(cudaStreamSynchronize(s));
  }
  R->iterations = hs.n_hist;
  R->status = (hs.status == GBF_RUNNING) ? GBF_MAX_ITER : hs.status;
  R->final_residual = hs.res;
  R->initial_residual = hs.res0;
  R->launches = 1 + 3 * launched;
  return GBF_OK;
}
