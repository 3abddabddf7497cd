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
#include "barrier.cuh"

namespace gbf {

struct PcgState {
  double rz, alpha, beta, res0, res, pAp;
  int iter, status, n_hist, pad;
  unsigned int ticket[4];
  GridBarrier bar;
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

// ---------------------------------------------------------------------------
// Single-launch PCG for launch-bound (small and medium) systems.
//
// The three phases of an iteration run inside one cooperative launch whose
// blocks are all resident, separated by a grid barrier; every block reduces
// the per-block partials itself in the same fixed order, so all blocks hold
// the same scalars and take the same decisions without a further barrier.
// Same arithmetic per element and same ResidualMonitor rules as the
// three-kernel form.  Vectors that other blocks rewrite during the launch
// (p, and the partials) are read from L2 (__ldcg), never through L1.
//
// Every barrier wait is bounded: after kBarrierPolls polls (a few seconds)
// the block records a fault and returns; a block waiting at a barrier that
// sees the fault returns within 16 polls.  The host turns a fault into
// GBF_DEVICE_TIMEOUT.
// ---------------------------------------------------------------------------
template <int KIND, bool PREC>
__global__ void __launch_bounds__(kBlock)
    pcg_persistent_kernel(gbf_layout L, const double* __restrict__ coef,
                          const double* __restrict__ diag, const double* __restrict__ pd,
                          const double* __restrict__ b, double* __restrict__ x, PcgVecs v,
                          double* hist, gbf_solve_params P) {
  __shared__ double sh[kBlock / 32];
  const int G = gridDim.x, n = L.n_cells;
  const int c0 = blockIdx.x * blockDim.x + threadIdx.x, cs = G * blockDim.x;
  const bool lead = blockIdx.x == 0 && threadIdx.x == 0;
  PcgState* st = v.st;
  GridBarrier* bar = &st->bar;
  double* partA = v.partials;       // p.Ap partials      [G]
  double* partB = v.partials + G;   // r.r, r.z partials  [2G]

  // r = b - A x, z = M^-1 r, p = z
  double rr = 0.0, rz = 0.0;
  for (int c = c0; c < n; c += cs) {
    const double y = cell_amul_k<KIND, double, double, false>(L, coef, diag, x, c, __ldg(x + c));
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
    partB[blockIdx.x] = rr;
    partB[G + blockIdx.x] = rz;
  }
  if (!grid_barrier(bar, G)) return;
  double s0 = reduce_partials(partB, G, sh);
  double s1 = reduce_partials(partB + G, G, sh);
  __shared__ double bc[2];
  if (threadIdx.x == 0) {
    bc[0] = s0;
    bc[1] = s1;
  }
  __syncthreads();
  const double res0 = sqrt(bc[0]);
  double rzv = bc[1], res = res0;
  int iter = 1, n_hist = 1;
  int status = monitor_converged(res0, res0, 0, P) ? GBF_CONVERGED
               : (P.max_iter < 1 ? GBF_MAX_ITER : GBF_RUNNING);
  if (lead) hist[0] = res0;

  for (int launched = 0; status == GBF_RUNNING && launched < P.max_iter; ++launched) {
    // Ap = A p, p.Ap
    double acc = 0.0;
    for (int c = c0; c < n; c += cs) {
      const double pc = __ldcg(v.p + c);
      const double y = cell_amul_k<KIND, double, double, false, true>(L, coef, diag, v.p, c, pc);
      v.Ap[c] = y;
      acc = fma(pc, y, acc);
    }
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) partA[blockIdx.x] = acc;
    if (!grid_barrier(bar, G)) return;
    s0 = reduce_partials(partA, G, sh);
    if (threadIdx.x == 0) bc[0] = s0;
    __syncthreads();
    const double pAp = bc[0];
    if (fabs(pAp) < 1e-30) {  // pcg.py:153-156: x returned as is
      status = GBF_BREAKDOWN;
      break;
    }
    const double alpha = rzv / pAp;
    // x += alpha p, r -= alpha Ap, z = M^-1 r, r.r, r.z
    rr = 0.0;
    rz = 0.0;
    for (int c = c0; c < n; c += cs) {
      const double xc = __dadd_rn(x[c], __dmul_rn(alpha, __ldcg(v.p + c)));
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
      partB[blockIdx.x] = rr;
      partB[G + blockIdx.x] = rz;
    }
    if (!grid_barrier(bar, G)) return;
    s0 = reduce_partials(partB, G, sh);
    s1 = reduce_partials(partB + G, G, sh);
    if (threadIdx.x == 0) {
      bc[0] = s0;
      bc[1] = s1;
    }
    __syncthreads();
    const int it = iter;
    res = sqrt(bc[0]);
    if (lead) hist[it] = res;
    n_hist = it + 1;
    if (monitor_converged(res, res0, it, P)) {
      status = GBF_CONVERGED;
      break;
    }
    const double beta = bc[1] / rzv;
    rzv = bc[1];
    iter = it + 1;
    if (it >= P.max_iter) {
      status = GBF_MAX_ITER;
      break;
    }
    // p = z + beta p
    for (int c = c0; c < n; c += cs) v.p[c] = __dadd_rn(v.z[c], __dmul_rn(beta, v.p[c]));
    if (!grid_barrier(bar, G)) return;
  }
  if (lead) {
    st->status = status;
    st->res = res;
    st->res0 = res0;
    st->n_hist = n_hist;
    st->iter = iter;
    st->rz = rzv;
  }
}

// Blocks of the single-launch PCG that can be resident at once (0 if the
// device cannot launch it cooperatively).
template <int KIND, bool PREC>
static int persistent_grid(int n) {
  int dev = 0, coop = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (!coop || sms <= 0) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pcg_persistent_kernel<KIND, PREC>,
                                                    kBlock, 0) != cudaSuccess || per_sm <= 0)
    return 0;
  long long g = (long long)per_sm * sms;
  const long long need = (n + kBlock - 1) / kBlock;
  if (g > need) g = need;
  if (g > kMaxGrid / 2) g = kMaxGrid / 2;  // partA + partB fit the partials buffer
  return g < 1 ? 1 : (int)g;
}

template <int KIND, bool PREC>
static cudaError_t launch_persistent(int grid, const gbf_layout* L, const double* coef,
                                     const double* diag, const double* pd, const double* b,
                                     double* x, PcgVecs v, double* hist,
                                     const gbf_solve_params* P, cudaStream_t s) {
  gbf_layout Lc = *L;
  gbf_solve_params Pc = *P;
  void* args[] = {&Lc, (void*)&coef, (void*)&diag, (void*)&pd, (void*)&b, &x, &v, &hist, &Pc};
  return cudaLaunchCooperativeKernel((const void*)pcg_persistent_kernel<KIND, PREC>,
                                     dim3(grid), dim3(kBlock), args, 0, s);
}

// Systems up to this many cells run the single-launch form under
// variant 0 (above it the per-iteration launch cost is negligible).
constexpr int kPersistentMaxCells = 1 << 21;

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
  ::gbf::NvtxScope nvtx_("gbf_pcg_solve_f64");
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

  GBF_REQUIRE(P->variant >= 0 && P->variant <= 2, "pcg: variant must be 0, 1 or 2");
  GBF_CHECK_CUDA(cudaMemsetAsync(v.st, 0, sizeof(PcgState), s));

  // single launch (variant 2, or variant 0 on a launch-bound system)
  if (P->variant == 2 || (P->variant == 0 && n <= kPersistentMaxCells)) {
    const bool hex = layout_kind(*L) == kLayoutHex33;
    const int Gp = hex ? (pd ? persistent_grid<kLayoutHex33, true>(n)
                             : persistent_grid<kLayoutHex33, false>(n))
                       : (pd ? persistent_grid<kLayoutGeneric, true>(n)
                             : persistent_grid<kLayoutGeneric, false>(n));
    if (Gp > 0) {
      cudaError_t e;
      if (hex)
        e = pd ? launch_persistent<kLayoutHex33, true>(Gp, L, coef, diag, pd, b, x, v, hist, P, s)
               : launch_persistent<kLayoutHex33, false>(Gp, L, coef, diag, pd, b, x, v, hist, P,
                                                        s);
      else
        e = pd ? launch_persistent<kLayoutGeneric, true>(Gp, L, coef, diag, pd, b, x, v, hist, P,
                                                         s)
               : launch_persistent<kLayoutGeneric, false>(Gp, L, coef, diag, pd, b, x, v, hist,
                                                          P, s);
      GBF_CHECK_CUDA(e);
      PcgState hs;
      GBF_CHECK_CUDA(cudaMemcpyAsync(&hs, v.st, sizeof(hs), cudaMemcpyDeviceToHost, s));
      GBF_CHECK_CUDA(cudaStreamSynchronize(s));
      R->iterations = hs.n_hist;
      R->status = hs.bar.fault ? GBF_DEVICE_TIMEOUT
                               : (hs.status == GBF_RUNNING ? GBF_MAX_ITER : hs.status);
      R->final_residual = hs.res;
      R->initial_residual = hs.res0;
      R->launches = 1;
      return GBF_OK;
    }
    GBF_REQUIRE(P->variant != 2, "pcg: the device cannot run the single-launch form");
  }

  int G = reduction_grid();
  const int need = (n + kBlock - 1) / kBlock;
  if (G > need) G = need;
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
// solve.  Examples are real-time or embedded time loops that must never wait
// on the allocator or handle an out-of-memory error mid-step, host programs
// (a C, C++ or Fortran CFD code) whose device memory is owned by their own
// pool or runs under a fixed budget and which hand the solver only their own
// input and output buffers, and plugin hosts that expose no allocator to the
// library they load.  Such a caller keeps x, b, the matrix and the history
// buffer; everything else the solve needs (the four iteration vectors r, z,
// p, Ap, the per-block partial sums and the state block) lives in one
// file-scope device array of fixed size.
//
// Limits and rules:
//   * at most kNoAllocMaxCells (1,048,576) cells; larger systems are refused
//     with GBF_ERR_ARG -- use gbf_pcg_solve_f64 with a workspace for them;
//   * the array occupies 32.1 MiB on every GPU that loads the library, until
//     the process exits;
//   * it always runs the three-kernel-per-iteration form (variant 0 and 1
//     alike); variant 2, which demands the single cooperative launch, is
//     refused with GBF_ERR_ARG, as is any value outside 0..2;
//   * the solve cannot run inside a stream capture: between chunks of
//     iterations it copies the state block to the host and synchronises the
//     stream, which a capturing stream refuses;
//   * every call looks up the array's device address on the current device
//     (cudaGetSymbolAddress; no cache, so an address never outlives a
//     cudaDeviceReset that reloads the module); the first call on a device
//     loads the module there if it is not loaded yet;
//   * all calls share the one array, which keeps the previous call's
//     contents: the state block is cleared at the start of every call, and
//     calls whose work overlaps on the GPU (different streams, or different
//     host threads on one device) race on the array and must be serialised
//     by the caller;
//   * nothing here calls cudaMalloc, cudaFree or any allocating routine.
// ---------------------------------------------------------------------------
namespace gbf {

constexpr int kNoAllocMaxCells = 1 << 20;
constexpr size_t kNoAllocVecBytes = sizeof(double) * (size_t)kNoAllocMaxCells;  // 256-aligned
constexpr size_t kNoAllocPartialBytes = ((sizeof(double) * 2 * kMaxGrid) + 255) & ~(size_t)255;
constexpr size_t kNoAllocStateBytes = (sizeof(PcgState) + 255) & ~(size_t)255;
constexpr size_t kNoAllocBytes = 4 * kNoAllocVecBytes + kNoAllocPartialBytes + kNoAllocStateBytes;

static __device__ __align__(256) unsigned char g_pcg_noalloc_scratch[kNoAllocBytes];

// Device address of the scratch array on the current device, looked up on
// every call (a few microseconds of host time).
static int noalloc_scratch(void** out) {
  void* p = nullptr;
  GBF_CHECK_CUDA(cudaGetSymbolAddress(&p, g_pcg_noalloc_scratch));
  GBF_REQUIRE(p != nullptr, "pcg_noalloc: scratch address lookup returned NULL");
  *out = p;
  return GBF_OK;
}

}  // namespace gbf

extern "C" int gbf_pcg_solve_f64_noalloc(const gbf_layout* L, const double* coef,
                                         const double* diag, const double* pd, const double* b,
                                         double* x, double* hist, const gbf_solve_params* P,
                                         gbf_solve_result* R, void* stream) {
  ::gbf::NvtxScope nvtx_("gbf_pcg_solve_f64_noalloc");
  int rc = check_layout(L);
  if (rc) return rc;
  GBF_REQUIRE(P && R, "pcg_noalloc: NULL params/result");
  GBF_REQUIRE(P->max_iter >= 0, "pcg_noalloc: negative max_iter");
  GBF_REQUIRE(P->variant == 0 || P->variant == 1,
              "pcg_noalloc: variant must be 0 or 1 (this entry point always runs three kernels "
              "per iteration; the single-launch form, variant 2, needs gbf_pcg_solve_f64)");
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
  const bool hex = layout_kind(*L) == kLayoutHex33;
  int launched = 0;
  while (hs.status == GBF_RUNNING && launched < P->max_iter) {
    for (int j = 0; j < chunk && launched < P->max_iter; ++j, ++launched) {
      if (hex)
        pcg_ap_kernel<kLayoutHex33><<<G, kBlock, 0, s>>>(*L, coef, diag, v);
      else
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
