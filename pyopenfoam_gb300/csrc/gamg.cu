// GAMG transfer kernels (solvers/gamg.py:249-393): Galerkin-style coarse
// coefficients, restriction by aggregate sums and prolongation by
// injection.  The aggregation itself depends on the mesh topology only and
// is built once on the host (gbf_gamg_aggregate, gbf_gamg_coarse_faces); the
// kernels here run per matrix and per V-cycle.  Every sum runs over its
// members in ascending index order, as the reference's scatter_add and its
// Python face loop do, so the coarse matrices and transfers are bitwise the
// reference's.
#include "common.cuh"

namespace gbf {

// dst[C] = (0 + src[i0]) + src[i1] + ... over the fine cells i of aggregate
// C in ascending order (scatter_add of the fine vector onto the aggregates).
__global__ void __launch_bounds__(kBlock)
    gamg_restrict_kernel(int n_coarse, const int32_t* __restrict__ ptr,
                         const int32_t* __restrict__ members, const double* __restrict__ src,
                         double* __restrict__ dst) {
  const int C = blockIdx.x * blockDim.x + threadIdx.x;
  if (C >= n_coarse) return;
  double s = 0.0;
  for (int k = __ldg(ptr + C), e = __ldg(ptr + C + 1); k < e; ++k)
    s = __dadd_rn(s, __ldg(src + __ldg(members + k)));
  dst[C] = s;
}

// Coarse lower/upper: the first fine face's value, then += every later fine
// face of the same aggregate pair in face order.
__global__ void __launch_bounds__(kBlock)
    gamg_coarse_coeff_kernel(int n_cfaces, const int32_t* __restrict__ ptr,
                             const int32_t* __restrict__ faces, const double* __restrict__ lower,
                             const double* __restrict__ upper, double* __restrict__ clower,
                             double* __restrict__ cupper) {
  const int K = blockIdx.x * blockDim.x + threadIdx.x;
  if (K >= n_cfaces) return;
  const int b = __ldg(ptr + K), e = __ldg(ptr + K + 1);
  const int f0 = __ldg(faces + b);
  double sl = __ldg(lower + f0), su = __ldg(upper + f0);
  for (int k = b + 1; k < e; ++k) {
    const int f = __ldg(faces + k);
    sl = __dadd_rn(sl, __ldg(lower + f));
    su = __dadd_rn(su, __ldg(upper + f));
  }
  clower[K] = sl;
  cupper[K] = su;
}

// x[i] = x[i] + e[f2c[i]]
__global__ void __launch_bounds__(kBlock)
    gamg_prolong_add_kernel(int n_fine, const int32_t* __restrict__ f2c,
                            const double* __restrict__ e, double* __restrict__ x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_fine) return;
  x[i] = __dadd_rn(x[i], __ldg(e + __ldg(f2c + i)));
}

}  // namespace gbf

using namespace gbf;

extern "C" int gbf_gamg_restrict_f64(int32_t n_coarse, const int32_t* agg_ptr,
                                     const int32_t* agg_cells, const double* fine,
                                     double* coarse, void* stream) {
  GBF_REQUIRE(n_coarse >= 0, "gamg_restrict: negative n_coarse");
  if (n_coarse == 0) return GBF_OK;
  GBF_REQUIRE(agg_ptr && agg_cells && fine && coarse, "gamg_restrict: NULL pointer");
  gamg_restrict_kernel<<<(n_coarse + kBlock - 1) / kBlock, kBlock, 0, as_stream(stream)>>>(
      n_coarse, agg_ptr, agg_cells, fine, coarse);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_gamg_coarse_coeffs_f64(int32_t n_cfaces, const int32_t* cf_ptr,
                                          const int32_t* cf_faces, const double* lower,
                                          const double* upper, double* coarse_lower,
                                          double* coarse_upper, void* stream) {
  GBF_REQUIRE(n_cfaces >= 0, "gamg_coarse_coeffs: negative n_cfaces");
  if (n_cfaces == 0) return GBF_OK;
  GBF_REQUIRE(cf_ptr && cf_faces && lower && upper && coarse_lower && coarse_upper,
              "gamg_coarse_coeffs: NULL pointer");
  gamg_coarse_coeff_kernel<<<(n_cfaces + kBlock - 1) / kBlock, kBlock, 0, as_stream(stream)>>>(
      n_cfaces, cf_ptr, cf_faces, lower, upper, coarse_lower, coarse_upper);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_gamg_prolong_add_f64(int32_t n_fine, const int32_t* f2c, const double* e,
                                        double* x, void* stream) {
  GBF_REQUIRE(n_fine >= 0, "gamg_prolong_add: negative n_fine");
  if (n_fine == 0) return GBF_OK;
  GBF_REQUIRE(f2c && e && x, "gamg_prolong_add: NULL pointer");
  gamg_prolong_add_kernel<<<(n_fine + kBlock - 1) / kBlock, kBlock, 0, as_stream(stream)>>>(
      n_fine, f2c, e, x);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}
