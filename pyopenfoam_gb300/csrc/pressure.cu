// The pressure-corrector steps either side of the pressure solve:
//   HbyA = H / |A_p|                    rhie_chow.py:56-78 (compute_HbyA)
//   phi  = HbyA_f . S_f  (+ Rhie-Chow)  rhie_chow.py:81-250
//   U    = HbyA - alpha/|A_p| grad(p)   pressure_equation.py:187-266
//   phi  = phi + (1/A_p)_f (p_P - p_N) |S_f| delta_f
//                                       pressure_equation.py:269-332
//   adjustPhi on closed domains         pressure_equation.py:335-377
// One thread per face or per cell.  Every product, sum and quotient is an
// explicitly rounded intrinsic in the reference's order of operations
// (face value w*a + (1-w)*b, |S| as ATen's fma norm, the Gauss gradient
// accumulated like index_add_: owner-side faces, then neighbour-side faces,
// then boundary faces, each in ascending face order), so the results are
// bitwise the reference's; the boundary-flux sum of adjustPhi is a
// deterministic tree sum (the reference's torch.sum order is not
// reproduced).
#include <math.h>

#include "common.cuh"

namespace gbf {

__device__ __forceinline__ double inv_abs_clamped(double a) {
  const double m = fabs(a);
  return __ddiv_rn(1.0, m > 1e-30 ? m : 1e-30);
}

// w*a + (1 - w)*b with each operation rounded.
__device__ __forceinline__ double lerp_w(double w, double a, double b) {
  return __dadd_rn(__dmul_rn(w, a), __dmul_rn(__dsub_rn(1.0, w), b));
}

__device__ __forceinline__ double fma_norm3(const double* __restrict__ a) {
  const double x = __ldg(a), y = __ldg(a + 1), z = __ldg(a + 2);
  return __dsqrt_rn(__fma_rn(z, z, __fma_rn(y, y, __dmul_rn(x, x))));
}

__global__ void __launch_bounds__(kBlock)
    hbya_kernel(int n, const double* __restrict__ H, const double* __restrict__ A,
                double* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const double m = fabs(__ldg(A + c));
  const double d = m > 1e-30 ? m : 1e-30;
  for (int k = 0; k < 3; ++k) out[3 * (size_t)c + k] = __ddiv_rn(__ldg(H + 3 * (size_t)c + k), d);
}

__global__ void __launch_bounds__(kBlock)
    inv_abs_kernel(int n, const double* __restrict__ A, double* __restrict__ inv) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) inv[c] = inv_abs_clamped(__ldg(A + c));
}

// (1/A_p)_f (p_P - p_N) |S_f| delta_f of internal face f; ia = the per-cell
// 1 / max(|A_p|, 1e-30) (one division per cell, as the reference computes
// it before interpolating).
__device__ __forceinline__ double rc_term(int f, const int32_t* __restrict__ own,
                                          const int32_t* __restrict__ nei,
                                          const double* __restrict__ p,
                                          const double* __restrict__ inv_A,
                                          const double* __restrict__ areas,
                                          const double* __restrict__ delta,
                                          const double* __restrict__ w) {
  const int P = __ldg(own + f), N = __ldg(nei + f);
  const double wf = w ? __ldg(w + f) : 0.5;
  const double ia = lerp_w(wf, __ldg(inv_A + P), __ldg(inv_A + N));
  const double dp = __dsub_rn(__ldg(p + P), __ldg(p + N));
  return __dmul_rn(__dmul_rn(__dmul_rn(ia, dp), fma_norm3(areas + 3 * (size_t)f)),
                   __ldg(delta + f));
}

// phi_f = (w HbyA_P + (1-w) HbyA_N) . S_f on internal faces, HbyA_P . S_f on
// boundary faces (dot = ((0 + x) + y) + z); plus the Rhie-Chow term when p
// is given.
__global__ void __launch_bounds__(kBlock)
    face_flux_kernel(int nf, int nint, const int32_t* __restrict__ own,
                     const int32_t* __restrict__ nei, const double* __restrict__ HbyA,
                     const double* __restrict__ areas, const double* __restrict__ w,
                     const double* __restrict__ p, const double* __restrict__ A,
                     const double* __restrict__ delta, double* __restrict__ phi) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int P = __ldg(own + f);
  double s = 0.0;
  if (f < nint) {
    const int N = __ldg(nei + f);
    const double wf = w ? __ldg(w + f) : 0.5;
    for (int k = 0; k < 3; ++k) {
      const double hf = lerp_w(wf, __ldg(HbyA + 3 * (size_t)P + k), __ldg(HbyA + 3 * (size_t)N + k));
      s = __dadd_rn(s, __dmul_rn(hf, __ldg(areas + 3 * (size_t)f + k)));
    }
    if (p) s = __dadd_rn(s, rc_term(f, own, nei, p, A, areas, delta, w));
  } else {
    for (int k = 0; k < 3; ++k)
      s = __dadd_rn(s, __dmul_rn(__ldg(HbyA + 3 * (size_t)P + k), __ldg(areas + 3 * (size_t)f + k)));
    if (p) s = __dadd_rn(s, 0.0);
  }
  phi[f] = s;
}

// mode 0: out = Rhie-Chow correction (0 on boundary faces);
// mode 1: out = phi_in + correction on internal faces, phi_in on boundary.
__global__ void __launch_bounds__(kBlock)
    rc_kernel(int mode, int nf, int nint, const int32_t* __restrict__ own,
              const int32_t* __restrict__ nei, const double* __restrict__ p,
              const double* __restrict__ A, const double* __restrict__ areas,
              const double* __restrict__ delta, const double* __restrict__ w,
              const double* __restrict__ phi_in, double* __restrict__ out) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  if (f >= nint) {
    out[f] = mode == 0 ? 0.0 : __ldg(phi_in + f);
    return;
  }
  const double c = rc_term(f, own, nei, p, A, areas, delta, w);
  out[f] = mode == 0 ? c : __dadd_rn(__ldg(phi_in + f), c);
}

// U = HbyA - (alpha / |A_p|) (sum_f p_f S_f) / V, limited to |U| <= 1e4.
__global__ void __launch_bounds__(kBlock)
    correct_velocity_kernel(gbf_layout L, const int32_t* __restrict__ bnd_ptr,
                            const int32_t* __restrict__ bnd_face,
                            const double* __restrict__ areas, const double* __restrict__ w,
                            const double* __restrict__ V, const double* __restrict__ p,
                            const double* __restrict__ A, const double* __restrict__ HbyA,
                            double alpha, double* __restrict__ U) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= L.n_cells) return;
  double g[3] = {0.0, 0.0, 0.0};
  if (L.n_faces > 0) {
    const CellSlots cs = cell_slots(L, c);
    for (int side = 0; side < 2; ++side) {
      const int k0 = side == 0 ? 0 : cs.wo, k1 = side == 0 ? cs.wo : cs.wo + cs.wn;
      for (int k = k0; k < k1; ++k) {
        const int f = __ldg(L.slot_face + cs.base + 32 * k);
        if (f < 0) continue;
        const int P = __ldg(L.owner + f), N = __ldg(L.neighbour + f);
        const double pf = lerp_w(__ldg(w + f), __ldg(p + P), __ldg(p + N));
        for (int q = 0; q < 3; ++q) {
          const double t = __dmul_rn(pf, __ldg(areas + 3 * (size_t)f + q));
          g[q] = __dadd_rn(g[q], side == 0 ? t : -t);
        }
      }
    }
  }
  const double pc = __ldg(p + c);
  for (int i = __ldg(bnd_ptr + c), e = __ldg(bnd_ptr + c + 1); i < e; ++i) {
    const int f = __ldg(bnd_face + i);
    for (int q = 0; q < 3; ++q) g[q] = __dadd_rn(g[q], __dmul_rn(pc, __ldg(areas + 3 * (size_t)f + q)));
  }
  const double v = __ldg(V + c);
  const double vc = v > 1e-30 ? v : 1e-30;
  const double s = __dmul_rn(alpha, inv_abs_clamped(__ldg(A + c)));
  double u[3];
  for (int q = 0; q < 3; ++q)
    u[q] = __dsub_rn(__ldg(HbyA + 3 * (size_t)c + q), __dmul_rn(s, __ddiv_rn(g[q], vc)));
  double m = __dsqrt_rn(__fma_rn(u[2], u[2], __fma_rn(u[1], u[1], __dmul_rn(u[0], u[0]))));
  m = m > 1e-30 ? m : 1e-30;
  if (m > 1e4) {
    const double r = __ddiv_rn(1e4, m);
    for (int q = 0; q < 3; ++q) u[q] = __dmul_rn(u[q], r);
  }
  for (int q = 0; q < 3; ++q) U[3 * (size_t)c + q] = u[q];
}

// Sum of phi[nint..nf) by one block in a fixed order.
__global__ void __launch_bounds__(1024)
    boundary_sum_kernel(int nf, int nint, const double* __restrict__ phi,
                        double* __restrict__ out) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int f = nint + threadIdx.x; f < nf; f += blockDim.x) s = __dadd_rn(s, __ldg(phi + f));
  s = block_sum(s, sh);
  if (threadIdx.x == 0) *out = s;
}

__global__ void __launch_bounds__(kBlock)
    adjust_phi_kernel(int nf, int nint, const double* __restrict__ sum, double* __restrict__ phi) {
  const int f = nint + blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const double corr = __ddiv_rn(*sum, (double)(nf - nint));
  phi[f] = __dsub_rn(phi[f], corr);
}

inline int grid_of(long long n) { return (int)((n + kBlock - 1) / kBlock); }

}  // namespace gbf

using namespace gbf;

extern "C" int gbf_hbya_f64(int32_t n_cells, const double* H, const double* A_p, double* HbyA,
                            void* stream) {
  GBF_REQUIRE(n_cells >= 0, "hbya: negative n_cells");
  if (n_cells == 0) return GBF_OK;
  GBF_REQUIRE(H && A_p && HbyA, "hbya: NULL pointer");
  hbya_kernel<<<grid_of(n_cells), kBlock, 0, as_stream(stream)>>>(n_cells, H, A_p, HbyA);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_inv_abs_clamped_f64(int32_t n, const double* A, double* inv, void* stream) {
  GBF_REQUIRE(n >= 0, "inv_abs_clamped: negative n");
  if (n == 0) return GBF_OK;
  GBF_REQUIRE(A && inv, "inv_abs_clamped: NULL pointer");
  inv_abs_kernel<<<grid_of(n), kBlock, 0, as_stream(stream)>>>(n, A, inv);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_face_flux_f64(int32_t n_faces, int32_t n_internal, const int32_t* owner,
                                 const int32_t* neighbour, const double* HbyA,
                                 const double* face_areas, const double* weights, const double* p,
                                 const double* inv_A_p, const double* delta, double* phi,
                                 void* stream) {
  GBF_REQUIRE(n_faces >= 0 && n_internal >= 0 && n_internal <= n_faces,
              "face_flux: bad face counts");
  if (n_faces == 0) return GBF_OK;
  GBF_REQUIRE(owner && HbyA && face_areas && phi && (n_internal == 0 || neighbour) &&
                  (!p || (inv_A_p && delta)),
              "face_flux: NULL pointer");
  face_flux_kernel<<<grid_of(n_faces), kBlock, 0, as_stream(stream)>>>(
      n_faces, n_internal, owner, neighbour, HbyA, face_areas, weights, p, inv_A_p, delta, phi);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_rhie_chow_f64(int32_t n_faces, int32_t n_internal, const int32_t* owner,
                                 const int32_t* neighbour, const double* p, const double* inv_A_p,
                                 const double* face_areas, const double* delta,
                                 const double* weights, const double* phi_in, double* out,
                                 void* stream) {
  GBF_REQUIRE(n_faces >= 0 && n_internal >= 0 && n_internal <= n_faces,
              "rhie_chow: bad face counts");
  if (n_faces == 0) return GBF_OK;
  GBF_REQUIRE(out && (n_internal == 0 || (owner && neighbour && p && inv_A_p && face_areas &&
                                          delta)),
              "rhie_chow: NULL pointer");
  rc_kernel<<<grid_of(n_faces), kBlock, 0, as_stream(stream)>>>(
      phi_in ? 1 : 0, n_faces, n_internal, owner, neighbour, p, inv_A_p, face_areas, delta,
      weights,
      phi_in, out);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_correct_velocity_f64(const gbf_layout* L, const int32_t* bnd_ptr,
                                        const int32_t* bnd_face, const double* face_areas,
                                        const double* weights, const double* volumes,
                                        const double* p, const double* A_p, const double* HbyA,
                                        double alpha, double* U, void* stream) {
  int rc = check_layout(L);
  if (rc) return rc;
  if (L->n_cells == 0) return GBF_OK;
  GBF_REQUIRE(bnd_ptr && bnd_face && face_areas && volumes && p && A_p && HbyA && U &&
                  (L->n_faces == 0 || weights),
              "correct_velocity: NULL pointer");
  correct_velocity_kernel<<<grid_of(L->n_cells), kBlock, 0, as_stream(stream)>>>(
      *L, bnd_ptr, bnd_face, face_areas, weights, volumes, p, A_p, HbyA, alpha, U);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_boundary_flux_sum_f64(int32_t n_faces, int32_t n_internal, const double* phi,
                                         double* sum, void* stream) {
  GBF_REQUIRE(n_faces >= 0 && n_internal >= 0 && n_internal <= n_faces,
              "boundary_flux_sum: bad face counts");
  GBF_REQUIRE(sum && (n_faces == n_internal || phi), "boundary_flux_sum: NULL pointer");
  boundary_sum_kernel<<<1, 1024, 0, as_stream(stream)>>>(n_faces, n_internal, phi, sum);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_adjust_phi_f64(int32_t n_faces, int32_t n_internal, const double* sum,
                                  double* phi, void* stream) {
  GBF_REQUIRE(n_faces >= 0 && n_internal >= 0 && n_internal <= n_faces,
              "adjust_phi: bad face counts");
  if (n_faces == n_internal) return GBF_OK;
  GBF_REQUIRE(sum && phi, "adjust_phi: NULL pointer");
  adjust_phi_kernel<<<grid_of(n_faces - n_internal), kBlock, 0, as_stream(stream)>>>(
      n_faces, n_internal, sum, phi);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}
