// Finite-volume assembly of the LDU coefficients:
//   fvm.laplacian (discretisation/operators.py:432-518) and
//   fvm.div with the upwind scheme (discretisation/operators.py:351-429).
//
// Face kernels write lower/upper in face order; cell kernels sum the
// diagonal with the same per-cell face order as the reference's
// scatter_add (owner-side faces ascending, then neighbour-side faces
// ascending, then boundary faces ascending), one rounding per operation, so
// the coefficients are bitwise identical to the reference's.
#include <math.h>

#include "common.cuh"

namespace gbf {

// |S| of a face area vector as ATen's CPU p=2 norm over a length-3 row
// accumulates it: sqrt(fma(z, z, fma(y, y, x*x))).
__device__ __forceinline__ double face_smag(const double* __restrict__ a) {
  const double x = a[0], y = a[1], z = a[2];
  return __dsqrt_rn(__fma_rn(z, z, __fma_rn(y, y, __dmul_rn(x, x))));
}

// Face diffusivity: constant, per face, or linearly interpolated from cells
// (LinearInterpolation.interpolate, interpolation.py:101-145:
//  w*phi_P + (1 - w)*phi_N on internal faces, phi_P on boundary faces).
// Mode 3 is the pressure equation's 1/A_p: the per-cell values are
// 1 / max(|A_p|, 1e-30) (pressure_equation.py:103-104), then interpolated
// like mode 2.
struct DiffSpec {
  int mode;            // 0 constant, 1 per face, 2 per cell, 3 per-cell 1/|A_p|
  double value;        // mode 0
  const double* face;  // mode 1: [n_faces]
  const double* cell;  // modes 2, 3: [n_cells]
  const double* w;     // modes 2, 3: [n_faces] interpolation weights
};

__device__ __forceinline__ double cell_D(const DiffSpec& D, int c) {
  const double v = __ldg(D.cell + c);
  if (D.mode != 3) return v;
  const double a = fabs(v);
  return __ddiv_rn(1.0, a < 1e-30 ? 1e-30 : a);  // clamp(min) keeps NaN
}

__device__ __forceinline__ double face_D(const DiffSpec& D, int f, int p, int q, bool internal) {
  if (D.mode == 0) return D.value;
  if (D.mode == 1) return __ldg(D.face + f);
  const double dp = cell_D(D, p);
  if (!internal) return dp;
  const double w = __ldg(D.w + f);
  return __dadd_rn(__dmul_rn(w, dp), __dmul_rn(__dsub_rn(1.0, w), cell_D(D, q)));
}

__global__ void __launch_bounds__(kBlock)
    lap_face_kernel(int nint, const int32_t* __restrict__ own, const int32_t* __restrict__ nei,
                    const double* __restrict__ areas, const double* __restrict__ delta,
                    DiffSpec D, const double* __restrict__ V, double* __restrict__ lower,
                    double* __restrict__ upper) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nint) return;
  const int p = __ldg(own + f), q = __ldg(nei + f);
  double c = __dmul_rn(face_D(D, f, p, q, true), face_smag(areas + 3 * (size_t)f));
  c = __dmul_rn(c, __ldg(delta + f));
  lower[f] = __ddiv_rn(-c, __ldg(V + p));
  upper[f] = __ddiv_rn(-c, __ldg(V + q));
}

// diag[c] = ((0 + sum_own c/V) + sum_nei c/V) + sum_bnd c_b/V, using
// c/V = -lower[f] (owner side) and -upper[f] (neighbour side) exactly.
__global__ void __launch_bounds__(kBlock)
    lap_diag_kernel(gbf_layout L, const double* __restrict__ lower,
                    const double* __restrict__ upper, const int32_t* __restrict__ bnd_ptr,
                    const int32_t* __restrict__ bnd_face, const double* __restrict__ areas,
                    const double* __restrict__ delta, DiffSpec D, const double* __restrict__ V,
                    int has_bnd, double* __restrict__ diag) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= L.n_cells) return;
  double so = 0.0, sn = 0.0;
  if (L.n_faces > 0) {
    const CellSlots cs = cell_slots(L, c);
    for (int k = 0; k < cs.wo; ++k) {
      const int f = __ldg(L.slot_face + cs.base + 32 * k);
      if (f >= 0) so = __dadd_rn(so, -__ldg(lower + f));
    }
    for (int k = 0; k < cs.wn; ++k) {
      const int f = __ldg(L.slot_face + cs.base + 32 * (cs.wo + k));
      if (f >= 0) sn = __dadd_rn(sn, -__ldg(upper + f));
    }
  }
  double d = __dadd_rn(0.0, so);
  d = __dadd_rn(d, sn);
  if (has_bnd) {
    double sb = 0.0;
    const double vc = __ldg(V + c);
    for (int k = __ldg(bnd_ptr + c); k < __ldg(bnd_ptr + c + 1); ++k) {
      const int f = __ldg(bnd_face + k);
      double cb = __dmul_rn(face_D(D, f, c, c, false), face_smag(areas + 3 * (size_t)f));
      cb = __dmul_rn(cb, __ldg(delta + f));
      sb = __dadd_rn(sb, __ddiv_rn(cb, vc));
    }
    d = __dadd_rn(d, sb);
  }
  diag[c] = d;
}

// Upwind convection: F+ = F if F >= 0 else 0, F- = F if F < 0 else 0;
// lower = F-/V_P, upper = F+/V_N.
__global__ void __launch_bounds__(kBlock)
    div_face_kernel(int nint, const int32_t* __restrict__ own, const int32_t* __restrict__ nei,
                    const double* __restrict__ flux, const double* __restrict__ V,
                    double* __restrict__ lower, double* __restrict__ upper) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nint) return;
  const double F = __ldg(flux + f);
  const bool pos = F >= 0.0;
  lower[f] = __ddiv_rn(pos ? 0.0 : F, __ldg(V + __ldg(own + f)));
  upper[f] = __ddiv_rn(pos ? F : 0.0, __ldg(V + __ldg(nei + f)));
}

// diag = (0 + sum_own (-F+)/V_P) + sum_nei |F-|/V_N
__global__ void __launch_bounds__(kBlock)
    div_diag_kernel(gbf_layout L, const double* __restrict__ flux, const double* __restrict__ V,
                    double* __restrict__ diag) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= L.n_cells) return;
  const double vc = __ldg(V + c);
  double so = 0.0, sn = 0.0;
  if (L.n_faces > 0) {
    const CellSlots cs = cell_slots(L, c);
    for (int k = 0; k < cs.wo; ++k) {
      const int f = __ldg(L.slot_face + cs.base + 32 * k);
      if (f < 0) continue;
      const double F = __ldg(flux + f);
      so = __dadd_rn(so, __ddiv_rn(-(F >= 0.0 ? F : 0.0), vc));
    }
    for (int k = 0; k < cs.wn; ++k) {
      const int f = __ldg(L.slot_face + cs.base + 32 * (cs.wo + k));
      if (f < 0) continue;
      const double F = __ldg(flux + f);
      sn = __dadd_rn(sn, __ddiv_rn(fabs(F >= 0.0 ? 0.0 : F), vc));
    }
  }
  diag[c] = __dadd_rn(__dadd_rn(0.0, so), sn);
}

// Linear-interpolation weights w = |d_N| / (|d_P| + |d_N|) of internal faces
// (weights.py:21-95), boundary faces 1; distances with the same fma norm.
__global__ void __launch_bounds__(kBlock)
    centre_weights_kernel(int nint, int nfaces, const int32_t* __restrict__ own,
                          const int32_t* __restrict__ nei, const double* __restrict__ cc,
                          const double* __restrict__ fc, double* __restrict__ w) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nfaces) return;
  if (f >= nint) {
    w[f] = 1.0;
    return;
  }
  const int p = __ldg(own + f), q = __ldg(nei + f);
  double a[3], b[3];
  for (int k = 0; k < 3; ++k) {
    a[k] = __dsub_rn(__ldg(fc + 3 * (size_t)f + k), __ldg(cc + 3 * (size_t)p + k));
    b[k] = __dsub_rn(__ldg(fc + 3 * (size_t)f + k), __ldg(cc + 3 * (size_t)q + k));
  }
  const double dP = face_smag(a), dN = face_smag(b);
  const double den = __dadd_rn(dP, dN);
  w[f] = __ddiv_rn(dN, den > 1e-30 ? den : 1.0);
}

}  // namespace gbf

using namespace gbf;

static DiffSpec make_spec(int mode, double value, const double* Dface, const double* Dcell,
                          const double* w) {
  DiffSpec D;
  D.mode = mode;
  D.value = value;
  D.face = Dface;
  D.cell = Dcell;
  D.w = w;
  return D;
}

extern "C" int gbf_laplacian_assemble_f64(const gbf_layout* L, int32_t n_faces_total,
                                          const int32_t* owner_all, const int32_t* bnd_ptr,
                                          const int32_t* bnd_face, const double* face_areas,
                                          const double* delta, int32_t d_mode, double d_value,
                                          const double* d_face, const double* d_cell,
                                          const double* weights, const double* volumes,
                                          double* lower, double* upper, double* diag,
                                          void* stream) {
  int rc = check_layout(L);
  if (rc) return rc;
  const int n = L->n_cells, nint = L->n_faces;
  GBF_REQUIRE(n_faces_total >= nint, "laplacian: n_faces_total < n_internal_faces");
  GBF_REQUIRE(d_mode >= 0 && d_mode <= 2, "laplacian: bad diffusivity mode %d", d_mode);
  GBF_REQUIRE(d_mode != 1 || d_face, "laplacian: per-face diffusivity is NULL");
  GBF_REQUIRE(d_mode != 2 || (d_cell && weights), "laplacian: per-cell diffusivity is NULL");
  if (n == 0) return GBF_OK;
  GBF_REQUIRE(diag && volumes && (n_faces_total == 0 || (face_areas && delta)),
              "laplacian: NULL pointer");
  const bool has_bnd = n_faces_total > nint;
  GBF_REQUIRE(!has_bnd || (bnd_ptr && bnd_face && owner_all), "laplacian: NULL boundary lists");
  const DiffSpec D = make_spec(d_mode, d_value, d_face, d_cell, weights);
  cudaStream_t s = as_stream(stream);
  if (nint > 0) {
    GBF_REQUIRE(lower && upper && L->owner && L->neighbour, "laplacian: NULL pointer");
    lap_face_kernel<<<(nint + kBlock - 1) / kBlock, kBlock, 0, s>>>(
        nint, L->owner, L->neighbour, face_areas, delta, D, volumes, lower, upper);
    GBF_CHECK_LAUNCH();
  }
  lap_diag_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, s>>>(
      *L, lower, upper, bnd_ptr, bnd_face, face_areas, delta, D, volumes, has_bnd ? 1 : 0, diag);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_div_upwind_assemble_f64(const gbf_layout* L, const double* flux,
                                           const double* volumes, double* lower, double* upper,
                                           double* diag, void* stream) {
  int rc = check_layout(L);
  if (rc) return rc;
  const int n = L->n_cells, nint = L->n_faces;
  if (n == 0) return GBF_OK;
  GBF_REQUIRE(diag && volumes && (nint == 0 || (flux && lower && upper)),
              "div_upwind: NULL pointer");
  cudaStream_t s = as_stream(stream);
  if (nint > 0) {
    div_face_kernel<<<(nint + kBlock - 1) / kBlock, kBlock, 0, s>>>(nint, L->owner, L->neighbour,
                                                                    flux, volumes, lower, upper);
    GBF_CHECK_LAUNCH();
  }
  div_diag_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, s>>>(*L, flux, volumes, diag);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_centre_weights_f64(int32_t n_internal, int32_t n_faces, const int32_t* owner,
                                      const int32_t* neighbour, const double* cell_centres,
                                      const double* face_centres, double* weights,
                                      void* stream) {
  GBF_REQUIRE(n_internal >= 0 && n_faces >= n_internal, "centre_weights: bad sizes");
  if (n_faces == 0) return GBF_OK;
  GBF_REQUIRE(weights && (n_internal == 0 || (owner && neighbour && cell_centres && face_centres)),
              "centre_weights: NULL pointer");
  centre_weights_kernel<<<(n_faces + kBlock - 1) / kBlock, kBlock, 0, as_stream(stream)>>>(
      n_internal, n_faces, owner, neighbour, cell_centres, face_centres, weights);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

// ---------------------------------------------------------------------------
// Backward of the Laplacian assembly with respect to a per-face diffusivity.
// For an internal face c_f = D_f |S_f| delta_f enters lower_f = -c_f/V_P,
// upper_f = -c_f/V_N, diag_P += c_f/V_P, diag_N += c_f/V_N; a boundary face
// enters diag_P += c_f/V_P.  Hence
//   dL/dD_f = |S_f| delta_f ((g_diag_P - g_lower_f)/V_P + (g_diag_N - g_upper_f)/V_N)
//   dL/dD_b = |S_b| delta_b g_diag_P / V_P.
// One thread per face, no atomics.  (No reference counterpart as a kernel:
// the reference gets this from autograd through its torch ops.)
// ---------------------------------------------------------------------------
namespace gbf {
__global__ void __launch_bounds__(kBlock)
    lap_grad_gamma_kernel(int nint, int nfaces, const int32_t* __restrict__ own_all,
                          const int32_t* __restrict__ nei, const double* __restrict__ areas,
                          const double* __restrict__ delta, const double* __restrict__ V,
                          const double* __restrict__ gl, const double* __restrict__ gu,
                          const double* __restrict__ gd, double* __restrict__ gD) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nfaces) return;
  const int p = __ldg(own_all + f);
  const double sd = face_smag(areas + 3 * (size_t)f) * __ldg(delta + f);
  double g = (__ldg(gd + p) - (f < nint ? __ldg(gl + f) : 0.0)) / __ldg(V + p);
  if (f < nint) {
    const int q = __ldg(nei + f);
    g += (__ldg(gd + q) - __ldg(gu + f)) / __ldg(V + q);
  }
  gD[f] = sd * g;
}

// DifferentiableLinearSolve.backward gradients
// (differentiable/linear_solver.py:139-149), reference rounding:
//   g_diag = (-lam)*x, g_lower_f = (-lam[own])*x[nei], g_upper_f = (-lam[nei])*x[own]
__global__ void __launch_bounds__(kBlock)
    dls_grad_kernel(int n, int nint, const int32_t* __restrict__ own,
                    const int32_t* __restrict__ nei, const double* __restrict__ lam,
                    const double* __restrict__ x, double* __restrict__ gd,
                    double* __restrict__ gl, double* __restrict__ gu) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) gd[i] = __dmul_rn(-__ldg(lam + i), __ldg(x + i));
  if (i < nint) {
    const int p = __ldg(own + i), q = __ldg(nei + i);
    gl[i] = __dmul_rn(-__ldg(lam + p), __ldg(x + q));
    gu[i] = __dmul_rn(-__ldg(lam + q), __ldg(x + p));
  }
}

// Fused adjoint face gradient of a Laplacian system A(D) x = b with respect
// to the per-face diffusivity, from the adjoint lam (A^T lam = dL/dx) and x:
// dL/dD_f = -lam^T (dA/dD_f) x
//         = |S| delta ((x_N - x_P)(lam_P/V_P - lam_N/V_N))   (internal)
//         = -|S| delta lam_P x_P / V_P                       (boundary)
// i.e. dls_grad followed by lap_grad_gamma without materialising the
// per-coefficient gradients.  `accumulate` adds into gD.
__global__ void __launch_bounds__(kBlock)
    adjoint_face_grad_kernel(int nint, int nfaces, const int32_t* __restrict__ own_all,
                             const int32_t* __restrict__ nei, const double* __restrict__ areas,
                             const double* __restrict__ delta, const double* __restrict__ V,
                             const double* __restrict__ lam, const double* __restrict__ x,
                             double scale, int accumulate, double* __restrict__ gD) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nfaces) return;
  const int p = __ldg(own_all + f);
  const double sd = face_smag(areas + 3 * (size_t)f) * __ldg(delta + f);
  double g;
  if (f < nint) {
    const int q = __ldg(nei + f);
    g = (__ldg(x + q) - __ldg(x + p)) * (__ldg(lam + p) / __ldg(V + p) - __ldg(lam + q) / __ldg(V + q));
  } else {
    g = -__ldg(lam + p) * __ldg(x + p) / __ldg(V + p);
  }
  g = scale * sd * g;
  gD[f] = accumulate ? gD[f] + g : g;
}
}  // namespace gbf

extern "C" int gbf_laplacian_grad_gamma_f64(const gbf_layout* L, int32_t n_faces_total,
                                            const int32_t* owner_all, const double* face_areas,
                                            const double* delta, const double* volumes,
                                            const double* g_lower, const double* g_upper,
                                            const double* g_diag, double* g_gamma,
                                            void* stream) {
  int rc = check_layout(L);
  if (rc) return rc;
  GBF_REQUIRE(n_faces_total >= L->n_faces, "laplacian_grad: n_faces_total < n_internal_faces");
  if (n_faces_total == 0) return GBF_OK;
  GBF_REQUIRE(owner_all && face_areas && delta && volumes && g_diag && g_gamma &&
                  (L->n_faces == 0 || (g_lower && g_upper && L->neighbour)),
              "laplacian_grad: NULL pointer");
  lap_grad_gamma_kernel<<<(n_faces_total + kBlock - 1) / kBlock, kBlock, 0, as_stream(stream)>>>(
      L->n_faces, n_faces_total, owner_all, L->neighbour, face_areas, delta, volumes, g_lower,
      g_upper, g_diag, g_gamma);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_dls_grads_f64(const gbf_layout* L, const double* lam, const double* x,
                                 double* g_diag, double* g_lower, double* g_upper, void* stream) {
  int rc = check_layout(L);
  if (rc) return rc;
  const int n = L->n_cells, nint = L->n_faces;
  const int m = n > nint ? n : nint;
  if (m == 0) return GBF_OK;
  GBF_REQUIRE(lam && x && g_diag && (nint == 0 || (g_lower && g_upper && L->owner)),
              "dls_grads: NULL pointer");
  dls_grad_kernel<<<(m + kBlock - 1) / kBlock, kBlock, 0, as_stream(stream)>>>(
      n, nint, L->owner, L->neighbour, lam, x, g_diag, g_lower, g_upper);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_adjoint_face_grad_f64(const gbf_layout* L, int32_t n_faces_total,
                                         const int32_t* owner_all, const double* face_areas,
                                         const double* delta, const double* volumes,
                                         const double* lam, const double* x, double scale,
                                         int32_t accumulate, double* g_gamma, void* stream) {
  int rc = check_layout(L);
  if (rc) return rc;
  GBF_REQUIRE(n_faces_total >= L->n_faces, "adjoint_face_grad: n_faces_total < n_internal");
  if (n_faces_total == 0) return GBF_OK;
  GBF_REQUIRE(owner_all && face_areas && delta && volumes && lam && x && g_gamma &&
                  (L->n_faces == 0 || L->neighbour),
              "adjoint_face_grad: NULL pointer");
  adjoint_face_grad_kernel<<<(n_faces_total + kBlock - 1) / kBlock, kBlock, 0,
                             as_stream(stream)>>>(L->n_faces, n_faces_total, owner_all,
                                                  L->neighbour, face_areas, delta, volumes, lam, x,
                                                  scale, accumulate, g_gamma);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

// ---------------------------------------------------------------------------
// DifferentiableLaplacian (differentiable/operators.py:409-643): the
// explicit Laplacian of a cell field and its backward.
//
// forward (:421-522), per cell c, faces in ascending order on each side:
//   flux_f = ((D_f * (phi_N - phi_P)) * |S_f|) * delta_f
//   lap = (0 + sum_own flux) + sum_nei (-flux)
//         [+ sum_bnd ((D_b * |S_b|) * delta_b) * phi_c]      (if boundary faces)
//   lap /= max(V_c, 1e-30)
// The phi-gradient of backward (:542-567) is the same operator applied to
// grad_output.  Each face flux is recomputed by both of its cells (same
// operands, same roundings), so the cell gather needs no scatter and no
// atomics.
// ---------------------------------------------------------------------------
namespace gbf {

__device__ __forceinline__ double clamp_volume(double v) { return v < 1e-30 ? 1e-30 : v; }

__global__ void __launch_bounds__(kBlock)
    explicit_lap_kernel(gbf_layout L, const int32_t* __restrict__ bnd_ptr,
                        const int32_t* __restrict__ bnd_face, const double* __restrict__ areas,
                        const double* __restrict__ delta, DiffSpec D,
                        const double* __restrict__ V, const double* __restrict__ phi,
                        int has_bnd, double* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= L.n_cells) return;
  const double pc = __ldg(phi + c);
  double so = 0.0, sn = 0.0;
  if (L.n_faces > 0) {
    const CellSlots cs = cell_slots(L, c);
    for (int k = 0; k < cs.wo; ++k) {
      const int i = cs.base + 32 * k;
      const int f = __ldg(L.slot_face + i);
      if (f < 0) continue;
      const int q = __ldg(L.slot_col + i);
      double fl = __dmul_rn(face_D(D, f, c, q, true), __dsub_rn(__ldg(phi + q), pc));
      fl = __dmul_rn(fl, face_smag(areas + 3 * (size_t)f));
      fl = __dmul_rn(fl, __ldg(delta + f));
      so = __dadd_rn(so, fl);
    }
    for (int k = 0; k < cs.wn; ++k) {
      const int i = cs.base + 32 * (cs.wo + k);
      const int f = __ldg(L.slot_face + i);
      if (f < 0) continue;
      const int p = __ldg(L.slot_col + i);
      double fl = __dmul_rn(face_D(D, f, p, c, true), __dsub_rn(pc, __ldg(phi + p)));
      fl = __dmul_rn(fl, face_smag(areas + 3 * (size_t)f));
      fl = __dmul_rn(fl, __ldg(delta + f));
      sn = __dadd_rn(sn, -fl);
    }
  }
  double y = __dadd_rn(0.0, so);
  y = __dadd_rn(y, sn);
  if (has_bnd) {
    double sb = 0.0;
    for (int k = __ldg(bnd_ptr + c); k < __ldg(bnd_ptr + c + 1); ++k) {
      const int f = __ldg(bnd_face + k);
      double cb = __dmul_rn(face_D(D, f, c, c, false), face_smag(areas + 3 * (size_t)f));
      cb = __dmul_rn(cb, __ldg(delta + f));
      sb = __dadd_rn(sb, __dmul_rn(cb, pc));
    }
    y = __dadd_rn(y, sb);
  }
  out[c] = __ddiv_rn(y, clamp_volume(__ldg(V + c)));
}

// D-gradient per face (:570-600):
//   internal: (((g_P/V_P - g_N/V_N) * (phi_N - phi_P)) * |S|) * delta
//   boundary: (((g_P/V_P) * phi_P) * |S|) * delta
__global__ void __launch_bounds__(kBlock)
    explicit_lap_grad_d_kernel(int nint, int nfaces, const int32_t* __restrict__ own_all,
                               const int32_t* __restrict__ nei, const double* __restrict__ areas,
                               const double* __restrict__ delta, const double* __restrict__ V,
                               const double* __restrict__ phi, const double* __restrict__ g,
                               double* __restrict__ gface) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nfaces) return;
  const int p = __ldg(own_all + f);
  const double gp = __ddiv_rn(__ldg(g + p), clamp_volume(__ldg(V + p)));
  double a;
  if (f < nint) {
    const int q = __ldg(nei + f);
    const double gq = __ddiv_rn(__ldg(g + q), clamp_volume(__ldg(V + q)));
    a = __dmul_rn(__dsub_rn(gp, gq), __dsub_rn(__ldg(phi + q), __ldg(phi + p)));
  } else {
    a = __dmul_rn(gp, __ldg(phi + p));
  }
  a = __dmul_rn(a, face_smag(areas + 3 * (size_t)f));
  gface[f] = __dmul_rn(a, __ldg(delta + f));
}

// Per-cell D (:608-625): ((0 + sum_own gf*0.5) + sum_nei gf*0.5) [+ sum_bnd gf].
__global__ void __launch_bounds__(kBlock)
    face_grad_to_cells_kernel(gbf_layout L, const int32_t* __restrict__ bnd_ptr,
                              const int32_t* __restrict__ bnd_face,
                              const double* __restrict__ gface, int has_bnd,
                              double* __restrict__ gcell) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= L.n_cells) return;
  double so = 0.0, sn = 0.0;
  if (L.n_faces > 0) {
    const CellSlots cs = cell_slots(L, c);
    for (int k = 0; k < cs.wo; ++k) {
      const int f = __ldg(L.slot_face + cs.base + 32 * k);
      if (f >= 0) so = __dadd_rn(so, __dmul_rn(__ldg(gface + f), 0.5));
    }
    for (int k = 0; k < cs.wn; ++k) {
      const int f = __ldg(L.slot_face + cs.base + 32 * (cs.wo + k));
      if (f >= 0) sn = __dadd_rn(sn, __dmul_rn(__ldg(gface + f), 0.5));
    }
  }
  double y = __dadd_rn(0.0, so);
  y = __dadd_rn(y, sn);
  if (has_bnd) {
    double sb = 0.0;
    for (int k = __ldg(bnd_ptr + c); k < __ldg(bnd_ptr + c + 1); ++k)
      sb = __dadd_rn(sb, __ldg(gface + __ldg(bnd_face + k)));
    y = __dadd_rn(y, sb);
  }
  gcell[c] = y;
}

// Scalar D: the sum of the face gradients in one 1024-thread block, in a
// fixed order (strided per-thread sums, then the warp / block tree), so the
// result is reproducible run to run.
constexpr int kSumBlock = 1024;
__global__ void __launch_bounds__(kSumBlock)
    fixed_order_sum_kernel(int n, const double* __restrict__ a, double* __restrict__ out) {
  __shared__ double sh[kSumBlock / 32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += kSumBlock) s = __dadd_rn(s, __ldg(a + i));
  s = block_sum(s, sh);
  if (threadIdx.x == 0) *out = s;
}

}  // namespace gbf

extern "C" int gbf_explicit_laplacian_f64(const gbf_layout* L, int32_t n_faces_total,
                                          const int32_t* bnd_ptr, const int32_t* bnd_face,
                                          const double* face_areas, const double* delta,
                                          int32_t d_mode, double d_value, const double* d_face,
                                          const double* d_cell, const double* weights,
                                          const double* volumes, const double* phi, double* out,
                                          void* stream) {
  int rc = check_layout(L);
  if (rc) return rc;
  const int n = L->n_cells, nint = L->n_faces;
  GBF_REQUIRE(n_faces_total >= nint, "explicit_laplacian: n_faces_total < n_internal_faces");
  GBF_REQUIRE(d_mode >= 0 && d_mode <= 2, "explicit_laplacian: bad diffusivity mode %d", d_mode);
  GBF_REQUIRE(d_mode != 1 || d_face, "explicit_laplacian: per-face diffusivity is NULL");
  GBF_REQUIRE(d_mode != 2 || (d_cell && (nint == 0 || weights)),
              "explicit_laplacian: per-cell diffusivity is NULL");
  if (n == 0) return GBF_OK;
  GBF_REQUIRE(volumes && phi && out && (n_faces_total == 0 || (face_areas && delta)),
              "explicit_laplacian: NULL pointer");
  const bool has_bnd = n_faces_total > nint;
  GBF_REQUIRE(!has_bnd || (bnd_ptr && bnd_face), "explicit_laplacian: NULL boundary lists");
  const DiffSpec D = make_spec(d_mode, d_value, d_face, d_cell, weights);
  explicit_lap_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, as_stream(stream)>>>(
      *L, bnd_ptr, bnd_face, face_areas, delta, D, volumes, phi, has_bnd ? 1 : 0, out);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_explicit_laplacian_grad_d_f64(const gbf_layout* L, int32_t n_faces_total,
                                                 const int32_t* owner_all,
                                                 const int32_t* bnd_ptr, const int32_t* bnd_face,
                                                 const double* face_areas, const double* delta,
                                                 const double* volumes, const double* phi,
                                                 const double* g, double* g_face, double* g_cell,
                                                 double* g_sum, void* stream) {
  int rc = check_layout(L);
  if (rc) return rc;
  const int nint = L->n_faces;
  GBF_REQUIRE(n_faces_total >= nint, "explicit_laplacian_grad_d: n_faces_total < n_internal");
  cudaStream_t s = as_stream(stream);
  if (n_faces_total > 0) {
    GBF_REQUIRE(owner_all && face_areas && delta && volumes && phi && g && g_face &&
                    (nint == 0 || L->neighbour),
                "explicit_laplacian_grad_d: NULL pointer");
    explicit_lap_grad_d_kernel<<<(n_faces_total + kBlock - 1) / kBlock, kBlock, 0, s>>>(
        nint, n_faces_total, owner_all, L->neighbour, face_areas, delta, volumes, phi, g, g_face);
    GBF_CHECK_LAUNCH();
  }
  const bool has_bnd = n_faces_total > nint;
  if (g_cell && L->n_cells > 0) {
    GBF_REQUIRE(!has_bnd || (bnd_ptr && bnd_face),
                "explicit_laplacian_grad_d: NULL boundary lists");
    face_grad_to_cells_kernel<<<(L->n_cells + kBlock - 1) / kBlock, kBlock, 0, s>>>(
        *L, bnd_ptr, bnd_face, g_face, has_bnd ? 1 : 0, g_cell);
    GBF_CHECK_LAUNCH();
  }
  if (g_sum) {
    fixed_order_sum_kernel<<<1, kSumBlock, 0, s>>>(n_faces_total, g_face, g_sum);
    GBF_CHECK_LAUNCH();
  }
  return GBF_OK;
}

// ---------------------------------------------------------------------------
// Pressure equation (solvers/pressure_equation.py:49-148):
//   face_coeff = ((1/A_p)_f |S_f|) delta_f with (1/A_p)_f linearly
//   interpolated from 1/max(|A_p|, 1e-30) with the given face weights;
//   lower = -fc/V_P, upper = -fc/V_N; diag = (0 + sum_own fc/V_P) + sum_nei fc/V_N
//   (no boundary term); source = (((0 + sum_own -phi_f) + sum_nei phi_f)
//   [+ sum_bnd -phi_b]) / V.
// ---------------------------------------------------------------------------
namespace gbf {
__global__ void __launch_bounds__(kBlock)
    pressure_source_kernel(gbf_layout L, const int32_t* __restrict__ bnd_ptr,
                           const int32_t* __restrict__ bnd_face, const double* __restrict__ phi,
                           const double* __restrict__ V, int has_bnd, double* __restrict__ src) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= L.n_cells) return;
  double so = 0.0, sn = 0.0;
  if (L.n_faces > 0) {
    const CellSlots cs = cell_slots(L, c);
    for (int k = 0; k < cs.wo; ++k) {
      const int f = __ldg(L.slot_face + cs.base + 32 * k);
      if (f >= 0) so = __dadd_rn(so, -__ldg(phi + f));
    }
    for (int k = 0; k < cs.wn; ++k) {
      const int f = __ldg(L.slot_face + cs.base + 32 * (cs.wo + k));
      if (f >= 0) sn = __dadd_rn(sn, __ldg(phi + f));
    }
  }
  double y = __dadd_rn(0.0, so);
  y = __dadd_rn(y, sn);
  if (has_bnd) {
    double sb = 0.0;
    for (int k = __ldg(bnd_ptr + c); k < __ldg(bnd_ptr + c + 1); ++k)
      sb = __dadd_rn(sb, -__ldg(phi + __ldg(bnd_face + k)));
    y = __dadd_rn(y, sb);
  }
  src[c] = __ddiv_rn(y, __ldg(V + c));
}
}  // namespace gbf

extern "C" int gbf_pressure_assemble_f64(const gbf_layout* L, int32_t n_faces_total,
                                         const int32_t* bnd_ptr, const int32_t* bnd_face,
                                         const double* face_areas, const double* delta,
                                         const double* face_weights, const double* A_p,
                                         const double* volumes, const double* phiHbyA,
                                         double* lower, double* upper, double* diag,
                                         double* source, void* stream) {
  int rc = check_layout(L);
  if (rc) return rc;
  const int n = L->n_cells, nint = L->n_faces;
  GBF_REQUIRE(n_faces_total >= nint, "pressure_assemble: n_faces_total < n_internal_faces");
  if (n == 0) return GBF_OK;
  GBF_REQUIRE(A_p && volumes && diag && source && (n_faces_total == 0 || phiHbyA),
              "pressure_assemble: NULL pointer");
  const bool has_bnd = n_faces_total > nint;
  GBF_REQUIRE(!has_bnd || (bnd_ptr && bnd_face), "pressure_assemble: NULL boundary lists");
  const DiffSpec D = make_spec(3, 0.0, nullptr, A_p, face_weights);
  cudaStream_t s = as_stream(stream);
  if (nint > 0) {
    GBF_REQUIRE(lower && upper && face_areas && delta && face_weights && L->owner &&
                    L->neighbour,
                "pressure_assemble: NULL pointer");
    lap_face_kernel<<<(nint + kBlock - 1) / kBlock, kBlock, 0, s>>>(
        nint, L->owner, L->neighbour, face_areas, delta, D, volumes, lower, upper);
    GBF_CHECK_LAUNCH();
  }
  lap_diag_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, s>>>(
      *L, lower, upper, nullptr, nullptr, face_areas, delta, D, volumes, 0, diag);
  GBF_CHECK_LAUNCH();
  pressure_source_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, s>>>(
      *L, bnd_ptr, bnd_face, phiHbyA, volumes, has_bnd ? 1 : 0, source);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}
