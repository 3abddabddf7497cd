// Finite-volume mesh geometry on the GPU: face centres and area vectors,
// cell volumes and centres, interpolation weights and delta coefficients of
// a polyhedral mesh given as points + face-vertex lists + owner/neighbour.
//
// The formulas and their order of operations follow the reference's
// mesh/mesh_geometry.py:
//   face centre      = mean of the face's vertices            (:35-63)
//   face area vector = 1/2 sum_j v_j x v_{j+1}                (:66-108)
//   cell volume      = sum |tet(ref, fc, v_j, v_{j+1})| over the cell's
//                      faces, vertex order reversed on its neighbour-side
//                      faces; ref = mean of the cell's distinct vertices;
//                      centre = volume-weighted tet centroids  (:139-254)
//   weight           = |d_N| / (|d_P| + |d_N|), 1 on boundary   (:262-327)
//   delta            = 1 / |(C_N - C_P) . n_hat|, 0 on boundary (:330-395)
// with one thread per face or per cell instead of the reference's Python
// loops.  Every product and sum is an explicitly rounded intrinsic: face
// centres, area vectors are bitwise the reference's; cell volumes and
// centres (whose reference sums run over a Python set of vertex ids and a
// library dot product) agree to rounding.
#include <math.h>

#include "common.cuh"

namespace gbf {

constexpr int kMaxCellPoints = 64;

struct V3 {
  double x, y, z;
};

__device__ __forceinline__ V3 ld3(const double* __restrict__ p, int i) {
  return V3{__ldg(p + 3 * (size_t)i), __ldg(p + 3 * (size_t)i + 1), __ldg(p + 3 * (size_t)i + 2)};
}
__device__ __forceinline__ void st3(double* __restrict__ p, int i, V3 v) {
  p[3 * (size_t)i] = v.x;
  p[3 * (size_t)i + 1] = v.y;
  p[3 * (size_t)i + 2] = v.z;
}
__device__ __forceinline__ V3 add3(V3 a, V3 b) {
  return V3{__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y), __dadd_rn(a.z, b.z)};
}
__device__ __forceinline__ V3 sub3(V3 a, V3 b) {
  return V3{__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z)};
}
__device__ __forceinline__ V3 scale3(V3 a, double s) {
  return V3{__dmul_rn(a.x, s), __dmul_rn(a.y, s), __dmul_rn(a.z, s)};
}
__device__ __forceinline__ V3 div3(V3 a, double s) {
  return V3{__ddiv_rn(a.x, s), __ddiv_rn(a.y, s), __ddiv_rn(a.z, s)};
}
// a x b with each component rounded as fma(a_i, b_j, -(a_j b_i)), the
// rounding of ATen's CPU cross product (torch.linalg.cross).
__device__ __forceinline__ V3 cross3(V3 a, V3 b) {
  return V3{__fma_rn(a.y, b.z, -__dmul_rn(a.z, b.y)),
            __fma_rn(a.z, b.x, -__dmul_rn(a.x, b.z)),
            __fma_rn(a.x, b.y, -__dmul_rn(a.y, b.x))};
}
__device__ __forceinline__ double dot3(V3 a, V3 b) {
  return __dadd_rn(__dadd_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)), __dmul_rn(a.z, b.z));
}
// |v| accumulated as sqrt(fma(z, z, fma(y, y, x*x))), the rounding of
// ATen's CPU p=2 norm over a length-3 row.
__device__ __forceinline__ double norm3(V3 v) {
  return __dsqrt_rn(__fma_rn(v.z, v.z, __fma_rn(v.y, v.y, __dmul_rn(v.x, v.x))));
}

__global__ void __launch_bounds__(kBlock)
    face_geometry_kernel(int n_faces, const int32_t* __restrict__ face_ptr,
                         const int32_t* __restrict__ face_pts, const double* __restrict__ points,
                         double* __restrict__ centres, double* __restrict__ areas) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= n_faces) return;
  const int b = __ldg(face_ptr + f), nv = __ldg(face_ptr + f + 1) - b;
  V3 s{0.0, 0.0, 0.0};
  for (int j = 0; j < nv; ++j) s = add3(s, ld3(points, __ldg(face_pts + b + j)));
  st3(centres, f, div3(s, (double)nv));  // 0/0 = NaN for a face without vertices
  V3 a{0.0, 0.0, 0.0};
  if (nv >= 3) {
    V3 v0 = ld3(points, __ldg(face_pts + b));
    V3 vj = v0;
    for (int j = 0; j < nv; ++j) {
      const V3 vn = (j + 1 < nv) ? ld3(points, __ldg(face_pts + b + j + 1)) : v0;
      a = add3(a, cross3(vj, vn));
      vj = vn;
    }
    a = scale3(a, 0.5);
  }
  st3(areas, f, a);
}

// Vertex k of face f as seen from a cell: reversed order on the cell's
// neighbour-side faces (so that the face normal points out of the cell).
__device__ __forceinline__ int face_vertex(const int32_t* __restrict__ face_pts, int b, int nv,
                                           bool flip, int k) {
  return __ldg(face_pts + b + (flip ? nv - 1 - k : k));
}

__global__ void __launch_bounds__(128)
    cell_geometry_kernel(int n_cells, const int32_t* __restrict__ cell_ptr,
                         const int32_t* __restrict__ cell_faces,
                         const int32_t* __restrict__ face_ptr,
                         const int32_t* __restrict__ face_pts, const double* __restrict__ points,
                         const double* __restrict__ face_centres, double* __restrict__ volumes,
                         double* __restrict__ centres, int32_t* __restrict__ status) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_cells) return;
  const int q0 = __ldg(cell_ptr + c), q1 = __ldg(cell_ptr + c + 1);
  if (q0 == q1) {  // a cell without faces keeps zero volume and centre
    volumes[c] = 0.0;
    st3(centres, c, V3{0.0, 0.0, 0.0});
    return;
  }
  // distinct vertices of the cell, ascending
  int pts[kMaxCellPoints];
  int np = 0;
  for (int q = q0; q < q1; ++q) {
    const int e = __ldg(cell_faces + q);
    const int f = e >= 0 ? e : ~e;
    const int b = __ldg(face_ptr + f), nv = __ldg(face_ptr + f + 1) - b;
    for (int k = 0; k < nv; ++k) {
      const int p = __ldg(face_pts + b + k);
      int i = 0;
      while (i < np && pts[i] < p) ++i;
      if (i < np && pts[i] == p) continue;
      if (np == kMaxCellPoints) {
        atomicExch(status, 1);
        volumes[c] = NAN;
        st3(centres, c, V3{NAN, NAN, NAN});
        return;
      }
      for (int j = np; j > i; --j) pts[j] = pts[j - 1];
      pts[i] = p;
      ++np;
    }
  }
  V3 ref{0.0, 0.0, 0.0};
  for (int i = 0; i < np; ++i) ref = add3(ref, ld3(points, pts[i]));
  ref = div3(ref, (double)np);

  double total = 0.0;
  V3 wc{0.0, 0.0, 0.0};
  for (int q = q0; q < q1; ++q) {
    const int e = __ldg(cell_faces + q);
    const bool flip = e < 0;
    const int f = flip ? ~e : e;
    const int b = __ldg(face_ptr + f), nv = __ldg(face_ptr + f + 1) - b;
    if (nv < 3) continue;
    const V3 fc = ld3(face_centres, f);
    const V3 bf = sub3(fc, ref);
    const V3 w0 = ld3(points, face_vertex(face_pts, b, nv, flip, 0));
    V3 wj = w0;
    for (int j = 0; j < nv; ++j) {
      const V3 wn = (j + 1 < nv) ? ld3(points, face_vertex(face_pts, b, nv, flip, j + 1)) : w0;
      const double vol = __ddiv_rn(dot3(bf, cross3(sub3(wj, ref), sub3(wn, ref))), 6.0);
      if (fabs(vol) >= 1e-30) {
        const double av = fabs(vol);
        const V3 cen = div3(add3(add3(add3(ref, fc), wj), wn), 4.0);
        total = __dadd_rn(total, av);
        wc = add3(wc, scale3(cen, av));
      }
      wj = wn;
    }
  }
  if (fabs(total) > 1e-30) {
    volumes[c] = fabs(total);
    st3(centres, c, div3(wc, total));
  } else {  // degenerate cell: mean of its face centres
    V3 s{0.0, 0.0, 0.0};
    for (int q = q0; q < q1; ++q) {
      const int e = __ldg(cell_faces + q);
      s = add3(s, ld3(face_centres, e >= 0 ? e : ~e));
    }
    volumes[c] = 0.0;
    st3(centres, c, div3(s, (double)(q1 - q0)));
  }
}

__global__ void __launch_bounds__(kBlock)
    face_interp_kernel(int n_faces, int n_internal, const int32_t* __restrict__ owner,
                       const int32_t* __restrict__ neighbour,
                       const double* __restrict__ cell_centres,
                       const double* __restrict__ face_centres,
                       const double* __restrict__ face_areas, double* __restrict__ weights,
                       double* __restrict__ delta) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= n_faces) return;
  if (f >= n_internal) {
    weights[f] = 1.0;
    delta[f] = 0.0;
    return;
  }
  const V3 cp = ld3(cell_centres, __ldg(owner + f));
  const V3 cn = ld3(cell_centres, __ldg(neighbour + f));
  const V3 fc = ld3(face_centres, f);
  const double dP = norm3(sub3(fc, cp)), dN = norm3(sub3(fc, cn));
  const double den = __dadd_rn(dP, dN);
  weights[f] = __ddiv_rn(dN, den > 1e-30 ? den : 1.0);
  const V3 A = ld3(face_areas, f);
  const double am = norm3(A);
  const V3 nh = div3(A, am > 1e-30 ? am : 1.0);
  const double ddn = fabs(dot3(sub3(cn, cp), nh));
  delta[f] = __ddiv_rn(1.0, ddn > 1e-30 ? ddn : 1.0);
}

}  // namespace gbf

using namespace gbf;

extern "C" int gbf_face_geometry_f64(int32_t n_faces, const int32_t* face_ptr,
                                     const int32_t* face_pts, const double* points,
                                     double* face_centres, double* face_areas, void* stream) {
  GBF_REQUIRE(n_faces >= 0, "face_geometry: negative n_faces");
  if (n_faces == 0) return GBF_OK;
  GBF_REQUIRE(face_ptr && face_pts && points && face_centres && face_areas,
              "face_geometry: NULL pointer");
  face_geometry_kernel<<<(n_faces + kBlock - 1) / kBlock, kBlock, 0, as_stream(stream)>>>(
      n_faces, face_ptr, face_pts, points, face_centres, face_areas);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_cell_geometry_f64(int32_t n_cells, const int32_t* cell_ptr,
                                     const int32_t* cell_faces, const int32_t* face_ptr,
                                     const int32_t* face_pts, const double* points,
                                     const double* face_centres, double* volumes,
                                     double* cell_centres, int32_t* status, void* stream) {
  GBF_REQUIRE(n_cells >= 0, "cell_geometry: negative n_cells");
  GBF_REQUIRE(status, "cell_geometry: NULL status");
  cudaStream_t s = as_stream(stream);
  GBF_CHECK_CUDA(cudaMemsetAsync(status, 0, sizeof(int32_t), s));
  if (n_cells == 0) return GBF_OK;
  GBF_REQUIRE(cell_ptr && cell_faces && face_ptr && face_pts && points && face_centres &&
                  volumes && cell_centres,
              "cell_geometry: NULL pointer");
  cell_geometry_kernel<<<(n_cells + 127) / 128, 128, 0, s>>>(
      n_cells, cell_ptr, cell_faces, face_ptr, face_pts, points, face_centres, volumes,
      cell_centres, status);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_face_interp_f64(int32_t n_faces, int32_t n_internal, const int32_t* owner,
                                   const int32_t* neighbour, const double* cell_centres,
                                   const double* face_centres, const double* face_areas,
                                   double* weights, double* delta, void* stream) {
  GBF_REQUIRE(n_faces >= 0 && n_internal >= 0 && n_internal <= n_faces,
              "face_interp: bad face counts");
  if (n_faces == 0) return GBF_OK;
  GBF_REQUIRE(weights && delta && (n_internal == 0 || (owner && neighbour && cell_centres &&
                                                       face_centres && face_areas)),
              "face_interp: NULL pointer");
  face_interp_kernel<<<(n_faces + kBlock - 1) / kBlock, kBlock, 0, as_stream(stream)>>>(
      n_faces, n_internal, owner, neighbour, cell_centres, face_centres, face_areas, weights,
      delta);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}
