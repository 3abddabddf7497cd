// Cell-centred LDU gather (Amul) used by every kernel that needs A*x.
//
// One thread per cell, one warp per 32-cell slice.  Owner-side and
// neighbour-side slot sums are formed separately, each starting from 0.0 in
// ascending face order, and combined as (diag*x + S_first) + S_second --
// the association and rounding of the reference's
//   y = diag*x; y = y + scatter_add(...); y = y + scatter_add(...)
// (core/ldu_matrix.py:200-215, core/backend.py:58-64).
#pragma once

#include "common.cuh"

namespace gbf {

// Load of the multiplied vector: through the read-only path, or (COH) from
// L2 only -- for persistent kernels in which other blocks rewrite the vector
// between phases, so that no stale L1 line is read.
template <bool COH, typename T>
__device__ __forceinline__ T ldx(const T* p) {
  if constexpr (COH)
    return __ldcg(p);
  else
    return __ldg(p);
}

// Sum over `cnt` slots starting at slot k0 of cell c (slot index i0 =
// base + 32*k0, compressed entry e0 + k0) of coef[slot] * x[col[slot]],
// skipping padding (col < 0).  Products are rounded in T, sums in A.
template <typename T, typename A, bool COH = false>
__device__ __forceinline__ A slot_sum(const gbf_layout& L, const T* __restrict__ coef,
                                      const T* __restrict__ x, int c, int i0, int e0, int cnt) {
  A s = (A)0;
  if (cnt <= 4) {
    int col[4];
    T a[4], xv[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) col[k] = (k < cnt) ? slot_column(L, e0 + k, i0 + 32 * k, c) : -1;
    // coefficients do not wait for the columns: every slot k < cnt exists
    // (holes hold 0), so the loads are issued together with the columns'
#pragma unroll
    for (int k = 0; k < 4; ++k) a[k] = (k < cnt) ? __ldg(coef + i0 + 32 * k) : (T)0;
#pragma unroll
    for (int k = 0; k < 4; ++k) xv[k] = (col[k] >= 0) ? ldx<COH>(x + col[k]) : (T)0;
    if (col[0] >= 0) s = first_term((A)mul_rn(a[0], xv[0]));
#pragma unroll
    for (int k = 1; k < 4; ++k)
      if (col[k] >= 0) s = add_rn(s, (A)mul_rn(a[k], xv[k]));
  } else {
    const int col0 = slot_column(L, e0, i0, c);
    if (col0 >= 0) s = first_term((A)mul_rn(__ldg(coef + i0), ldx<COH>(x + col0)));
#pragma unroll 4
    for (int k = 1; k < cnt; ++k) {
      const int col = slot_column(L, e0 + k, i0 + 32 * k, c);
      if (col >= 0) s = add_rn(s, (A)mul_rn(__ldg(coef + i0 + 32 * k), ldx<COH>(x + col)));
    }
  }
  return s;
}

// (A x)[c] with x[c] already loaded as xc.
template <typename T, typename A, bool NEI_FIRST, bool COH = false>
__device__ __forceinline__ A cell_amul(const gbf_layout& L, const T* __restrict__ coef,
                                       const T* __restrict__ diag, const T* __restrict__ x,
                                       int c, T xc) {
  A y = (A)mul_rn(__ldg(diag + c), xc);
  if (L.n_faces > 0) {
    const CellSlots cs = cell_slots(L, c);
    A so = (A)0, sn = (A)0;
    if (cs.wo <= 4 && cs.wn <= 4) {
      // both sides in one predicated block: every column, coefficient and x
      // load of the cell is in flight at once
      int col[8];
      T a[8], xv[8];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        col[k] = (k < cs.wo) ? slot_column(L, cs.e0 + k, cs.base + 32 * k, c) : -1;
        col[4 + k] = (k < cs.wn) ? slot_column(L, cs.e0 + cs.wo + k,
                                               cs.base + 32 * (cs.wo + k), c) : -1;
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        a[k] = (k < cs.wo) ? __ldg(coef + cs.base + 32 * k) : (T)0;
        a[4 + k] = (k < cs.wn) ? __ldg(coef + cs.base + 32 * (cs.wo + k)) : (T)0;
      }
#pragma unroll
      for (int k = 0; k < 8; ++k) xv[k] = (col[k] >= 0) ? ldx<COH>(x + col[k]) : (T)0;
      if (col[0] >= 0) so = first_term((A)mul_rn(a[0], xv[0]));
#pragma unroll
      for (int k = 1; k < 4; ++k)
        if (col[k] >= 0) so = add_rn(so, (A)mul_rn(a[k], xv[k]));
      if (col[4] >= 0) sn = first_term((A)mul_rn(a[4], xv[4]));
#pragma unroll
      for (int k = 5; k < 8; ++k)
        if (col[k] >= 0) sn = add_rn(sn, (A)mul_rn(a[k], xv[k]));
    } else {
      so = slot_sum<T, A, COH>(L, coef, x, c, cs.base, cs.e0, cs.wo);
      sn = slot_sum<T, A, COH>(L, coef, x, c, cs.base + 32 * cs.wo, cs.e0 + cs.wo, cs.wn);
    }
    if (NEI_FIRST) {
      y = add_rn(y, sn);
      y = add_rn(y, so);
    } else {
      y = add_rn(y, so);
      y = add_rn(y, sn);
    }
  }
  return y;
}

// ---------------------------------------------------------------------------
// Fixed-width gather for layouts whose slices all have WO owner-side and WN
// neighbour-side slots, every slot offset-uniform (all_uniform): the slot
// addresses are arithmetic, the slice's {delta, mask} entries come in W/2
// 128-bit loads, and no slot needs a width predicate or a slot_col
// fallback.  Same products and summation order as cell_amul.
// ---------------------------------------------------------------------------
template <typename T, typename A, bool NEI_FIRST, int WO, int WN, bool COH = false>
__device__ __forceinline__ A cell_amul_fixed(const gbf_layout& L, const T* __restrict__ coef,
                                             const T* __restrict__ diag,
                                             const T* __restrict__ x, int c, T xc) {
  constexpr int W = WO + WN;
  static_assert(W % 2 == 0, "fixed-width gather loads entry pairs");
  const int s = c >> 5, lane = c & 31;
  const int base = 32 * W * s + lane;
  const int4* __restrict__ dm4 = reinterpret_cast<const int4*>(L.slot_dm) + (W / 2) * s;
  int d[W];
  unsigned m[W];
#pragma unroll
  for (int q = 0; q < W / 2; ++q) {
    const int4 v = __ldg(dm4 + q);
    d[2 * q] = v.x;
    m[2 * q] = (unsigned)v.y;
    d[2 * q + 1] = v.z;
    m[2 * q + 1] = (unsigned)v.w;
  }
  T a[W], xv[W];
  bool on[W];
  if constexpr (sizeof(T) == 4) {
    // FP32 coefficients are a read-once stream per pass: L2 evict-first
    const unsigned long long ef = l2_evict_first();
#pragma unroll
    for (int k = 0; k < W; ++k) a[k] = ld_nc_hint(coef + base + 32 * k, ef);
  } else {
#pragma unroll
    for (int k = 0; k < W; ++k) a[k] = __ldg(coef + base + 32 * k);
  }
#pragma unroll
  for (int k = 0; k < W; ++k) {
    on[k] = (m[k] >> lane) & 1u;
    xv[k] = on[k] ? ldx<COH>(x + c + d[k]) : (T)0;
  }
  A so = (A)0, sn = (A)0;
  if (WO > 0 && on[0]) so = first_term((A)mul_rn(a[0], xv[0]));
#pragma unroll
  for (int k = 1; k < WO; ++k)
    if (on[k]) so = add_rn(so, (A)mul_rn(a[k], xv[k]));
  if (WN > 0 && on[WO]) sn = first_term((A)mul_rn(a[WO], xv[WO]));
#pragma unroll
  for (int k = WO + 1; k < W; ++k)
    if (on[k]) sn = add_rn(sn, (A)mul_rn(a[k], xv[k]));
  A y = (A)mul_rn(__ldg(diag + c), xc);
  if (NEI_FIRST) {
    y = add_rn(y, sn);
    y = add_rn(y, so);
  } else {
    y = add_rn(y, so);
    y = add_rn(y, sn);
  }
  return y;
}

// ---------------------------------------------------------------------------
// Symmetric hex 3+3 gather: the owner-side coefficients come from the
// owner-side half `own` (32*3 floats per slice), the neighbour-side ones from
// the owner cells' slots, whose owner-side slot j is L.slot_mirror's entry.
// Same products and summation order as cell_amul_fixed<float, A, false, 3, 3>
// on the full packing of the same (symmetric) matrix.
// ---------------------------------------------------------------------------
template <typename A>
__device__ __forceinline__ A cell_amul_sym33(const gbf_layout& L, const float* __restrict__ own,
                                             const float* __restrict__ diag,
                                             const float* __restrict__ x, int c, float xc) {
  const int s = c >> 5, lane = c & 31;
  const int4* __restrict__ dm4 = reinterpret_cast<const int4*>(L.slot_dm) + 3 * s;
  int d[6];
  unsigned m[6];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const int4 v = __ldg(dm4 + q);
    d[2 * q] = v.x;
    m[2 * q] = (unsigned)v.y;
    d[2 * q + 1] = v.z;
    m[2 * q + 1] = (unsigned)v.w;
  }
  float a[6], xv[6];
  bool on[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) on[k] = (m[k] >> lane) & 1u;
#pragma unroll
  for (int k = 0; k < 3; ++k) a[k] = __ldg(own + 96 * s + 32 * k + lane);
#pragma unroll
  for (int k = 3; k < 6; ++k) {
    const int c2 = c + d[k];
    const int j = __ldg(L.slot_mirror + 6 * s + k);
    a[k] = on[k] ? __ldg(own + 96 * (c2 >> 5) + 32 * j + (c2 & 31)) : 0.0f;
  }
#pragma unroll
  for (int k = 0; k < 6; ++k) xv[k] = on[k] ? __ldg(x + c + d[k]) : 0.0f;
  A so = (A)0, sn = (A)0;
  if (on[0]) so = first_term((A)__fmul_rn(a[0], xv[0]));
#pragma unroll
  for (int k = 1; k < 3; ++k)
    if (on[k]) so = add_rn(so, (A)__fmul_rn(a[k], xv[k]));
  if (on[3]) sn = first_term((A)__fmul_rn(a[3], xv[3]));
#pragma unroll
  for (int k = 4; k < 6; ++k)
    if (on[k]) sn = add_rn(sn, (A)__fmul_rn(a[k], xv[k]));
  A y = (A)__fmul_rn(__ldg(diag + c), xc);
  y = add_rn(y, so);
  return add_rn(y, sn);
}

// Layout kinds with a fixed-width kernel instantiation.
// kLayoutHex33Sym: hex 3+3 with the coefficients of a symmetric matrix
// stored as the owner-side half (FP32 only; chosen by the caller).
enum { kLayoutGeneric = 0, kLayoutHex33 = 33, kLayoutHex33Sym = 34 };

// The fixed-width gather reads slot_dm as int4, so it needs a 16-byte
// aligned table.
inline int layout_kind(const gbf_layout& L) {
  if (L.n_faces > 0 && L.all_uniform && L.slot_dm && L.uniform_wo == 3 && L.uniform_wn == 3 &&
      (reinterpret_cast<uintptr_t>(L.slot_dm) & 15u) == 0)
    return kLayoutHex33;
  return kLayoutGeneric;
}

// Runs the statement list with the compile-time constant KIND set to the
// layout's kind, so a kernel templated on it is launched in its fixed-width
// form where one exists.
#define GBF_LAYOUT_DISPATCH(layout, KIND, ...)      \
  do {                                              \
    if (::gbf::layout_kind(layout) == ::gbf::kLayoutHex33) { \
      constexpr int KIND = ::gbf::kLayoutHex33;     \
      __VA_ARGS__;                                  \
    } else {                                        \
      constexpr int KIND = ::gbf::kLayoutGeneric;   \
      __VA_ARGS__;                                  \
    }                                               \
  } while (0)

// One side of (A x)[c]: the owner-side sum (side 0) or the neighbour-side
// sum (side 1), each from 0.0 in ascending face order with the products and
// additions of cell_amul / cell_amul_fixed -- the two halves that a pair of
// threads computes when a cell has two threads.  The caller forms
// (diag * x + owner sum) + neighbour sum, the order of the one-thread forms.
template <int KIND, typename T, typename A, bool COH = false>
__device__ __forceinline__ A cell_side_sum(const gbf_layout& L, const T* __restrict__ coef,
                                           const T* __restrict__ x, int c, int side) {
  if constexpr (KIND == kLayoutHex33) {
    const int s = c >> 5, lane = c & 31;
    const int base = 32 * 6 * s + 32 * 3 * side + lane;
    const int2* __restrict__ dm = reinterpret_cast<const int2*>(L.slot_dm) + 6 * s + 3 * side;
    int d[3];
    bool on[3];
    T a[3], xv[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int2 e = __ldg(dm + k);
      d[k] = e.x;
      on[k] = ((unsigned)e.y >> lane) & 1u;
    }
    if constexpr (sizeof(T) == 4) {
      const unsigned long long ef = l2_evict_first();
#pragma unroll
      for (int k = 0; k < 3; ++k) a[k] = ld_nc_hint(coef + base + 32 * k, ef);
    } else {
#pragma unroll
      for (int k = 0; k < 3; ++k) a[k] = __ldg(coef + base + 32 * k);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) xv[k] = on[k] ? ldx<COH>(x + c + d[k]) : (T)0;
    A sum = (A)0;
    if (on[0]) sum = first_term((A)mul_rn(a[0], xv[0]));
#pragma unroll
    for (int k = 1; k < 3; ++k)
      if (on[k]) sum = add_rn(sum, (A)mul_rn(a[k], xv[k]));
    return sum;
  } else {
    if (L.n_faces == 0) return (A)0;
    const CellSlots cs = cell_slots(L, c);
    return side == 0 ? slot_sum<T, A, COH>(L, coef, x, c, cs.base, cs.e0, cs.wo)
                     : slot_sum<T, A, COH>(L, coef, x, c, cs.base + 32 * cs.wo, cs.e0 + cs.wo,
                                           cs.wn);
  }
}

// True when a symmetric matrix on this layout may be stored as its
// owner-side half (hex 3+3 kind with a mirror table).
inline bool layout_sym_ok(const gbf_layout& L) {
  return layout_kind(L) == kLayoutHex33 && L.slot_mirror != nullptr;
}

template <int KIND, typename T, typename A, bool NEI_FIRST, bool COH = false>
__device__ __forceinline__ A cell_amul_k(const gbf_layout& L, const T* __restrict__ coef,
                                         const T* __restrict__ diag, const T* __restrict__ x,
                                         int c, T xc) {
  if constexpr (KIND == kLayoutHex33Sym) {
    static_assert(!NEI_FIRST, "a symmetric matrix is its own transpose");
    return cell_amul_sym33<A>(L, coef, diag, x, c, xc);
  } else if constexpr (KIND == kLayoutHex33) {
    return cell_amul_fixed<T, A, NEI_FIRST, 3, 3, COH>(L, coef, diag, x, c, xc);
  } else {
    return cell_amul<T, A, NEI_FIRST, COH>(L, coef, diag, x, c, xc);
  }
}

}  // namespace gbf
