// Coefficient packing and the stand-alone Amul entry points.
#include <type_traits>

#include "bulk.cuh"

namespace gbf {

// Set by a staged Amul block whose bounded wait ran out (gbf_stream_fault).
static __device__ unsigned int g_stream_fault;

// One thread per lane of every slice (padding lanes of the last slice
// included, so that all slots are written).
template <typename S, typename T>
__global__ void __launch_bounds__(kBlock)
    pack_kernel(gbf_layout L, const S* __restrict__ own_src, const S* __restrict__ nei_src,
                T* __restrict__ coef) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= L.n_slices * 32) return;
  const CellSlots cs = cell_slots(L, c);
  for (int k = 0; k < cs.wo; ++k) {
    const int i = cs.base + 32 * k;
    const int f = L.slot_face[i];
    coef[i] = (f >= 0) ? (T)own_src[f] : (T)0;
  }
  for (int k = 0; k < cs.wn; ++k) {
    const int i = cs.base + 32 * (cs.wo + k);
    const int f = L.slot_face[i];
    coef[i] = (f >= 0) ? (T)nei_src[f] : (T)0;
  }
}

template <int KIND, typename T, typename A, bool NEI_FIRST>
__global__ void __launch_bounds__(kBlock)
    amul_kernel(gbf_layout L, const T* __restrict__ coef, const T* __restrict__ diag,
                const T* __restrict__ x, A* __restrict__ y) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < L.n_cells; c += gridDim.x * blockDim.x)
    y[c] = cell_amul_k<KIND, T, A, NEI_FIRST>(L, coef, diag, x, c, __ldg(x + c));
}

// FP32 Amul of a hex 3+3 layout with the coefficient / x / diagonal stream
// staged through shared memory by bulk asynchronous copies; the cells of the
// last, partial tile are computed from global memory by one block.
// SYM: coef is the owner-side half of a symmetric matrix (pack_sym_kernel).
template <typename A, bool NEI_FIRST, bool SYM>
__global__ void __launch_bounds__(kTileCells, kStreamBlocksPerSM)
    amul_stream_kernel(gbf_layout L, const float* __restrict__ coef,
                       const float* __restrict__ diag, const float* __restrict__ x,
                       A* __restrict__ y, int n_tiles) {
  __shared__ HexRing<SYM> ring;
  const bool ok = hex_stream_tiles<A, NEI_FIRST, SYM>(ring, n_tiles, coef, x, diag, L.slot_dm,
                                                      L.slot_mirror,
                                                      [&](int c, A v, float) { y[c] = v; });
  if (blockIdx.x == n_tiles % gridDim.x) {
    const int c = n_tiles * kTileCells + threadIdx.x;
    if (c < L.n_cells) {
      if constexpr (SYM)
        y[c] = cell_amul_sym33<A>(L, coef, diag, x, c, __ldg(x + c));
      else
        y[c] = cell_amul_fixed<float, A, NEI_FIRST, 3, 3>(L, coef, diag, x, c, __ldg(x + c));
    }
  }
  if (!ok && threadIdx.x == 0) atomicExch(&g_stream_fault, 1u);
}

template <typename A, bool NEI_FIRST, bool SYM = false>
static void launch_amul_stream(const gbf_layout* L, const float* coef, const float* diag,
                               const float* x, A* y, cudaStream_t s) {
  const int n_tiles = L->n_cells / kTileCells;
  const int grid = wave_grid(amul_stream_kernel<A, NEI_FIRST, SYM>, kTileCells,
                             (long long)(n_tiles > 0 ? n_tiles : 1) * kTileCells);
  amul_stream_kernel<A, NEI_FIRST, SYM>
      <<<grid, kTileCells, 0, s>>>(*L, coef, diag, x, y, n_tiles);
}

// Owner-side half of a symmetric matrix: one thread per lane of every slice;
// lanes whose face has lower != upper (bitwise) set *differs.
__global__ void __launch_bounds__(kBlock)
    pack_sym_kernel(gbf_layout L, const double* __restrict__ lower,
                    const double* __restrict__ upper, float* __restrict__ own,
                    int32_t* __restrict__ differs) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= L.n_slices * 32) return;
  const CellSlots cs = cell_slots(L, c);
  const int s = c >> 5, lane = c & 31;
  bool diff = false;
  for (int k = 0; k < cs.wo; ++k) {
    const int f = L.slot_face[cs.base + 32 * k];
    float v = 0.0f;
    if (f >= 0) {
      const double lo = lower[f];
      diff |= __double_as_longlong(lo) != __double_as_longlong(upper[f]);
      v = (float)lo;
    }
    own[32 * cs.wo * s + 32 * k + lane] = v;
  }
  if (diff) atomicOr(differs, 1);
}

__global__ void __launch_bounds__(kBlock)
    amul_sym_kernel(gbf_layout L, const float* __restrict__ own, const float* __restrict__ diag,
                    const float* __restrict__ x, float* __restrict__ y) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < L.n_cells; c += gridDim.x * blockDim.x)
    y[c] = cell_amul_sym33<float>(L, own, diag, x, c, __ldg(x + c));
}

template <int KIND, typename T, typename A, bool NEI_FIRST>
static void launch_amul(const gbf_layout* L, const T* coef, const T* diag, const T* x, A* y,
                        cudaStream_t s) {
  const int grid = wave_grid(amul_kernel<KIND, T, A, NEI_FIRST>, kBlock, L->n_cells);
  amul_kernel<KIND, T, A, NEI_FIRST><<<grid, kBlock, 0, s>>>(*L, coef, diag, x, y);
}

int check_layout(const gbf_layout* L) {
  GBF_REQUIRE(L != nullptr, "layout is NULL");
  GBF_REQUIRE(L->n_cells >= 0 && L->n_faces >= 0, "negative layout size");
  // The kernels index cells, faces and slots with 32-bit integers, and a
  // grid-stride loop may step up to kMaxGrid * 1024 past the last item.
  constexpr int64_t kIndexLimit = (int64_t)INT_MAX - (int64_t)kMaxGrid * 1024;
  GBF_REQUIRE(L->n_cells <= kIndexLimit && L->n_faces <= kIndexLimit && L->n_slots >= 0 &&
                  L->n_slots <= kIndexLimit,
              "layout too large for 32-bit indices: %d cells, %d faces, %lld slots (limit %lld)",
              L->n_cells, L->n_faces, (long long)L->n_slots, (long long)kIndexLimit);
  GBF_REQUIRE(L->n_slices == (L->n_cells + 31) / 32, "layout n_slices does not match n_cells");
  if (L->n_cells > 0)
    GBF_REQUIRE(L->slice_off && L->slice_w && L->slot_col && L->slot_face,
                "layout arrays are NULL");
  return GBF_OK;
}

template <typename S, typename T>
static int pack(const gbf_layout* L, const S* own_src, const S* nei_src, T* coef, void* stream) {
  int rc = check_layout(L);
  if (rc) return rc;
  if (L->n_slots == 0) return GBF_OK;
  GBF_REQUIRE(coef && (L->n_faces == 0 || (own_src && nei_src)), "pack: NULL pointer");
  const int grid = (L->n_slices * 32 + kBlock - 1) / kBlock;
  pack_kernel<S, T><<<grid, kBlock, 0, as_stream(stream)>>>(*L, own_src, nei_src, coef);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

template <typename T, typename A>
static int amul(const gbf_layout* L, const T* coef, const T* diag, const T* x, A* y,
                int nei_first, void* stream) {
  int rc = check_layout(L);
  if (rc) return rc;
  if (L->n_cells == 0) return GBF_OK;
  GBF_REQUIRE(diag && x && y && (L->n_faces == 0 || coef), "amul: NULL pointer");
  cudaStream_t s = as_stream(stream);
  const bool hex = layout_kind(*L) == kLayoutHex33;
  if constexpr (std::is_same<T, float>::value) {
    if (hex && hex_stream_aligned(coef, x, diag, L->slot_dm)) {
      if (nei_first)
        launch_amul_stream<A, true>(L, coef, diag, x, y, s);
      else
        launch_amul_stream<A, false>(L, coef, diag, x, y, s);
      GBF_CHECK_LAUNCH();
      return GBF_OK;
    }
  }
  if (nei_first) {
    if (hex)
      launch_amul<kLayoutHex33, T, A, true>(L, coef, diag, x, y, s);
    else
      launch_amul<kLayoutGeneric, T, A, true>(L, coef, diag, x, y, s);
  } else {
    if (hex)
      launch_amul<kLayoutHex33, T, A, false>(L, coef, diag, x, y, s);
    else
      launch_amul<kLayoutGeneric, T, A, false>(L, coef, diag, x, y, s);
  }
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

}  // namespace gbf

extern "C" int gbf_stream_fault(int32_t* fault) {
  GBF_REQUIRE(fault, "stream_fault: NULL pointer");
  unsigned int v = 0, zero = 0;
  GBF_CHECK_CUDA(cudaMemcpyFromSymbol(&v, gbf::g_stream_fault, sizeof(v)));
  GBF_CHECK_CUDA(cudaMemcpyToSymbol(gbf::g_stream_fault, &zero, sizeof(zero)));
  *fault = (int32_t)v;
  return GBF_OK;
}

extern "C" int gbf_pack_f64(const gbf_layout* L, const double* own_src, const double* nei_src,
                            double* slot_coef, void* stream) {
  return gbf::pack<double, double>(L, own_src, nei_src, slot_coef, stream);
}
extern "C" int gbf_pack_f32(const gbf_layout* L, const float* own_src, const float* nei_src,
                            float* slot_coef, void* stream) {
  return gbf::pack<float, float>(L, own_src, nei_src, slot_coef, stream);
}
extern "C" int gbf_pack_f64_to_f32(const gbf_layout* L, const double* own_src,
                                   const double* nei_src, float* slot_coef, void* stream) {
  return gbf::pack<double, float>(L, own_src, nei_src, slot_coef, stream);
}

extern "C" int gbf_pack_sym_f64_to_f32(const gbf_layout* L, const double* lower,
                                       const double* upper, float* coef_own, int32_t* differs,
                                       void* stream) {
  using namespace gbf;
  int rc = check_layout(L);
  if (rc) return rc;
  GBF_REQUIRE(differs, "pack_sym: NULL differs");
  GBF_REQUIRE(L->uniform_wo > 0 || L->n_faces == 0, "pack_sym: needs a uniform-width layout");
  cudaStream_t s = as_stream(stream);
  GBF_CHECK_CUDA(cudaMemsetAsync(differs, 0, sizeof(int32_t), s));
  if (L->n_slices == 0 || L->n_faces == 0) return GBF_OK;
  GBF_REQUIRE(coef_own && lower && upper, "pack_sym: NULL pointer");
  const int grid = (L->n_slices * 32 + kBlock - 1) / kBlock;
  pack_sym_kernel<<<grid, kBlock, 0, s>>>(*L, lower, upper, coef_own, differs);
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_amul_sym_f32(const gbf_layout* L, const float* coef_own, const float* diag,
                                const float* x, float* y, void* stream) {
  using namespace gbf;
  int rc = check_layout(L);
  if (rc) return rc;
  if (L->n_cells == 0) return GBF_OK;
  GBF_REQUIRE(layout_sym_ok(*L), "amul_sym: needs a hex 3+3 layout with a mirror table");
  GBF_REQUIRE(diag && x && y && coef_own, "amul_sym: NULL pointer");
  cudaStream_t s = as_stream(stream);
  if (kSymStaged && hex_stream_aligned(coef_own, x, diag, L->slot_dm) &&
      (reinterpret_cast<uintptr_t>(L->slot_mirror) & 15u) == 0) {
    launch_amul_stream<float, false, true>(L, coef_own, diag, x, y, s);
  } else {
    const int grid = wave_grid(amul_sym_kernel, kBlock, L->n_cells);
    amul_sym_kernel<<<grid, kBlock, 0, s>>>(*L, coef_own, diag, x, y);
  }
  GBF_CHECK_LAUNCH();
  return GBF_OK;
}

extern "C" int gbf_amul_f64(const gbf_layout* L, const double* slot_coef, const double* diag,
                            const double* x, double* y, int32_t nei_first, void* stream) {
  return gbf::amul<double, double>(L, slot_coef, diag, x, y, nei_first, stream);
}
extern "C" int gbf_amul_f32_f64out(const gbf_layout* L, const float* slot_coef,
                                   const float* diag, const float* x, double* y,
                                   int32_t nei_first, void* stream) {
  return gbf::amul<float, double>(L, slot_coef, diag, x, y, nei_first, stream);
}
extern "C" int gbf_amul_f32(const gbf_layout* L, const float* slot_coef, const float* diag,
                            const float* x, float* y, int32_t nei_first, void* stream) {
  return gbf::amul<float, float>(L, slot_coef, diag, x, y, nei_first, stream);
}
