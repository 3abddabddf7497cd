// Host-side topology analysis, run once per mesh: the cell-sliced slot layout
// and the wavefront schedules of the DIC and DILU factorisations.
//
// The reference recomputes its per-cell face lists on every preconditioner
// build with Python loops (solvers/preconditioners.py:116-122, :254-268);
// here they are computed once, in O(n + F), and reused by every launch.
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <climits>
#include <unordered_map>
#include <vector>

#include "gbfoam.h"

namespace gbf {
void set_error(const char* fmt, ...);
}

namespace {

int check_faces(int32_t n, int32_t nf, const int32_t* own, const int32_t* nei) {
  if (n < 0 || nf < 0) {
    gbf::set_error("negative size: n_cells=%d n_faces=%d", n, nf);
    return GBF_ERR_ARG;
  }
  if (nf > 0 && (!own || !nei)) {
    gbf::set_error("owner/neighbour pointer is NULL");
    return GBF_ERR_ARG;
  }
  for (int32_t f = 0; f < nf; ++f) {
    if (own[f] < 0 || own[f] >= n || nei[f] < 0 || nei[f] >= n) {
      gbf::set_error("face %d addresses a cell outside [0, %d): owner=%d neighbour=%d", f, n,
                     own[f], nei[f]);
      return GBF_ERR_RANGE;
    }
    if (own[f] == nei[f]) {
      gbf::set_error("face %d has owner == neighbour (%d)", f, own[f]);
      return GBF_ERR_RANGE;
    }
  }
  return GBF_OK;
}

// counts of owner-side / neighbour-side faces per cell
void face_counts(int32_t n, int32_t nf, const int32_t* own, const int32_t* nei,
                 std::vector<int32_t>& co, std::vector<int32_t>& cn) {
  co.assign((size_t)n, 0);
  cn.assign((size_t)n, 0);
  for (int32_t f = 0; f < nf; ++f) {
    co[own[f]]++;
    cn[nei[f]]++;
  }
}

// Stable per-cell lists of neighbour-side faces (ascending face order).
void neighbour_lists(int32_t n, int32_t nf, const int32_t* nei, std::vector<int64_t>& ptr,
                     std::vector<int32_t>& faces) {
  ptr.assign((size_t)n + 1, 0);
  for (int32_t f = 0; f < nf; ++f) ptr[(size_t)nei[f] + 1]++;
  for (int32_t c = 0; c < n; ++c) ptr[c + 1] += ptr[c];
  faces.resize((size_t)nf);
  std::vector<int64_t> cur(ptr.begin(), ptr.end() - 1);
  for (int32_t f = 0; f < nf; ++f) faces[cur[nei[f]]++] = f;
}

// Counting sort of items by level (stable: ascending item index per level).
void bucket_by_level(int32_t n_items, const std::vector<int32_t>& level, int32_t n_levels,
                     int32_t* level_ptr, int32_t* items, int32_t* max_size) {
  std::vector<int32_t> cnt((size_t)n_levels + 1, 0);
  for (int32_t i = 0; i < n_items; ++i) cnt[(size_t)level[i] + 1]++;
  int32_t mx = 0;
  for (int32_t l = 0; l < n_levels; ++l) {
    mx = std::max(mx, cnt[(size_t)l + 1]);
    cnt[(size_t)l + 1] += cnt[l];
  }
  for (int32_t l = 0; l <= n_levels; ++l) level_ptr[l] = cnt[l];
  for (int32_t i = 0; i < n_items; ++i) items[cnt[level[i]]++] = i;
  *max_size = mx;
}

}  // namespace

// ---------------------------------------------------------------------------
// Slot assignment of one slice side (owner- or neighbour-side faces of its
// 32 cells).  Each lane's faces, in ascending face order, carry the column
// offset d = column - cell.  The slots of the slice form one sequence of
// offsets M, built so that every lane's offset sequence is a subsequence of
// M (greedy merge); a lane's faces then go to the slots where their offsets
// sit in M, in order, and the other slots of that lane are holes.  Every
// cell still visits its faces in ascending face order (the reference's
// summation order), and every slot holds one offset for the whole slice,
// which the offset compression below stores once.  If merging would widen
// the side by more than 4 slots over the densest lane, the side falls back
// to the dense assignment (k-th face in slot k).
// ---------------------------------------------------------------------------
struct SideLists {
  std::vector<int64_t> ptr;    // per cell, into face
  std::vector<int32_t> face;   // ascending face order per cell
};

static void side_lists(int32_t n, int32_t nf, const int32_t* key, SideLists& L) {
  L.ptr.assign((size_t)n + 1, 0);
  for (int32_t f = 0; f < nf; ++f) L.ptr[(size_t)key[f] + 1]++;
  for (int32_t c = 0; c < n; ++c) L.ptr[c + 1] += L.ptr[c];
  L.face.resize((size_t)nf);
  std::vector<int64_t> cur(L.ptr.begin(), L.ptr.end() - 1);
  for (int32_t f = 0; f < nf; ++f) L.face[cur[key[f]]++] = f;
}

// Slots of the faces of slice s on one side: slot_of[k] for the k-th face
// (in cell-major, ascending-face order) of the slice; returns the width.
static int32_t assign_side(int32_t s, int32_t n, const SideLists& L, const int32_t* other,
                           std::vector<int32_t>& slot_of) {
  const int32_t c0 = s * 32, c1 = std::min(n, c0 + 32);
  int32_t dense = 0;
  for (int32_t c = c0; c < c1; ++c) dense = std::max<int32_t>(dense, (int32_t)(L.ptr[c + 1] - L.ptr[c]));
  std::vector<int64_t> M;
  for (int32_t c = c0; c < c1; ++c) {
    size_t pos = 0;
    for (int64_t k = L.ptr[c]; k < L.ptr[c + 1]; ++k) {
      const int64_t d = (int64_t)other[L.face[k]] - c;
      size_t j = pos;
      while (j < M.size() && M[j] != d) ++j;
      if (j == M.size()) {
        M.insert(M.begin() + (long)pos, d);
        j = pos;
      }
      pos = j + 1;
    }
  }
  slot_of.clear();
  if ((int32_t)M.size() > dense + 4) {  // irregular slice: dense slots
    for (int32_t c = c0; c < c1; ++c)
      for (int64_t k = L.ptr[c]; k < L.ptr[c + 1]; ++k) slot_of.push_back((int32_t)(k - L.ptr[c]));
    return dense;
  }
  for (int32_t c = c0; c < c1; ++c) {
    size_t pos = 0;
    for (int64_t k = L.ptr[c]; k < L.ptr[c + 1]; ++k) {
      const int64_t d = (int64_t)other[L.face[k]] - c;
      size_t j = pos;
      while (M[j] != d) ++j;  // an embedding exists by construction
      slot_of.push_back((int32_t)j);
      pos = j + 1;
    }
  }
  return (int32_t)M.size();
}

// Widths of every slice side; decides uniform padding.
static int plan_widths(int32_t n, int32_t nf, const int32_t* own, const int32_t* nei,
                       const SideLists& lo, const SideLists& ln, int32_t pad_pct,
                       std::vector<int32_t>& wo, std::vector<int32_t>& wn, int32_t& uni_o,
                       int32_t& uni_n) {
  const int32_t ns = (n + 31) / 32;
  wo.resize((size_t)ns);
  wn.resize((size_t)ns);
  std::vector<int32_t> tmp;
  int64_t slots = 0;
  int32_t mo = 0, mn = 0;
  for (int32_t s = 0; s < ns; ++s) {
    wo[s] = assign_side(s, n, lo, nei, tmp);
    wn[s] = assign_side(s, n, ln, own, tmp);
    if (wo[s] > 0xffff || wn[s] > 0x7fff) {
      gbf::set_error("a slice needs more than 32767 slots");
      return GBF_ERR_ARG;
    }
    slots += 32 * (int64_t)(wo[s] + wn[s]);
    mo = std::max(mo, wo[s]);
    mn = std::max(mn, wn[s]);
  }
  uni_o = uni_n = 0;
  const int64_t uni_slots = 32 * (int64_t)ns * (mo + mn);
  if (pad_pct >= 0 && ns > 0 && uni_slots * 100 <= slots * (100 + (int64_t)pad_pct)) {
    uni_o = mo;
    uni_n = mn;
    for (int32_t s = 0; s < ns; ++s) {
      wo[s] = mo;
      wn[s] = mn;
    }
  }
  return GBF_OK;
}

extern "C" int gbf_layout_plan(int32_t n, int32_t nf, const int32_t* own, const int32_t* nei,
                               int32_t pad_pct, int32_t* n_slices, int64_t* n_slots,
                               int32_t* max_width, int32_t* uniform) {
  int rc = check_faces(n, nf, own, nei);
  if (rc) return rc;
  SideLists lo, ln;
  side_lists(n, nf, own, lo);
  side_lists(n, nf, nei, ln);
  std::vector<int32_t> wo, wn;
  int32_t uo, un;
  rc = plan_widths(n, nf, own, nei, lo, ln, pad_pct, wo, wn, uo, un);
  if (rc) return rc;
  const int32_t ns = (n + 31) / 32;
  int64_t slots = 0;
  int32_t mw = 0;
  for (int32_t s = 0; s < ns; ++s) {
    slots += 32 * (int64_t)(wo[s] + wn[s]);
    mw = std::max(mw, wo[s] + wn[s]);
  }
  if (slots >= ((int64_t)1 << 31)) {
    gbf::set_error("matrix needs %lld slots; the layout holds < 2^31", (long long)slots);
    return GBF_ERR_ARG;
  }
  *n_slices = ns;
  *n_slots = slots;
  *max_width = mw;
  if (uniform) *uniform = uo > 0 || un > 0 ? 1 : 0;
  return GBF_OK;
}

extern "C" int gbf_layout_fill(int32_t n, int32_t nf, const int32_t* own, const int32_t* nei,
                               int32_t pad_pct, int32_t* slice_off, int32_t* slice_w,
                               int32_t* slot_col, int32_t* slot_face) {
  int rc = check_faces(n, nf, own, nei);
  if (rc) return rc;
  SideLists lo, ln;
  side_lists(n, nf, own, lo);
  side_lists(n, nf, nei, ln);
  std::vector<int32_t> wos, wns;
  int32_t uo, un;
  rc = plan_widths(n, nf, own, nei, lo, ln, pad_pct, wos, wns, uo, un);
  if (rc) return rc;
  const int32_t ns = (n + 31) / 32;
  int64_t off = 0;
  std::vector<int32_t> so, sn;
  for (int32_t s = 0; s < ns; ++s) {
    assign_side(s, n, lo, nei, so);
    assign_side(s, n, ln, own, sn);
    const int32_t wo = wos[s], wn = wns[s];
    slice_off[s] = (int32_t)off;
    slice_w[s] = wo | (wn << 16);
    for (int64_t i = off; i < off + 32 * (int64_t)(wo + wn); ++i) {
      slot_col[i] = -1;
      slot_face[i] = -1;
    }
    const int32_t c0 = s * 32, c1 = std::min(n, c0 + 32);
    size_t qo = 0, qn = 0;
    for (int32_t c = c0; c < c1; ++c) {
      const int32_t lane = c & 31;
      for (int64_t k = lo.ptr[c]; k < lo.ptr[c + 1]; ++k) {
        const int32_t f = lo.face[k];
        const int64_t slot = off + 32 * (int64_t)so[qo++] + lane;
        slot_col[slot] = nei[f];
        slot_face[slot] = f;
      }
      for (int64_t k = ln.ptr[c]; k < ln.ptr[c + 1]; ++k) {
        const int32_t f = ln.face[k];
        const int64_t slot = off + 32 * (int64_t)(wo + sn[qn++]) + lane;
        slot_col[slot] = own[f];
        slot_face[slot] = f;
      }
    }
    off += 32 * (int64_t)(wo + wn);
  }
  slice_off[ns] = (int32_t)off;
  return GBF_OK;
}

extern "C" int gbf_dic_schedule(int32_t n, int32_t nf, const int32_t* own, const int32_t* nei,
                                int32_t* level_ptr, int32_t* level_cells, int32_t* n_levels,
                                int32_t* max_level_size) {
  int rc = check_faces(n, nf, own, nei);
  if (rc) return rc;
  std::vector<int64_t> ptr;
  std::vector<int32_t> faces;
  neighbour_lists(n, nf, nei, ptr, faces);
  std::vector<int32_t> level((size_t)n, 0);
  int32_t nl = (n > 0) ? 1 : 0;
  for (int32_t c = 0; c < n; ++c) {
    int32_t l = 0;
    for (int64_t k = ptr[c]; k < ptr[c + 1]; ++k) {
      const int32_t j = own[faces[k]];
      if (j < c) l = std::max(l, level[j] + 1);  // j > c reads the unfactored diagonal
    }
    level[c] = l;
    nl = std::max(nl, l + 1);
  }
  bucket_by_level(n, level, nl, level_ptr, level_cells, max_level_size);
  *n_levels = nl;
  return GBF_OK;
}

extern "C" int gbf_dilu_schedule(int32_t n, int32_t nf, const int32_t* own, const int32_t* nei,
                                 int32_t* level_ptr, int32_t* level_faces, int32_t* n_levels,
                                 int32_t* max_level_size) {
  int rc = check_faces(n, nf, own, nei);
  if (rc) return rc;
  std::vector<int32_t> last((size_t)n, -1), level((size_t)nf, 0);
  int32_t nl = 0;
  for (int32_t f = 0; f < nf; ++f) {
    const int32_t l = std::max(last[own[f]], last[nei[f]]) + 1;
    level[f] = l;
    last[own[f]] = l;
    last[nei[f]] = l;
    nl = std::max(nl, l + 1);
  }
  bucket_by_level(nf, level, nl, level_ptr, level_faces, max_level_size);
  *n_levels = nl;
  return GBF_OK;
}

// Links of the dataflow DILU factorisation.  Item i of the level schedule
// (face level_faces[i]) writes slots 2i (its owner's value after the face)
// and 2i+1 (its neighbour's); prev[2i] and prev[2i+1] name the slots that
// hold the two cells' values before the face -- the slot written by the
// previous face touching the cell in face order, the sequential order of
// preconditioners.py:254-268 -- or -1 where that is the diagonal.
// cell_last[c] is the slot of the last face touching c, or -1.  Refuses a
// level_faces that is not a permutation of the faces or that places a face
// before one it reads (the walk would wait on a later step).
extern "C" int gbf_dilu_flow_links(int32_t n, int32_t nf, const int32_t* own, const int32_t* nei,
                                   const int32_t* level_faces, int32_t* prev,
                                   int32_t* cell_last) {
  int rc = check_faces(n, nf, own, nei);
  if (rc) return rc;
  if (nf >= (1 << 30)) {
    gbf::set_error("dilu_flow_links: %d faces (at most 2^30 - 1)", nf);
    return GBF_ERR_ARG;
  }
  if (n > 0 && !cell_last) {
    gbf::set_error("dilu_flow_links: NULL pointer");
    return GBF_ERR_ARG;
  }
  if (nf > 0 && (!level_faces || !prev)) {
    gbf::set_error("dilu_flow_links: NULL pointer");
    return GBF_ERR_ARG;
  }
  std::vector<int32_t> pos((size_t)nf, -1);
  for (int32_t i = 0; i < nf; ++i) {
    const int32_t f = level_faces[i];
    if (f < 0 || f >= nf || pos[f] >= 0) {
      gbf::set_error("dilu_flow_links: level_faces is not a permutation of the faces (item %d)",
                     i);
      return GBF_ERR_ARG;
    }
    pos[f] = i;
  }
  for (int32_t c = 0; c < n; ++c) cell_last[c] = -1;
  for (int32_t f = 0; f < nf; ++f) {
    const int32_t i = pos[f], p = own[f], q = nei[f];
    const int32_t a = cell_last[p], b = cell_last[q];
    if ((a >= 0 && a / 2 >= i) || (b >= 0 && b / 2 >= i)) {
      gbf::set_error("dilu_flow_links: face %d is scheduled before a face it reads", f);
      return GBF_ERR_ARG;
    }
    prev[2 * (int64_t)i] = a;
    prev[2 * (int64_t)i + 1] = b;
    cell_last[p] = 2 * i;
    cell_last[q] = 2 * i + 1;
  }
  return GBF_OK;
}

// Links of the dataflow triangular sweep over the schedule of
// gbf_sweep_schedule(reverse, lower_only) (items = its level_faces, n_items
// of them).  Item i (face f, read cell R, written cell W) writes slot i, the
// value of W after the face; prev[2i] names the slot of W's value before the
// face and prev[2i+1] the slot of R's value at the face -- the slot of the
// last earlier face in sweep order that wrote the cell, or -1 for the
// cell's value on entry.  cell_last[c] is the slot of c's last write, or -1.
// Refuses items that are not distinct faces or that come before a face they
// read.
extern "C" int gbf_sweep_flow_links(int32_t n, int32_t nf, const int32_t* own,
                                    const int32_t* nei, int32_t reverse, int32_t n_items,
                                    const int32_t* items, int32_t* prev, int32_t* cell_last) {
  int rc = check_faces(n, nf, own, nei);
  if (rc) return rc;
  if (n_items < 0 || n_items > nf || (n_items > 0 && (!items || !prev)) ||
      (n > 0 && !cell_last)) {
    gbf::set_error("sweep_flow_links: bad arguments");
    return GBF_ERR_ARG;
  }
  std::vector<int32_t> pos((size_t)nf, -1);
  for (int32_t i = 0; i < n_items; ++i) {
    const int32_t f = items[i];
    if (f < 0 || f >= nf || pos[f] >= 0) {
      gbf::set_error("sweep_flow_links: items are not distinct faces (item %d)", i);
      return GBF_ERR_ARG;
    }
    pos[f] = i;
  }
  for (int32_t c = 0; c < n; ++c) cell_last[c] = -1;
  for (int32_t j = 0; j < nf; ++j) {
    const int32_t f = reverse ? nf - 1 - j : j;
    const int32_t i = pos[f];
    if (i < 0) continue;
    const int32_t R = reverse ? nei[f] : own[f];
    const int32_t W = reverse ? own[f] : nei[f];
    const int32_t a = cell_last[W], b = cell_last[R];
    if (a >= i || b >= i) {
      gbf::set_error("sweep_flow_links: face %d is scheduled before a face it reads", f);
      return GBF_ERR_ARG;
    }
    prev[2 * (int64_t)i] = a;
    prev[2 * (int64_t)i + 1] = b;
    cell_last[W] = i;
  }
  return GBF_OK;
}

// Per-cell lists of boundary faces in ascending face order (the order in
// which fvm.laplacian's boundary scatter_add, operators.py:508-515, adds
// them).  owner_b holds owner[n_internal .. n_internal + n_bnd); the listed
// face ids are n_internal + k.
extern "C" int gbf_boundary_lists(int32_t n, int32_t n_internal, int32_t n_bnd,
                                  const int32_t* owner_b, int32_t* bnd_ptr, int32_t* bnd_face) {
  if (n < 0 || n_internal < 0 || n_bnd < 0 || (n_bnd > 0 && !owner_b) || !bnd_ptr ||
      (n_bnd > 0 && !bnd_face)) {
    gbf::set_error("boundary_lists: bad arguments");
    return GBF_ERR_ARG;
  }
  for (int32_t k = 0; k < n_bnd; ++k)
    if (owner_b[k] < 0 || owner_b[k] >= n) {
      gbf::set_error("boundary face %d has owner %d outside [0, %d)", n_internal + k, owner_b[k], n);
      return GBF_ERR_RANGE;
    }
  for (int32_t c = 0; c <= n; ++c) bnd_ptr[c] = 0;
  for (int32_t k = 0; k < n_bnd; ++k) bnd_ptr[owner_b[k] + 1]++;
  for (int32_t c = 0; c < n; ++c) bnd_ptr[c + 1] += bnd_ptr[c];
  std::vector<int32_t> cur(bnd_ptr, bnd_ptr + (n > 0 ? n : 0));
  for (int32_t k = 0; k < n_bnd; ++k) bnd_face[cur[owner_b[k]]++] = n_internal + k;
  return GBF_OK;
}

// Wavefront schedule of a face-ordered triangular sweep (the full DIC / DILU
// solves, solvers/preconditioners.py:153-201, :290-337).  Face f reads cell
// R and updates cell W (forward: R = owner, W = neighbour, faces ascending;
// reverse: R = neighbour, W = owner, faces descending); with lower_only the
// faces with owner >= neighbour are skipped (the DIC sweeps' "if p < n").
// A face's level follows the last writer of R (read after write) and the last
// reader or writer of W (write after read / write), so every level can run
// in parallel and each cell sees its updates in the reference's face order.
extern "C" int gbf_sweep_schedule(int32_t n, int32_t nf, const int32_t* own, const int32_t* nei,
                                  int32_t reverse, int32_t lower_only, int32_t* level_ptr,
                                  int32_t* level_faces, int32_t* n_levels,
                                  int32_t* max_level_size) {
  int rc = check_faces(n, nf, own, nei);
  if (rc) return rc;
  std::vector<int32_t> last_w((size_t)n, -1), last_a((size_t)n, -1);
  std::vector<int32_t> level((size_t)nf, -1);
  int32_t nl = 0, used = 0;
  for (int32_t i = 0; i < nf; ++i) {
    const int32_t f = reverse ? nf - 1 - i : i;
    if (lower_only && !(own[f] < nei[f])) continue;
    const int32_t R = reverse ? nei[f] : own[f];
    const int32_t W = reverse ? own[f] : nei[f];
    const int32_t l = std::max(last_w[R], last_a[W]) + 1;
    level[f] = l;
    last_w[W] = l;
    last_a[W] = l;
    last_a[R] = std::max(last_a[R], l);
    nl = std::max(nl, l + 1);
    ++used;
  }
  // bucket by level; inside a level, faces in sweep order
  std::vector<int32_t> cnt((size_t)nl + 1, 0);
  for (int32_t f = 0; f < nf; ++f)
    if (level[f] >= 0) cnt[(size_t)level[f] + 1]++;
  int32_t mx = 0;
  for (int32_t l = 0; l < nl; ++l) {
    mx = std::max(mx, cnt[(size_t)l + 1]);
    cnt[(size_t)l + 1] += cnt[l];
  }
  for (int32_t l = 0; l <= nl; ++l) level_ptr[l] = cnt[l];
  for (int32_t i = 0; i < nf; ++i) {
    const int32_t f = reverse ? nf - 1 - i : i;
    if (level[f] >= 0) level_faces[cnt[level[f]]++] = f;
  }
  *n_levels = nl;
  *max_level_size = mx;
  (void)used;
  return GBF_OK;
}

// Offset compression of the slot columns.  For every (slice, slot) the 32
// lanes' columns are stored as one offset `delta` (column = cell + delta)
// plus a 32-bit mask of the lanes that hold a face, whenever all those
// lanes share the same offset -- the common case on meshes whose cells are
// numbered along a structured direction (a hex mesh has offsets +-1, +-nx,
// +-nx*ny).  Otherwise delta = INT32_MIN and the kernels read slot_col.
// Entry (s, k) lives at slice_off[s] / 32 + k as the int32 pair
// {delta, mask}: 8 bytes per 32 slots instead of 128.
extern "C" int gbf_layout_compress(int32_t n_slices, const int32_t* slice_off,
                                   const int32_t* slice_w, const int32_t* slot_col,
                                   int32_t* slot_dm, int64_t* n_uniform) {
  if (n_slices < 0 || !slice_off || !slice_w || !slot_col || !slot_dm) {
    gbf::set_error("layout_compress: bad arguments");
    return GBF_ERR_ARG;
  }
  int64_t uni = 0;
  for (int32_t s = 0; s < n_slices; ++s) {
    const int32_t w = (slice_w[s] & 0xffff) + (slice_w[s] >> 16);
    const int64_t e0 = slice_off[s] / 32;
    for (int32_t k = 0; k < w; ++k) {
      const int64_t base = (int64_t)slice_off[s] + 32 * (int64_t)k;
      uint32_t mask = 0;
      bool uniform = true, have = false;
      int64_t d = 0;
      for (int32_t l = 0; l < 32; ++l) {
        const int32_t col = slot_col[base + l];
        if (col < 0) continue;
        const int64_t dl = (int64_t)col - ((int64_t)s * 32 + l);
        if (!have) {
          d = dl;
          have = true;
        } else if (dl != d) {
          uniform = false;
        }
        mask |= 1u << l;
      }
      if (!have) {  // a slot that is a hole in every lane
        slot_dm[2 * (e0 + k)] = 0;
        ++uni;
      } else if (uniform && d > INT32_MIN && d <= INT32_MAX) {
        slot_dm[2 * (e0 + k)] = (int32_t)d;
        ++uni;
      } else {
        slot_dm[2 * (e0 + k)] = INT32_MIN;
      }
      slot_dm[2 * (e0 + k) + 1] = (int32_t)mask;
    }
  }
  if (n_uniform) *n_uniform = uni;
  return GBF_OK;
}

// Mirror table for symmetric matrices: each neighbour-side entry (s, k) of a
// uniform-width compressed layout gets the owner-side slot j holding the
// same face in its owner's slice, provided j is the same for every lane of
// the entry and the entry is offset-compressed.
extern "C" int gbf_layout_mirror(int32_t n_faces, int32_t n_slices, int32_t wo, int32_t wn,
                                 const int32_t* slot_face, const int32_t* owner,
                                 const int32_t* slot_dm, int8_t* slot_mirror, int32_t* ok) {
  if (n_faces < 0 || n_slices < 0 || wo < 0 || wn < 0 || !ok ||
      (n_slices > 0 && (!slot_face || !slot_dm || !slot_mirror)) || (n_faces > 0 && !owner)) {
    gbf::set_error("layout_mirror: bad arguments");
    return GBF_ERR_ARG;
  }
  *ok = (wo > 0 && wo <= 127 && n_faces > 0) ? 1 : 0;
  const int64_t W = (int64_t)wo + wn;
  std::vector<int8_t> own_j((size_t)n_faces, -1);
  for (int64_t s = 0; s < n_slices; ++s)
    for (int32_t j = 0; j < wo; ++j) {
      slot_mirror[s * W + j] = -1;
      for (int32_t l = 0; l < 32; ++l) {
        const int32_t f = slot_face[32 * (s * W + j) + l];
        if (f < 0) continue;
        if (f >= n_faces || j > 127 || owner[f] != (int32_t)(32 * s + l)) {
          *ok = 0;
          continue;
        }
        own_j[(size_t)f] = (int8_t)j;
      }
    }
  for (int64_t s = 0; s < n_slices; ++s)
    for (int32_t k = wo; k < W; ++k) {
      const int64_t e = s * W + k;
      int32_t jj = -1;
      for (int32_t l = 0; l < 32; ++l) {
        const int32_t f = slot_face[32 * e + l];
        if (f < 0) continue;
        const int32_t j = (f < n_faces) ? own_j[(size_t)f] : -1;
        if (j < 0 || (jj >= 0 && j != jj) || slot_dm[2 * e] == INT32_MIN ||
            (int64_t)owner[f] != 32 * s + l + (int64_t)slot_dm[2 * e])
          *ok = 0;
        if (jj < 0) jj = j;
      }
      slot_mirror[e] = (int8_t)jj;
    }
  return GBF_OK;
}

// Cell -> face lists in the order the reference's cell-geometry loop visits
// them (mesh/mesh_geometry.py:191-196): every face the cell owns, ascending
// (boundary faces included), then every internal face it neighbours,
// ascending, the latter stored as ~face.
extern "C" int gbf_cell_faces(int32_t n_cells, int32_t n_faces, int32_t n_internal,
                              const int32_t* owner, const int32_t* neighbour, int32_t* cell_ptr,
                              int32_t* cell_faces) {
  if (n_cells < 0 || n_faces < 0 || n_internal < 0 || n_internal > n_faces || !cell_ptr ||
      (n_faces > 0 && (!owner || !cell_faces)) || (n_internal > 0 && !neighbour)) {
    gbf::set_error("cell_faces: bad arguments");
    return GBF_ERR_ARG;
  }
  for (int32_t f = 0; f < n_faces; ++f)
    if (owner[f] < 0 || owner[f] >= n_cells || (f < n_internal &&
                                                 (neighbour[f] < 0 || neighbour[f] >= n_cells))) {
      gbf::set_error("cell_faces: face %d has a cell index outside [0, %d)", f, n_cells);
      return GBF_ERR_RANGE;
    }
  std::vector<int64_t> cnt((size_t)n_cells + 1, 0);
  for (int32_t f = 0; f < n_faces; ++f) cnt[(size_t)owner[f] + 1]++;
  for (int32_t f = 0; f < n_internal; ++f) cnt[(size_t)neighbour[f] + 1]++;
  for (int32_t c = 0; c < n_cells; ++c) cnt[c + 1] += cnt[c];
  if (cnt[n_cells] > INT32_MAX) {
    gbf::set_error("cell_faces: too many cell-face entries");
    return GBF_ERR_ARG;
  }
  std::vector<int64_t> cur(cnt.begin(), cnt.end() - 1);
  for (int32_t f = 0; f < n_faces; ++f) cell_faces[cur[owner[f]]++] = f;
  for (int32_t f = 0; f < n_internal; ++f) cell_faces[cur[neighbour[f]]++] = ~f;
  for (int32_t c = 0; c <= n_cells; ++c) cell_ptr[c] = (int32_t)cnt[c];
  return GBF_OK;
}

// Gauss-Seidel wavefront: forward (reverse = 0) level(c) = 1 + max level of
// the neighbours j < c (cells ascending); backward (reverse = 1) the same
// over the neighbours j > c (cells descending).  Neighbours never share a
// level, and every cell runs after the neighbours the sequential sweep has
// already updated when it reaches the cell.
extern "C" int gbf_gs_schedule(int32_t n, int32_t nf, const int32_t* own, const int32_t* nei,
                               int32_t reverse, int32_t* level_ptr, int32_t* level_cells,
                               int32_t* n_levels, int32_t* max_level_size) {
  int rc = check_faces(n, nf, own, nei);
  if (rc) return rc;
  std::vector<int64_t> ptr((size_t)n + 1, 0);
  for (int32_t f = 0; f < nf; ++f) {
    ptr[(size_t)own[f] + 1]++;
    ptr[(size_t)nei[f] + 1]++;
  }
  for (int32_t c = 0; c < n; ++c) ptr[c + 1] += ptr[c];
  std::vector<int32_t> adj((size_t)ptr[n]);
  std::vector<int64_t> cur(ptr.begin(), ptr.end() - 1);
  for (int32_t f = 0; f < nf; ++f) {
    adj[cur[own[f]]++] = nei[f];
    adj[cur[nei[f]]++] = own[f];
  }
  std::vector<int32_t> level((size_t)n, 0);
  int32_t nl = (n > 0) ? 1 : 0;
  for (int32_t q = 0; q < n; ++q) {
    const int32_t c = reverse ? n - 1 - q : q;
    int32_t l = 0;
    for (int64_t k = ptr[c]; k < ptr[c + 1]; ++k) {
      const int32_t j = adj[k];
      if (reverse ? j > c : j < c) l = std::max(l, level[j] + 1);
    }
    level[c] = l;
    nl = std::max(nl, l + 1);
  }
  bucket_by_level(n, level, nl, level_ptr, level_cells, max_level_size);
  *n_levels = nl;
  return GBF_OK;
}

// GAMG coarsening (solvers/gamg.py:183-245): greedy aggregation in cell
// order.  Each unaggregated cell seeds an aggregate and takes its
// unaggregated neighbours (adjacency in face order, owner side and
// neighbour side as the faces list them); once the target count is reached
// every remaining cell joins the aggregate of its first aggregated
// neighbour (cell 0's aggregate if none), in cell order.
extern "C" int gbf_gamg_aggregate(int32_t n, int32_t nf, const int32_t* own, const int32_t* nei,
                                  int32_t n_coarse_target, int32_t* f2c, int32_t* n_coarse) {
  int rc = check_faces(n, nf, own, nei);
  if (rc) return rc;
  if (!n_coarse || (n > 0 && !f2c)) {
    gbf::set_error("gamg_aggregate: NULL pointer");
    return GBF_ERR_ARG;
  }
  std::vector<int64_t> ptr((size_t)n + 1, 0);
  for (int32_t f = 0; f < nf; ++f) {
    ptr[(size_t)own[f] + 1]++;
    ptr[(size_t)nei[f] + 1]++;
  }
  for (int32_t c = 0; c < n; ++c) ptr[c + 1] += ptr[c];
  std::vector<int32_t> adj((size_t)ptr[n]);
  std::vector<int64_t> cur(ptr.begin(), ptr.end() - 1);
  for (int32_t f = 0; f < nf; ++f) {
    adj[cur[own[f]]++] = nei[f];
    adj[cur[nei[f]]++] = own[f];
  }
  for (int32_t c = 0; c < n; ++c) f2c[c] = -1;
  int32_t nag = 0;
  for (int32_t cell = 0; cell < n; ++cell) {
    if (f2c[cell] >= 0) continue;
    const int32_t id = nag++;
    f2c[cell] = id;
    for (int64_t k = ptr[cell]; k < ptr[cell + 1]; ++k)
      if (f2c[adj[k]] < 0) f2c[adj[k]] = id;
    if (nag >= n_coarse_target) {
      for (int32_t r = 0; r < n; ++r) {
        if (f2c[r] >= 0) continue;
        bool assigned = false;
        for (int64_t k = ptr[r]; k < ptr[r + 1]; ++k)
          if (f2c[adj[k]] >= 0) {
            f2c[r] = f2c[adj[k]];
            assigned = true;
            break;
          }
        if (!assigned) f2c[r] = 0;
      }
      break;
    }
  }
  for (int32_t c = 0; c < n; ++c)
    if (f2c[c] < 0) f2c[c] = 0;
  *n_coarse = nag;
  return GBF_OK;
}

// GAMG coarse faces (solvers/gamg.py:249-331): fine faces whose two cells
// fall in different aggregates, merged per unordered aggregate pair in order
// of first appearance; the coarse face keeps the (owner, neighbour)
// aggregates of its first fine face.  face_to_cface[f] = coarse face of
// fine face f, -1 inside an aggregate.  Output arrays hold n_faces entries.
extern "C" int gbf_gamg_coarse_faces(int32_t nf, const int32_t* own, const int32_t* nei,
                                     const int32_t* f2c, int32_t* coarse_own, int32_t* coarse_nei,
                                     int32_t* face_to_cface, int32_t* n_cfaces) {
  if (nf < 0 || !n_cfaces ||
      (nf > 0 && (!own || !nei || !f2c || !coarse_own || !coarse_nei || !face_to_cface))) {
    gbf::set_error("gamg_coarse_faces: bad arguments");
    return GBF_ERR_ARG;
  }
  std::unordered_map<uint64_t, int32_t> seen;
  seen.reserve((size_t)nf);
  int32_t nc = 0;
  for (int32_t f = 0; f < nf; ++f) {
    const int32_t cp = f2c[own[f]], cn = f2c[nei[f]];
    if (cp == cn) {
      face_to_cface[f] = -1;
      continue;
    }
    const uint64_t key = ((uint64_t)(uint32_t)std::min(cp, cn) << 32) | (uint32_t)std::max(cp, cn);
    auto it = seen.find(key);
    if (it != seen.end()) {
      face_to_cface[f] = it->second;
    } else {
      seen.emplace(key, nc);
      coarse_own[nc] = cp;
      coarse_nei[nc] = cn;
      face_to_cface[f] = nc++;
    }
  }
  *n_cfaces = nc;
  return GBF_OK;
}
