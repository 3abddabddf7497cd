/*
 * gbfoam.h -- C ABI of libgbfoam.so, the GB300 (sm_103a) kernels behind
 * pyopenfoam_gb300's LduMatrix / FvMatrix / PCG / PBiCGStab / DIC / DILU /
 * fvm.laplacian / DifferentiableLinearSolve.
 *
 * Conventions
 *   - Every function returns an int status: 0 = OK, non-zero = error code;
 *     gbf_last_error() returns a message for the calling thread's last error.
 *   - Pointers are DEVICE pointers unless the parameter name ends in _h
 *     (host pointer).  Sizes are element counts.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default).
 *   - Nothing allocates device memory: callers pass workspaces sized by the
 *     *_workspace_bytes queries.
 *   - Cell/face indices are int32; a matrix holds < 2^31 slots.
 *
 * Each entry point names the reference routine it replaces, cited as
 * file:line inside alanZee/pyOpenFOAM (src/pyfoam/...).  The reference is
 * pure Python on PyTorch; its binding of these entry points is the ctypes
 * layer in pyopenfoam_gb300/_lib.py.
 */
#ifndef GBFOAM_H
#define GBFOAM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBF_OK 0
#define GBF_ERR_ARG 1      /* bad size / pointer / index                        */
#define GBF_ERR_CUDA 2     /* a CUDA runtime call failed                        */
#define GBF_ERR_WORKSPACE 3/* workspace too small                              */
#define GBF_ERR_RANGE 4    /* owner/neighbour index out of range                */

/* Solver status codes written to gbf_solve_result.status */
#define GBF_RUNNING 0
#define GBF_CONVERGED 1
#define GBF_BREAKDOWN 2
#define GBF_MAX_ITER 3
#define GBF_DEVICE_TIMEOUT 4 /* a bounded wait inside a kernel ran out; results invalid */

/* Cell-sliced LDU addressing (built once per mesh topology).
 *
 * Cells are grouped in slices of 32 consecutive cells (one warp).  Inside a
 * slice, slot k of lane l lives at slice_off[s] + 32*k + l, so every slot
 * read by a warp is one coalesced 128/256-byte line.  The first `wo` slots of
 * a slice are the cell's OWNER-side faces (faces with owner == cell, in
 * ascending face order), the next `wn` slots its NEIGHBOUR-side faces
 * (neighbour == cell, ascending face order); unused slots have col = -1.
 * This keeps the per-cell summation order of the reference's face-ordered
 * scatter_add, so the gather is bitwise identical to LduMatrix.Ax.
 */
typedef struct gbf_layout {
  int32_t n_cells;
  int32_t n_faces;         /* internal faces                                   */
  int32_t n_slices;        /* ceil(n_cells / 32)                               */
  int32_t max_width;       /* max over slices of wo + wn                       */
  int32_t uniform_wo;      /* > 0: every slice has wo = uniform_wo and
                              wn = uniform_wn, slice_off[s] = 32*s*(wo+wn)  */
  int32_t uniform_wn;
  int32_t all_uniform;     /* 1: slot_dm set and no entry is INT32_MIN      */
  int32_t reserved;
  int64_t n_slots;         /* total slots incl. padding                        */
  const int32_t* slice_off;/* [n_slices + 1]                                   */
  const int32_t* slice_w;  /* [n_slices]  wo | (wn << 16)                      */
  const int32_t* slot_col; /* [n_slots]   column cell, -1 = padding            */
  const int32_t* slot_face;/* [n_slots]   face of the slot, -1 = padding       */
  const int32_t* owner;    /* [n_faces]   face-order owner (int32)             */
  const int32_t* neighbour;/* [n_faces]   face-order neighbour (int32)         */
  /* optional offset compression (gbf_layout_compress); NULL = use slot_col:
   * per (slice, slot) {column - cell or INT32_MIN, mask of lanes with a face} */
  const int32_t* slot_dm;    /* [2 * n_slots/32]                            */
  /* optional mirror table for symmetric matrices (gbf_layout_mirror); NULL =
   * none.  Entry (s, k) of a NEIGHBOUR-side slot k >= wo: the owner-side slot
   * j that holds the same face in the slice of its owner cell, the same j for
   * every lane of the slice; -1 on owner-side and hole-only entries.        */
  const int8_t* slot_mirror; /* [n_slots/32]                                 */
} gbf_layout;

/* ---- library ----------------------------------------------------------- */
const char* gbf_last_error(void);
/* Reads and clears the fault flag of the stand-alone staged Amul kernels
 * (set when a bounded wait on a bulk copy ran out; their output is then
 * invalid).  No reference counterpart.                                     */
int gbf_stream_fault(int32_t* fault);
int gbf_version(void);
/* Number of SMs of the current device (grid sizing of the reductions).     */
int gbf_device_sm_count(int32_t* n_sm);
/* Host <-> device copies driven by the SMs (loads / stores of page-locked
 * host memory over NVLink-C2C) instead of the copy engines; no reference
 * counterpart (the reference moves tensors with torch's .to(), i.e. the copy
 * engines).  src_host / dst_host must be page-locked host memory
 * (cudaHostAlloc / cudaHostRegister; torch pin_memory), the other side
 * device memory; anything else is refused with GBF_ERR_ARG.  Asynchronous
 * on `stream`; any alignment and size.                                      */
int gbf_copy_from_host(void* dst, const void* src_host, size_t bytes, void* stream);
int gbf_copy_to_host(void* dst_host, const void* src, size_t bytes, void* stream);
/* Self-test of the bounded device-side waits (no reference counterpart):
 * makes a grid-barrier wait (one participant never arrives) and an mbarrier
 * wait (nothing ever completes it) run out after short poll limits, on the
 * current device.  timed_out_h[0] = 1 if the barrier wait gave up,
 * [1] = 1 if the mbarrier wait gave up, [2] = the barrier's fault word.
 * Allocates and frees a few bytes of device memory; synchronises.          */
int gbf_selftest_bounded_waits(int32_t* timed_out_h);
/* Self-test of the cooperative wavefronts' failure path: a two-level
 * wavefront whose grid barrier can never complete (1000-poll limit).
 * result_h[0] = the barrier's fault word (1 expected), result_h[1] = 1 if
 * the output was overwritten with NaN.  No GPU fault is involved.          */
int gbf_selftest_wavefront_fault(int32_t* result_h);
/* Self-test of the dataflow factorisations' failure path: two faces whose
 * slot links point at each other (a cycle, 1000-pass limit).  result_h[0] =
 * the fault word (1 expected), result_h[1] = 1 if the output is all NaN.
 * No GPU fault is involved.                                                */
int gbf_selftest_flow_fault(int32_t* result_h);
/* Kernel timing probes (no reference counterpart; used by the benchmark to
 * time the dominant kernel inside a solve).  While enabled, the solvers
 * bracket the launches of their Amul kernels with CUDA events on the
 * launching stream; gbf_timing_read synchronises and returns, per probe,
 * the number of timed launches and their summed duration in ms.
 * Probe ids: 0 = FP64 PCG Amul+dot, 1 = mixed PCG FP32 Amul+dot,
 * 2 = PBiCGStab Amul+dot (v and t), 3 = mixed PCG FP64 true residual,
 * 4 = mixed PBiCGStab FP32 Amul+dot (v = A y).                             */
int gbf_timing_enable(int32_t enable, int32_t max_events_per_probe);
int gbf_timing_read(int32_t probe, int32_t* launches, double* total_ms);

/* ---- topology (host, once per mesh) -------------------------------------
 * Replace the reference's per-call Python loops over faces
 * (solvers/preconditioners.py:116-122, :254-268) and CSR caching
 * (core/ldu_matrix.py:101-102, :336-343) with one O(n + F) host pass. */
/* uniform_pad_pct >= 0: pad every slice to the widest slice's (wo, wn) when
 * that adds at most uniform_pad_pct percent slots (then *uniform = 1 and
 * the kernels compute slot addresses without reading slice_off/slice_w);
 * < 0 never.  plan and fill must get the same value.                       */
int gbf_layout_plan(int32_t n_cells, int32_t n_faces, const int32_t* owner_h,
                    const int32_t* neighbour_h, int32_t uniform_pad_pct, int32_t* n_slices,
                    int64_t* n_slots, int32_t* max_width, int32_t* uniform);
int gbf_layout_fill(int32_t n_cells, int32_t n_faces, const int32_t* owner_h,
                    const int32_t* neighbour_h, int32_t uniform_pad_pct, int32_t* slice_off_h,
                    int32_t* slice_w_h, int32_t* slot_col_h, int32_t* slot_face_h);
/* Offset compression of slot_col: per (slice, slot) one column offset and
 * a lane mask when all lanes share the offset (INT32_MIN otherwise);
 * entry (s, k) at slice_off[s]/32 + k.  Kernels give identical results with
 * or without it; it removes most of the index traffic on structured
 * numberings.  slot_dm_h holds 2 * n_slots/32 int32: {delta, mask} per
 * entry.  n_uniform_h receives the number of compressed entries.           */
int gbf_layout_compress(int32_t n_slices, const int32_t* slice_off_h, const int32_t* slice_w_h,
                        const int32_t* slot_col_h, int32_t* slot_dm_h, int64_t* n_uniform_h);
/* Mirror table of a uniform-width offset-compressed layout (uniform wo, all
 * entries compressed): for every neighbour-side entry (s, k) the owner-side
 * slot j of the same face in the slice of its owner cell.  *ok = 1 when j is
 * the same for all lanes of every entry (then a symmetric matrix can be
 * stored as its owner-side slots only: 32*wo floats per slice, and the
 * neighbour-side coefficient of lane l is read at owner cell c' = cell +
 * delta, index 32*wo*(c' >> 5) + 32*j + (c' & 31)); *ok = 0 otherwise.
 * slot_mirror_h has n_slots/32 entries.  No reference counterpart (the
 * reference always stores lower and upper, core/ldu_matrix.py:89-100).    */
int gbf_layout_mirror(int32_t n_faces, int32_t n_slices, int32_t uniform_wo, int32_t uniform_wn,
                      const int32_t* slot_face_h, const int32_t* owner_h,
                      const int32_t* slot_dm_h, int8_t* slot_mirror_h, int32_t* ok);
/* DIC wavefront: level(c) = 1 + max level of the cells j < c that c reads in
 * the reference's cell-ordered factorisation (preconditioners.py:124-128).
 * level_ptr_h has room for n_cells + 1 entries, level_cells_h for n_cells. */
int gbf_dic_schedule(int32_t n_cells, int32_t n_faces, const int32_t* owner_h,
                     const int32_t* neighbour_h, int32_t* level_ptr_h,
                     int32_t* level_cells_h, int32_t* n_levels, int32_t* max_level_size);
/* DILU wavefront over faces: level(f) = 1 + max level of the previous faces
 * touching owner[f] or neighbour[f] (preconditioners.py:254-268).
 * level_ptr_h has room for n_faces + 1 entries, level_faces_h for n_faces. */
int gbf_dilu_schedule(int32_t n_cells, int32_t n_faces, const int32_t* owner_h,
                      const int32_t* neighbour_h, int32_t* level_ptr_h,
                      int32_t* level_faces_h, int32_t* n_levels, int32_t* max_level_size);

/* Links of the dataflow triangular sweep (gbf_sweep_flow_f64) over the
 * schedule of gbf_sweep_schedule(reverse, lower_only): items_h = its
 * level_faces (n_items = level_ptr[n_levels]).  Item i writes slot i (the
 * written cell's value after the face); prev_h[2i] (2 * n_items entries)
 * names the slot of that cell's value before it, prev_h[2i+1] the slot of
 * the read cell's value at it (-1: the value on entry), in the sequential
 * face order of preconditioners.py:170-201 / :306-337; cell_last_h
 * (n_cells) each cell's last slot, -1 if none.  GBF_ERR_ARG if the items are
 * not distinct faces or one comes before a face it reads.                 */
int gbf_sweep_flow_links(int32_t n_cells, int32_t n_faces, const int32_t* owner_h,
                         const int32_t* neighbour_h, int32_t reverse, int32_t n_items,
                         const int32_t* items_h, int32_t* prev_h, int32_t* cell_last_h);

/* Links of the dataflow DILU factorisation (gbf_dilu_build_flow_f64) for the
 * schedule level_faces_h of gbf_dilu_schedule: item i (face level_faces[i])
 * writes slots 2i (owner after the face) and 2i+1 (neighbour after it);
 * prev_h[2i], prev_h[2i+1] (2 * n_faces entries) name the slots holding the
 * two cells' values before the face in the sequential face order of
 * preconditioners.py:254-268, -1 for the diagonal; cell_last_h (n_cells)
 * the slot of each cell's last face, -1 if none.  GBF_ERR_ARG if
 * level_faces_h is not a permutation or puts a face before one it reads;
 * n_faces < 2^30.                                                          */
int gbf_dilu_flow_links(int32_t n_cells, int32_t n_faces, const int32_t* owner_h,
                        const int32_t* neighbour_h, const int32_t* level_faces_h,
                        int32_t* prev_h, int32_t* cell_last_h);

/* Per-cell boundary-face lists (ascending face order) for the assembly:
 * owner_b = owner of boundary faces n_internal..n_internal+n_bnd-1; bnd_ptr
 * has n_cells + 1 entries, bnd_face n_bnd (face ids).                      */
int gbf_boundary_lists(int32_t n_cells, int32_t n_internal, int32_t n_bnd,
                       const int32_t* owner_b_h, int32_t* bnd_ptr_h, int32_t* bnd_face_h);

/* Wavefront schedule of the face-ordered triangular sweeps of the full
 * DIC / DILU solves (preconditioners.py:153-201, :290-337): forward
 * (reverse = 0: faces ascending, owner read, neighbour updated) or backward
 * (reverse = 1: faces descending, neighbour read, owner updated);
 * lower_only keeps only faces with owner < neighbour (DIC).  Levels respect
 * read-after-write, write-after-write and write-after-read order, so the
 * sweep is bitwise the sequential one for any face order.  level_ptr_h has
 * room for n_faces + 1 entries, level_faces_h for n_faces.                */
int gbf_sweep_schedule(int32_t n_cells, int32_t n_faces, const int32_t* owner_h,
                       const int32_t* neighbour_h, int32_t reverse, int32_t lower_only,
                       int32_t* level_ptr_h, int32_t* level_faces_h, int32_t* n_levels,
                       int32_t* max_level_size);

/* ---- coefficient packing ------------------------------------------------
 * slot_coef[slot] = own_src[face] on owner-side slots, nei_src[face] on
 * neighbour-side slots, 0 on padding.  Ax packs (lower, upper); the
 * transposed product and the transposed matrix pack (upper, lower). */
int gbf_pack_f64(const gbf_layout* L, const double* own_src, const double* nei_src,
                 double* slot_coef, void* stream);
int gbf_pack_f32(const gbf_layout* L, const float* own_src, const float* nei_src,
                 float* slot_coef, void* stream);
/* Same, converting FP64 sources to an FP32 packed copy (mixed solver). */
int gbf_pack_f64_to_f32(const gbf_layout* L, const double* own_src, const double* nei_src,
                        float* slot_coef, void* stream);

/* Owner-side half of a symmetric FP64 matrix as FP32 (mixed solver): slot
 * (s, j < wo) of the layout goes to coef_own[32*wo*s + 32*j + lane].  Every
 * face's lower and upper are compared bit for bit; *differs (a DEVICE int32,
 * zeroed by this call) becomes 1 if any pair differs, in which case the half
 * storage does not represent the matrix and the caller keeps the full
 * packing.  Needs a uniform-width layout.  No reference counterpart.      */
int gbf_pack_sym_f64_to_f32(const gbf_layout* L, const double* lower, const double* upper,
                            float* coef_own, int32_t* differs, void* stream);

/* ---- Amul ----------------------------------------------------------------
 * LduMatrix.Ax, core/ldu_matrix.py:172-217 (nei_first = 0, coefficients
 * packed (lower, upper)) and LduMatrix.Ax_T, core/ldu_matrix.py:219-258
 * (nei_first = 1, packed (upper, lower)):
 *   y = (diag*x + S_first) + S_second, each S a sum from 0.0 in ascending
 *   face order, every product and sum rounded once (no FMA): bitwise equal to
 *   the reference.                                                         */
int gbf_amul_f64(const gbf_layout* L, const double* slot_coef, const double* diag,
                 const double* x, double* y, int32_t nei_first, void* stream);
/* float32 matrix, reference semantics: float32 products, float64 sums,
 * float64 y (core/backend.py:58-63 allocates the scatter output in the
 * float64 default dtype).                                                  */
int gbf_amul_f32_f64out(const gbf_layout* L, const float* slot_coef, const float* diag,
                        const float* x, double* y, int32_t nei_first, void* stream);
/* all-float Amul (float products and sums); no reference counterpart: the
 * inner operator of the mixed-precision solver.                            */
int gbf_amul_f32(const gbf_layout* L, const float* slot_coef, const float* diag,
                 const float* x, float* y, int32_t nei_first, void* stream);
/* gbf_amul_f32 of a symmetric matrix stored as its owner-side half
 * (gbf_pack_sym_f64_to_f32); the neighbour-side coefficients are read from
 * the owner cells' slots through L->slot_mirror.  Same products and sums,
 * so the same bits as gbf_amul_f32 on the full packing.  Needs a hex 3+3
 * layout (uniform wo = wn = 3, all entries compressed) with slot_mirror.
 * No reference counterpart.                                                */
int gbf_amul_sym_f32(const gbf_layout* L, const float* coef_own, const float* diag,
                     const float* x, float* y, void* stream);

/* ---- preconditioners -----------------------------------------------------
 * Level-scheduled wavefronts (factorisations, apply_full sweeps and the
 * Gauss-Seidel sweeps below) take `barrier`: device memory of
 * gbf_wavefront_barrier_bytes() bytes, any contents (the call zeroes it).
 * With it the whole schedule runs in one cooperative launch, levels
 * separated by a bounded grid barrier; with NULL (or a device without
 * cooperative launch) one kernel runs per level.  Same bits either way.
 * If a barrier wait runs out (a few seconds) the output is overwritten
 * with NaN and gbf_wavefront_fault reports 1 (it synchronises the stream).
 * Calls must not share one barrier buffer while in flight.                */
size_t gbf_wavefront_barrier_bytes(void);
int gbf_wavefront_fault(const void* barrier, int32_t* fault_h, void* stream);
/* DICPreconditioner._build, solvers/preconditioners.py:88-133: level-
 * scheduled, each cell's subtractions in the reference's face order; then
 * d = clamp(|d|, 1e-30).  slot_coef must be the (lower, upper) packing (the
 * neighbour-side slots carry upper[f]).  level_ptr / level_cells are DEVICE
 * copies of gbf_dic_schedule's output.                                     */
int gbf_dic_build_f64(const gbf_layout* L, const double* slot_coef, const double* diag,
                      const int32_t* level_ptr, const int32_t* level_cells, int32_t n_levels,
                      int32_t max_level_size, double* d_out, void* barrier, void* stream);
/* DILUPreconditioner._build, solvers/preconditioners.py:228-272, per face
 * level; lower/upper in face order.                                        */
int gbf_dilu_build_f64(const gbf_layout* L, const double* lower, const double* upper,
                       const double* diag, const int32_t* level_ptr,
                       const int32_t* level_faces, int32_t n_levels, int32_t max_level_size,
                       double* d_out, void* barrier, void* stream);
/* The same two factorisations as dataflow walks, the same bits: no barrier
 * between levels; every value a step reads sits in a slot that its producer
 * fills, and a step waits only on the slots it reads (bounded waits; on
 * timeout the barrier's fault word is set and d_out is NaN, as for the
 * cooperative level walk).  One cooperative launch plus one output kernel;
 * `barrier` (gbf_wavefront_barrier_bytes) is required.
 * DIC (preconditioners.py:102-133): the cells of gbf_dic_schedule in level
 * order; d_out doubles as the slots.                                       */
int gbf_dic_build_flow_f64(const gbf_layout* L, const double* coef, const double* diag,
                           const int32_t* level_cells, double* d_out, void* barrier,
                           void* stream);
/* DILU (preconditioners.py:228-272): the faces of gbf_dilu_schedule in level
 * order with the links of gbf_dilu_flow_links; slots = device scratch of
 * gbf_dilu_flow_slots_bytes(n_faces) bytes.                                */
size_t gbf_dilu_flow_slots_bytes(int32_t n_faces);
int gbf_dilu_build_flow_f64(const gbf_layout* L, const double* lower, const double* upper,
                            const double* diag, const int32_t* level_faces, const int32_t* prev,
                            const int32_t* cell_last, double* slots, double* d_out,
                            void* barrier, void* stream);
/* DIC/DILU apply(): z = r / d (preconditioners.py:151, :288).               */
/* One triangular sweep of apply_full: for the faces of each level,
 * res[W] -= (coef[f] * res[R]) / d[R] if |d[R]| > 1e-30 (coef in face order:
 * upper for the forward sweeps, upper (DIC) or lower (DILU) backward).     */
int gbf_sweep_f64(const gbf_layout* L, const double* coef, const double* d,
                  const int32_t* level_ptr, const int32_t* level_faces, int32_t n_levels,
                  int32_t max_level_size, int32_t reverse, double* res, void* barrier,
                  void* stream);
/* The same sweep as a dataflow walk (no barrier between levels; the same
 * bits): items = the schedule's level_faces (n_items of them), prev /
 * cell_last from gbf_sweep_flow_links, slots = n_items doubles of device
 * scratch; `barrier` (64 bytes) is required, and a wait that runs out sets
 * its fault word and makes res NaN.                                        */
int gbf_sweep_flow_f64(const gbf_layout* L, const double* coef, const double* d,
                       const int32_t* items, int32_t n_items, const int32_t* prev,
                       const int32_t* cell_last, int32_t reverse, double* res, double* slots,
                       void* barrier, void* stream);
int gbf_diag_apply_f64(int32_t n, const double* r, const double* d, double* z, void* stream);

/* ---- Krylov solvers --------------------------------------------------------
 * Convergence follows ResidualMonitor (solvers/residual.py:112-145): L2 norm
 * each check, |r| < tolerance or |r|/|r0| < rel_tol once iteration >=
 * min_iter; iterations = number of residual checks (len(history)).        */
typedef struct gbf_solve_params {
  double tolerance;
  double rel_tol;
  int32_t max_iter;
  int32_t min_iter;
  int32_t check_every;  /* iterations between host status reads (0 = 32)   */
  int32_t variant;      /* PBiCGStab: 0 = reference omega = (t.z)/(t.t)
                           (pbicgstab.py:210), 1 = standard (t.s)/(t.t).
                           FP64 PCG: 0 = automatic (one cooperative launch
                           for the whole solve up to 2^21 cells, three
                           kernels per iteration above), 1 = three kernels
                           per iteration, 2 = one cooperative launch.
                           Both forms apply the same per-element arithmetic
                           and monitor rules; their dot products differ in
                           summation order (block count).  A barrier wait
                           of the cooperative form that runs out gives
                           status GBF_DEVICE_TIMEOUT.                      */
} gbf_solve_params;

typedef struct gbf_solve_result {
  int32_t iterations;      /* len(history)                                  */
  int32_t status;          /* GBF_CONVERGED / GBF_BREAKDOWN / GBF_MAX_ITER  */
  double final_residual;
  double initial_residual;
  int32_t inner_iterations;/* mixed solver: low-precision iterations        */
  int32_t outer_updates;   /* mixed solver: FP64 residual replacements      */
  int32_t launches;        /* kernels launched by this call                 */
  int32_t reserved;
} gbf_solve_result;

size_t gbf_pcg_workspace_bytes(int32_t n_cells);
/* PCGSolver._solve, solvers/pcg.py:97-187.  x holds x0 on entry and the
 * solution on return.  precond_d = factorised DIC/DILU diagonal (z = r/d) or
 * NULL for "none".  history (device, max_iter + 1 doubles) receives |r| per
 * check.                                                                   */
int gbf_pcg_solve_f64(const gbf_layout* L, const double* slot_coef, const double* diag,
                      const double* precond_d, const double* b, double* x, double* history,
                      const gbf_solve_params* P, gbf_solve_result* R, void* workspace,
                      size_t workspace_bytes, void* stream);

/* No counterpart in the reference.  Same solve as gbf_pcg_solve_f64 for
 * callers that cannot allocate device memory when they solve (real-time
 * loops that must not touch the allocator, host codes whose device memory
 * is owned by their own pool or a fixed budget, plugin hosts that offer no
 * allocator): the scratch comes from one file-scope device array of 32.1 MiB
 * instead of a workspace, so at most 1,048,576 cells (larger systems return
 * GBF_ERR_ARG).  It always runs three kernels per iteration: P->variant 0
 * and 1 are accepted alike, 2 (single launch required) and anything else
 * return GBF_ERR_ARG.  It cannot run inside a stream capture (it reads its
 * state back to the host between chunks of iterations).  Every call looks
 * up the array's address on the current device, so a cudaDeviceReset
 * between calls is safe.  Calls that overlap on the GPU share the array and
 * race.                                                                    */
int gbf_pcg_solve_f64_noalloc(const gbf_layout* L, const double* slot_coef, const double* diag,
                              const double* precond_d, const double* b, double* x,
                              double* history, const gbf_solve_params* P, gbf_solve_result* R,
                              void* stream);

size_t gbf_pbicgstab_workspace_bytes(int32_t n_cells);
/* PBiCGSTABSolver._solve, solvers/pbicgstab.py:103-239 (two residual checks
 * per iteration: on s and on r).  history holds 2*max_iter + 1 doubles.     */
int gbf_pbicgstab_solve_f64(const gbf_layout* L, const double* slot_coef, const double* diag,
                            const double* precond_d, const double* b, double* x,
                            double* history, const gbf_solve_params* P, gbf_solve_result* R,
                            void* workspace, size_t workspace_bytes, void* stream);

/* ---- finite-volume assembly -----------------------------------------------
 * fvm.laplacian, discretisation/operators.py:432-518: for internal faces
 *   c = (D_f * |S_f|) * delta_f, lower = -c/V_P, upper = -c/V_N;
 *   diag = ((0 + sum_own c/V_P) + sum_nei c/V_N) + sum_bnd c_b/V_P,
 * |S| = sqrt(fma(z,z, fma(y,y, x*x))) (ATen's CPU row norm), all in the
 * reference's order: bitwise equal.  d_mode 0: D = d_value; 1: per face
 * d_face[n_faces_total]; 2: per cell d_cell[n_cells] interpolated with
 * weights (LinearInterpolation, interpolation.py:101-145).
 * face_areas is [n_faces_total][3]; delta and weights [n_faces_total].     */
int gbf_laplacian_assemble_f64(const gbf_layout* L, int32_t n_faces_total,
                               const int32_t* owner_all, const int32_t* bnd_ptr,
                               const int32_t* bnd_face, const double* face_areas,
                               const double* delta, int32_t d_mode, double d_value,
                               const double* d_face, const double* d_cell, const double* weights,
                               const double* volumes, double* lower, double* upper, double* diag,
                               void* stream);
/* fvm.div with the "Gauss upwind" scheme, operators.py:351-429 (no deferred
 * correction): lower = F-/V_P, upper = F+/V_N,
 * diag = (0 + sum_own (-F+)/V_P) + sum_nei |F-|/V_N.  flux[n_internal].    */
int gbf_div_upwind_assemble_f64(const gbf_layout* L, const double* flux, const double* volumes,
                                double* lower, double* upper, double* diag, void* stream);
/* Linear-interpolation weights |d_N| / (|d_P| + |d_N|) (boundary: 1),
 * discretisation/weights.py:21-95.                                         */
int gbf_centre_weights_f64(int32_t n_internal, int32_t n_faces, const int32_t* owner,
                           const int32_t* neighbour, const double* cell_centres,
                           const double* face_centres, double* weights, void* stream);

/* ---- differentiation -------------------------------------------------------
 * Backward of gbf_laplacian_assemble_f64 for a per-face diffusivity (the
 * reference obtains it from autograd through operators.py:488-517):
 * g_gamma[f] = |S| delta ((g_diag_P - g_lower_f)/V_P + (g_diag_N - g_upper_f)/V_N),
 * boundary faces |S| delta g_diag_P / V_P.                                 */
int gbf_laplacian_grad_gamma_f64(const gbf_layout* L, int32_t n_faces_total,
                                 const int32_t* owner_all, const double* face_areas,
                                 const double* delta, const double* volumes,
                                 const double* g_lower, const double* g_upper,
                                 const double* g_diag, double* g_gamma, void* stream);
/* DifferentiableLinearSolve.backward, differentiable/linear_solver.py:139-149:
 * g_diag = -lam*x, g_lower = -lam[own]*x[nei], g_upper = -lam[nei]*x[own]
 * (bitwise the reference's rounding).                                      */
int gbf_dls_grads_f64(const gbf_layout* L, const double* lam, const double* x, double* g_diag,
                      double* g_lower, double* g_upper, void* stream);
/* Fused adjoint face gradient of A(D) x = b, A from gbf_laplacian_assemble:
 * g_gamma[f] (+)= scale * (-lam^T dA/dD_f x), i.e. the two kernels above in
 * one pass without the per-coefficient gradients.                          */
int gbf_adjoint_face_grad_f64(const gbf_layout* L, int32_t n_faces_total,
                              const int32_t* owner_all, const double* face_areas,
                              const double* delta, const double* volumes, const double* lam,
                              const double* x, double scale, int32_t accumulate,
                              double* g_gamma, void* stream);

/* assemble_pressure_equation, solvers/pressure_equation.py:49-148: the
 * Laplacian of 1/A_p (1/max(|A_p|,1e-30) per cell, linearly interpolated with
 * face_weights[n_faces_total]) without a boundary diagonal term, and the
 * source -div(phiHbyA)/V over internal then boundary faces.  Bitwise the
 * reference's coefficients and source.                                     */
int gbf_pressure_assemble_f64(const gbf_layout* L, int32_t n_faces_total, const int32_t* bnd_ptr,
                              const int32_t* bnd_face, const double* face_areas,
                              const double* delta, const double* face_weights, const double* A_p,
                              const double* volumes, const double* phiHbyA, double* lower,
                              double* upper, double* diag, double* source, void* stream);

/* DifferentiableLaplacian.forward, differentiable/operators.py:421-522: the
 * explicit Laplacian out = div(D grad phi) per unit volume, with the
 * reference's face flux ((D_f (phi_N - phi_P)) |S_f|) delta_f, its per-cell
 * summation order and the boundary term ((D_b |S_b|) delta_b) phi_P.  D as in
 * gbf_laplacian_assemble_f64.  Called with phi := grad_output it is the
 * phi-gradient of backward (:542-567).  Bitwise the reference's results.   */
int gbf_explicit_laplacian_f64(const gbf_layout* L, int32_t n_faces_total,
                               const int32_t* bnd_ptr, const int32_t* bnd_face,
                               const double* face_areas, const double* delta, int32_t d_mode,
                               double d_value, const double* d_face, const double* d_cell,
                               const double* weights, const double* volumes, const double* phi,
                               double* out, void* stream);
/* DifferentiableLaplacian.backward D-gradient, operators.py:570-625:
 * g_face[n_faces_total] per face; if g_cell != NULL also the per-cell
 * mapping (half of each internal face to each side, boundary faces to the
 * owner); if g_sum != NULL the sum over all faces (a 0-d D) in a fixed order.
 * g_face and g_cell are bitwise the reference's; g_sum agrees to rounding. */
int gbf_explicit_laplacian_grad_d_f64(const gbf_layout* L, int32_t n_faces_total,
                                      const int32_t* owner_all, const int32_t* bnd_ptr,
                                      const int32_t* bnd_face, const double* face_areas,
                                      const double* delta, const double* volumes,
                                      const double* phi, const double* g, double* g_face,
                                      double* g_cell, double* g_sum, void* stream);

/* ---- smoothers -------------------------------------------------------------
 * Gauss-Seidel: SmoothSolver's "GaussSeidel" smoother
 * (solvers/smooth_solver.py:134-187; relax = 0: x_c = (b_c - off)/d_c) and
 * GaussSeidelSmoother's sweeps (solvers/smoothers.py:63-149; relax = 1:
 * x_c += omega (new - x_c)).  One sweep in the order of the level schedule
 * from gbf_gs_schedule (device level_ptr / level_cells, plus the host copy
 * of level_ptr that sizes the launches); slot_coef is the (lower, upper)
 * packing; each row sum runs over the cell's faces in ascending face order,
 * so the sweep is bitwise the reference's sequential loop.                 */
int gbf_gs_schedule(int32_t n_cells, int32_t n_faces, const int32_t* owner_h,
                    const int32_t* neighbour_h, int32_t reverse, int32_t* level_ptr_h,
                    int32_t* level_cells_h, int32_t* n_levels, int32_t* max_level_size);
int gbf_gauss_seidel_f64(const gbf_layout* L, const double* slot_coef, const double* diag,
                         const double* b, const int32_t* level_ptr, const int32_t* level_cells,
                         const int32_t* level_ptr_h, int32_t n_levels, double omega,
                         int32_t relax, double* x, void* barrier, void* stream);
/* The same sweep as a dataflow walk (no barrier between levels; the same
 * bits): the cells of gbf_gs_schedule(reverse) in level order, old values
 * read from x, new ones written to `scratch` (n_cells doubles of device
 * memory, not x) and copied back into x at the end.  `barrier` (64 bytes,
 * gbf_wavefront_barrier_bytes) is required; a wait that runs out sets its
 * fault word and x becomes NaN.                                            */
int gbf_gauss_seidel_flow_f64(const gbf_layout* L, const double* coef, const double* diag,
                              const double* b, const int32_t* level_cells, int32_t reverse,
                              double omega, int32_t relax, double* x, double* scratch,
                              void* barrier, void* stream);
/* r = b - A x, A x bitwise LduMatrix.Ax (core/ldu_matrix.py:172-217); the
 * residual of every smoother and of the smoothing solvers.                 */
int gbf_residual_f64(const gbf_layout* L, const double* slot_coef, const double* diag,
                     const double* b, const double* x, double* r, void* stream);
/* x += (omega / max(|diag|, 1e-30)) z (JacobiSmoother, smoothers.py:152-200)
 * or, with diag == NULL, x += omega z (the DIC / DILU Richardson updates,
 * smooth_solver.py:189-232, smoothers.py:203-260).                         */
int gbf_relax_f64(int32_t n, double omega, const double* diag, const double* z, double* x,
                  void* stream);
/* *out (DEVICE) = |r|_2 in a fixed summation order (the residual norm of
 * solvers/residual.py:112-145); workspace of gbf_norm2_workspace_bytes().  */
size_t gbf_norm2_workspace_bytes(void);
int gbf_norm2_f64(int32_t n, const double* r, double* out, void* workspace, void* stream);

/* ---- GAMG ---------------------------------------------------------------------
 * GAMGSolver (solvers/gamg.py:104-585).  Host, once per mesh topology:
 * greedy aggregation in cell order (gamg.py:183-245; f2c[n_cells], the
 * aggregate of each cell) and the coarse faces (gamg.py:249-331; arrays of
 * n_faces entries, *n_cfaces used; face_to_cface = -1 for a face inside an
 * aggregate).  Device, per matrix / V-cycle: restriction by aggregate sums
 * (agg_ptr / agg_cells: each aggregate's fine cells ascending), coarse
 * lower/upper as sums over each coarse face's fine faces in face order
 * (cf_ptr / cf_faces), prolongation x += e[f2c].  Bitwise the reference's. */
int gbf_gamg_aggregate(int32_t n_cells, int32_t n_faces, const int32_t* owner_h,
                       const int32_t* neighbour_h, int32_t n_coarse_target, int32_t* f2c_h,
                       int32_t* n_coarse);
int gbf_gamg_coarse_faces(int32_t n_faces, const int32_t* owner_h, const int32_t* neighbour_h,
                          const int32_t* f2c_h, int32_t* coarse_owner_h,
                          int32_t* coarse_neighbour_h, int32_t* face_to_cface_h,
                          int32_t* n_cfaces);
int gbf_gamg_restrict_f64(int32_t n_coarse, const int32_t* agg_ptr, const int32_t* agg_cells,
                          const double* fine, double* coarse, void* stream);
int gbf_gamg_coarse_coeffs_f64(int32_t n_cfaces, const int32_t* cf_ptr, const int32_t* cf_faces,
                               const double* lower, const double* upper, double* coarse_lower,
                               double* coarse_upper, void* stream);
int gbf_gamg_prolong_add_f64(int32_t n_fine, const int32_t* f2c, const double* e, double* x,
                             void* stream);

/* out = x + a*y (one rounding each; out may alias x or y): the vector
 * updates of PBiCGSolver (solvers/pbicg.py:161-200).                       */
int gbf_xpay_f64(int32_t n, const double* x, double a, const double* y, double* out,
                 void* stream);
/* *out (DEVICE) = a . b in a fixed summation order (torch.dot of the
 * reference solvers); workspace of gbf_norm2_workspace_bytes().            */
int gbf_dot_f64(int32_t n, const double* a, const double* b, double* out, void* workspace,
                void* stream);
/* FvMatrix.relax (core/fv_matrix.py:192-235), in place: diag = diag / a,
 * source = source + ((1 - a) * diag) * field_old with one_minus_a = 1 - a
 * computed by the caller.  True IEEE division (a torch division of a CUDA
 * tensor by a scalar multiplies by the reciprocal instead, which is not the
 * reference's CPU result).                                                  */
int gbf_fv_relax_f64(int32_t n, double a, double one_minus_a, double* diag, double* source,
                     const double* field_old, void* stream);
/* DiagonalSolver (solvers/diagonal.py:55-85): x = b / max(|diag|, 1e-30),
 * r = b - diag*x.                                                          */
int gbf_diagonal_solve_f64(int32_t n, const double* diag, const double* b, double* x, double* r,
                           void* stream);

/* ---- pressure-corrector steps ---------------------------------------------
 * The steps either side of the pressure solve in SIMPLE / PISO, bitwise the
 * reference's (one rounding per operation in its order).  owner is the
 * int32 owner of all n_faces faces, neighbour of the n_internal internal
 * ones; vectors are [n][3]; weights NULL means 0.5 on every face.          */
/* rhie_chow.py:56-78 compute_HbyA: HbyA = H / max(|A_p|, 1e-30).          */
int gbf_hbya_f64(int32_t n_cells, const double* H, const double* A_p, double* HbyA,
                 void* stream);
/* inv[c] = 1 / max(|A_p[c]|, 1e-30): the per-cell inverse diagonal that
 * the Rhie-Chow and face-flux corrections interpolate (rhie_chow.py:182-183,
 * pressure_equation.py:303-304).                                           */
int gbf_inv_abs_clamped_f64(int32_t n, const double* A_p, double* inv, void* stream);
/* rhie_chow.py:81-143 compute_face_flux_HbyA (p == NULL) and :206-250
 * compute_face_flux (p != NULL: plus the Rhie-Chow term of
 * gbf_rhie_chow_f64; inv_A_p from gbf_inv_abs_clamped_f64).                */
int gbf_face_flux_f64(int32_t n_faces, int32_t n_internal, const int32_t* owner,
                      const int32_t* neighbour, const double* HbyA, const double* face_areas,
                      const double* weights, const double* p, const double* inv_A_p,
                      const double* delta, double* phi, void* stream);
/* rhie_chow.py:146-203 rhie_chow_correction (phi_in == NULL: out = the
 * correction (1/A_p)_f (p_P - p_N) |S_f| delta_f, 0 on boundary faces) and
 * pressure_equation.py:269-332 correct_face_flux (phi_in != NULL: out =
 * phi_in + correction on internal faces, phi_in on boundary faces);
 * inv_A_p from gbf_inv_abs_clamped_f64.                                    */
int gbf_rhie_chow_f64(int32_t n_faces, int32_t n_internal, const int32_t* owner,
                      const int32_t* neighbour, const double* p, const double* inv_A_p,
                      const double* face_areas, const double* delta, const double* weights,
                      const double* phi_in, double* out, void* stream);
/* pressure_equation.py:187-266 correct_velocity: U = HbyA - alpha/|A_p|
 * grad(p), grad(p) by Gauss with linearly interpolated face pressure
 * (boundary faces: the owner's), |U| limited to 1e4.  bnd_ptr / bnd_face as
 * gbf_boundary_lists; weights [n_faces].                                   */
int gbf_correct_velocity_f64(const gbf_layout* L, const int32_t* bnd_ptr, const int32_t* bnd_face,
                             const double* face_areas, const double* weights,
                             const double* volumes, const double* p, const double* A_p,
                             const double* HbyA, double alpha, double* U, void* stream);
/* pressure_equation.py:335-377 adjust_phi: *sum (DEVICE) = the boundary
 * flux sum phi[n_internal..n_faces) (deterministic tree order), then
 * gbf_adjust_phi_f64 subtracts *sum / n_boundary from every boundary flux. */
int gbf_boundary_flux_sum_f64(int32_t n_faces, int32_t n_internal, const double* phi,
                              double* sum, void* stream);
int gbf_adjust_phi_f64(int32_t n_faces, int32_t n_internal, const double* sum, double* phi,
                       void* stream);

/* ---- mesh geometry ----------------------------------------------------------
 * FvMesh geometry (mesh/fv_mesh.py:75-148 on mesh/mesh_geometry.py:35-395)
 * of a polyhedral mesh: points [n_points][3]; faces as CSR face_ptr
 * [n_faces + 1] / face_pts (vertex indices, OpenFOAM ordering: normal by
 * the right-hand rule points out of the owner).  Vertex indices must lie in
 * [0, n_points): the caller validates them.                                */
/* Face centres (vertex mean) and area vectors (1/2 sum v_j x v_{j+1}), both
 * [n_faces][3] (mesh_geometry.py:35-108).                                  */
int gbf_face_geometry_f64(int32_t n_faces, const int32_t* face_ptr, const int32_t* face_pts,
                          const double* points, double* face_centres, double* face_areas,
                          void* stream);
/* Host: cell -> face lists in the reference's visiting order (owned faces
 * ascending, then neighboured internal faces ascending as ~face),
 * mesh_geometry.py:191-196.  cell_ptr_h has n_cells + 1 entries,
 * cell_faces_h n_faces + n_internal.                                       */
int gbf_cell_faces(int32_t n_cells, int32_t n_faces, int32_t n_internal, const int32_t* owner_h,
                   const int32_t* neighbour_h, int32_t* cell_ptr_h, int32_t* cell_faces_h);
/* Cell volumes [n_cells] and centres [n_cells][3] by the tet decomposition
 * about the mean of the cell's distinct vertices (mesh_geometry.py:139-254;
 * the mean is taken in ascending vertex order).  *status (a DEVICE int32,
 * zeroed by the call) becomes 1 if a cell has more than 64 distinct
 * vertices; that cell gets NaN.                                            */
int gbf_cell_geometry_f64(int32_t n_cells, const int32_t* cell_ptr, const int32_t* cell_faces,
                          const int32_t* face_ptr, const int32_t* face_pts, const double* points,
                          const double* face_centres, double* volumes, double* cell_centres,
                          int32_t* status, void* stream);
/* Linear interpolation weights and delta coefficients [n_faces]
 * (mesh_geometry.py:262-395): internal faces |d_N|/(|d_P|+|d_N|) and
 * 1/|(C_N - C_P).n_hat|; boundary faces 1 and 0.  owner/neighbour int32.   */
int gbf_face_interp_f64(int32_t n_faces, int32_t n_internal, const int32_t* owner,
                        const int32_t* neighbour, const double* cell_centres,
                        const double* face_centres, const double* face_areas, double* weights,
                        double* delta, void* stream);

/* ---- mixed precision -------------------------------------------------------
 * No reference counterpart (FP32 inner iterations, FP64 outer accuracy): PCG whose
 * Krylov recurrence, Amul (coef32 = FP32 packing of the FP64 matrix; with
 * coef32_sym = 1 the owner-side half of a symmetric matrix from
 * gbf_pack_sym_f64_to_f32, which needs L->slot_mirror and a hex 3+3 layout
 * and gives the same bits) and diagonal preconditioner run in FP32, with FP64 reliable updates: when the
 * FP32 residual has dropped by `delta` (0 < delta < 1) since the last update
 * or below max(tolerance, rel_tol*|r0|), the FP32 correction is folded into
 * the FP64 x and the residual is replaced by the true b - A64 x (bitwise
 * reference-order FP64 Amul).  Convergence is declared on true residuals
 * only.  precond_d = FP64 factorised DIC/DILU diagonal or NULL.  history
 * receives |r0| and the true |r| of every update (hist_cap entries max).
 * R->iterations = inner iterations + 1, R->outer_updates = FP64 updates.  */
size_t gbf_mixed_pcg_workspace_bytes(int32_t n_cells);
int gbf_mixed_pcg_solve(const gbf_layout* L, const double* coef64, const double* diag64,
                        const float* coef32, int32_t coef32_sym, const double* precond_d,
                        const double* b, double* x, double delta, double* history, int32_t hist_cap,
                        const gbf_solve_params* P, gbf_solve_result* R, void* workspace,
                        size_t workspace_bytes, void* stream);
/* Mixed-precision PBiCGStab: the iteration of gbf_pbicgstab_solve_f64
 * (pbicgstab.py:103-239, the same breakdown tests) with FP32 vectors, Amul
 * and diagonal preconditioner and the same FP64 reliable updates as
 * gbf_mixed_pcg_solve (residual replacement keeping p, r~ and rho).
 * Convergence on true residuals only (the FP64 solver's half-step check on
 * s is not taken).  P->variant bit 0: 0 omega = (t.z)/(t.t) as the
 * reference, 1 the standard (t.s)/(t.t); bits 1-3, the form: 0 automatic
 * (the persistent form up to 2^16 cells, the fused form up to 2^19, the
 * kernels with the plain gather up to 2^22, the staged kernels above), 1 six
 * kernels
 * per iteration (bulk-copy staged Amul on aligned hex layouts), 2 the same
 * with the plain L2 gather Amul, 3 the whole inner loop in one cooperative
 * launch (phases separated by a bounded grid barrier; its dot products sum
 * over its own grid, so it agrees with the kernels to rounding; a barrier
 * wait that runs out gives status GBF_DEVICE_TIMEOUT), 4 three kernels per
 * iteration, one per reduction (the p update folded into the next v = A y,
 * the s / z update into t = A z, the multiplied vector formed at neighbour
 * cells; hex 3+3 layouts, others run form 2).  coef32 = FP32
 * packing of the FP64 matrix; precond_d = FP64 DILU/DIC diagonal or NULL.
 * history / R as for gbf_mixed_pcg_solve.  Replaces PBiCGSTABSolver._solve
 * (solvers/pbicgstab.py:103) for the momentum solve.                        */
size_t gbf_mixed_pbicgstab_workspace_bytes(int32_t n_cells);
int gbf_mixed_pbicgstab_solve(const gbf_layout* L, const double* coef64, const double* diag64,
                              const float* coef32, const double* precond_d, const double* b,
                              double* x, double delta, double* history, int32_t hist_cap,
                              const gbf_solve_params* P, gbf_solve_result* R, void* workspace,
                              size_t workspace_bytes, void* stream);

/* ---- batching ---------------------------------------------------------------
 * No reference counterpart.  Many independent systems solved together: the
 * layout is their block-diagonal concatenation (each system's cells padded
 * to a multiple of 32), cut into tiles -- contiguous cell ranges of one
 * system.  Systems keep their own scalars, residual checks and convergence;
 * finished systems' tiles return at once.  Same iteration as
 * gbf_mixed_pcg_solve (FP32 inner, FP64 reliable updates).  form: 0 one
 * kernel per phase (one CTA per tile) launched directly, 1 the same with a
 * chunk of iterations captured once in a CUDA graph and replayed, 2 every
 * iteration of every system in one cooperative launch (phases separated by
 * a bounded grid barrier; at most 4096 systems), 3 that launch and its
 * set-up captured in a CUDA graph; + 4: the FP32 Amul runs two threads per
 * cell (one sums the owner-side slots, the other the neighbour-side ones;
 * same Amul bits, the p.Ap partial sums run over other threads).  All forms
 * give the same bits for the same block_size, tiles and threads per cell; a
 * barrier wait of forms 2 and 3 that runs out gives status
 * GBF_DEVICE_TIMEOUT in every system.  R has n_systems entries.
 * block_size: 128, 256 or 512.                                             */
typedef struct gbf_batch {
  int32_t n_systems;
  int32_t n_tiles;
  const int32_t* tile_sys;   /* [n_tiles] system of each tile               */
  const int32_t* tile_begin; /* [n_tiles] first cell                        */
  const int32_t* tile_end;   /* [n_tiles] one past the last cell            */
  const int32_t* sys_tile0;  /* [n_systems + 1] tiles of system s are
                                sys_tile0[s] .. sys_tile0[s+1]-1            */
} gbf_batch;

size_t gbf_batched_mixed_pcg_workspace_bytes(int32_t n_cells, int32_t n_systems,
                                             int32_t n_tiles);
int gbf_batched_mixed_pcg_solve(const gbf_layout* L, const gbf_batch* B, const double* coef64,
                                const double* diag64, const float* coef32,
                                const double* precond_d, const double* b, double* x,
                                double delta, const gbf_solve_params* P, int32_t block_size,
                                int32_t form, gbf_solve_result* R, void* workspace,
                                size_t workspace_bytes, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GBFOAM_H */
