/*
 * ldu_oracle.c -- CPU restatement of pyOpenFOAM's linear-solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the parity tests,
 * the smoke check and the benchmark's CPU-baseline leg compare the CUDA path
 * against.  Nothing in the product package links or calls it.
 *
 * Every routine restates one reference routine, cited by file:line of the
 * reference project (alanZee/pyOpenFOAM, src/pyfoam/...).  Arithmetic is IEEE
 * double (or float) with one rounding per source-level operation, exactly as
 * the reference's element-wise torch ops round: the file must be compiled
 * with -ffp-contract=off so that no multiply-add is fused.
 *
 * Two execution modes:
 *   - serial   : the reference's own face-ordered scatter / sequential loops;
 *                used for parity (bitwise where the reference is
 *                deterministic);
 *   - threaded : OpenMP over cells with per-cell gathers in ascending face
 *                order (bitwise identical Amul) and OpenMP reductions for
 *                dot products (order differs, as torch's threaded dot does);
 *                used only to time the CPU baseline.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef int64_t idx_t;

/* ------------------------------------------------------------------------ */
/* Amul: core/ldu_matrix.py:172-217 (Ax) and :219-258 (Ax_T)                 */
/* y = diag*x;  y = y + scatter_add(lower*x[nei], owner);                    */
/*              y = y + scatter_add(upper*x[own], neighbour)                 */
/* scatter_add (core/backend.py:34-64) starts from zeros and adds in face    */
/* order.                                                                    */
/* ------------------------------------------------------------------------ */
#define DEFINE_AMUL_SERIAL(T, A, SUF)                                           \
  void orc_amul_##SUF(idx_t n, idx_t nf, const idx_t* own, const idx_t* nei,   \
                      const T* diag, const T* lower, const T* upper,           \
                      const T* x, A* y, int transpose, A* work) {              \
    A* s1 = work;                                                              \
    A* s2 = work + n;                                                          \
    for (idx_t c = 0; c < n; ++c) { T t = diag[c] * x[c]; y[c] = (A)t; }      \
    if (nf <= 0) return;                                                       \
    for (idx_t c = 0; c < n; ++c) { s1[c] = (A)0; s2[c] = (A)0; }             \
    if (!transpose) {                                                          \
      for (idx_t f = 0; f < nf; ++f) { T t = lower[f] * x[nei[f]]; s1[own[f]] = s1[own[f]] + (A)t; } \
      for (idx_t f = 0; f < nf; ++f) { T t = upper[f] * x[own[f]]; s2[nei[f]] = s2[nei[f]] + (A)t; } \
    } else {                                                                   \
      for (idx_t f = 0; f < nf; ++f) { T t = lower[f] * x[own[f]]; s1[nei[f]] = s1[nei[f]] + (A)t; } \
      for (idx_t f = 0; f < nf; ++f) { T t = upper[f] * x[nei[f]]; s2[own[f]] = s2[own[f]] + (A)t; } \
    }                                                                          \
    for (idx_t c = 0; c < n; ++c) y[c] = y[c] + s1[c];                         \
    for (idx_t c = 0; c < n; ++c) y[c] = y[c] + s2[c];                         \
  }
/* FP64 matrices: everything in double. */
DEFINE_AMUL_SERIAL(double, double, f64)
/* FP32 matrices: the reference's scatter_add allocates its output in the   */
/* global default dtype (float64, core/backend.py:58-63), so the float32     */
/* products are accumulated in double and y comes back as float64.          */
DEFINE_AMUL_SERIAL(float, double, f32)
/* Pure-float variant (float products and float sums); no reference         */
/* counterpart -- it specifies the inner FP32 Amul of the mixed solver.     */
DEFINE_AMUL_SERIAL(float, float, f32acc)

/* Stable per-cell face lists (ascending face order): own_ptr/own_face list  */
/* the faces owned by each cell, nei_ptr/nei_face the faces whose neighbour  */
/* is the cell.  Counting sort, so stable.                                   */
void orc_build_csr(idx_t n, idx_t nf, const idx_t* own, const idx_t* nei,
                   idx_t* own_ptr, idx_t* own_face, idx_t* nei_ptr, idx_t* nei_face) {
  memset(own_ptr, 0, sizeof(idx_t) * (size_t)(n + 1));
  memset(nei_ptr, 0, sizeof(idx_t) * (size_t)(n + 1));
  for (idx_t f = 0; f < nf; ++f) { own_ptr[own[f] + 1]++; nei_ptr[nei[f] + 1]++; }
  for (idx_t c = 0; c < n; ++c) { own_ptr[c + 1] += own_ptr[c]; nei_ptr[c + 1] += nei_ptr[c]; }
  idx_t* co = (idx_t*)malloc(sizeof(idx_t) * (size_t)(n > 0 ? n : 1));
  idx_t* cn = (idx_t*)malloc(sizeof(idx_t) * (size_t)(n > 0 ? n : 1));
  for (idx_t c = 0; c < n; ++c) { co[c] = own_ptr[c]; cn[c] = nei_ptr[c]; }
  for (idx_t f = 0; f < nf; ++f) { own_face[co[own[f]]++] = f; nei_face[cn[nei[f]]++] = f; }
  free(co);
  free(cn);
}

/* Threaded per-cell gather: same per-cell summation order as the scatter.   */
#define DEFINE_AMUL_CSR(T, SUF)                                                \
  void orc_amul_csr_##SUF(idx_t n, idx_t nf, const idx_t* own, const idx_t* nei, \
                          const idx_t* own_ptr, const idx_t* own_face,         \
                          const idx_t* nei_ptr, const idx_t* nei_face,         \
                          const T* diag, const T* lower, const T* upper,       \
                          const T* x, T* y) {                                  \
    _Pragma("omp parallel for schedule(static)")                               \
    for (idx_t c = 0; c < n; ++c) {                                            \
      T yc = diag[c] * x[c];                                                   \
      if (nf > 0) {                                                            \
        T s1 = (T)0, s2 = (T)0;                                                \
        for (idx_t k = own_ptr[c]; k < own_ptr[c + 1]; ++k) {                  \
          idx_t f = own_face[k]; T t = lower[f] * x[nei[f]]; s1 = s1 + t; }    \
        for (idx_t k = nei_ptr[c]; k < nei_ptr[c + 1]; ++k) {                  \
          idx_t f = nei_face[k]; T t = upper[f] * x[own[f]]; s2 = s2 + t; }    \
        yc = yc + s1;                                                          \
        yc = yc + s2;                                                          \
      }                                                                        \
      y[c] = yc;                                                               \
    }                                                                          \
  }
DEFINE_AMUL_CSR(double, f64)
DEFINE_AMUL_CSR(float, f32)

/* ------------------------------------------------------------------------ */
/* DIC factorisation: solvers/preconditioners.py:88-133                      */
/* for cells ascending: for faces f with neighbour==i in face order:         */
/*   j = owner[f], a = upper[f], d_j = current d[j];                         */
/*   if |d_j| > 1e-30: d[i] = d[i] - (a*a)/d_j                               */
/* then d = clamp(|d|, min=1e-30)                                            */
/* ------------------------------------------------------------------------ */
static double clamp_abs(double v) {
  double a = fabs(v);
  return (a < 1e-30) ? 1e-30 : a; /* NaN propagates, as torch.clamp does */
}

void orc_dic_build_f64(idx_t n, idx_t nf, const idx_t* own, const idx_t* nei,
                       const double* diag, const double* upper, double* d,
                       idx_t* nei_ptr, idx_t* nei_face /* work: n+1, nf */) {
  memcpy(d, diag, sizeof(double) * (size_t)n);
  if (nf > 0) {
    /* lower_adj lists in face order (:116-122) */
    memset(nei_ptr, 0, sizeof(idx_t) * (size_t)(n + 1));
    for (idx_t f = 0; f < nf; ++f) nei_ptr[nei[f] + 1]++;
    for (idx_t c = 0; c < n; ++c) nei_ptr[c + 1] += nei_ptr[c];
    idx_t* cur = (idx_t*)malloc(sizeof(idx_t) * (size_t)(n > 0 ? n : 1));
    for (idx_t c = 0; c < n; ++c) cur[c] = nei_ptr[c];
    for (idx_t f = 0; f < nf; ++f) nei_face[cur[nei[f]]++] = f;
    free(cur);
    for (idx_t i = 0; i < n; ++i) {
      for (idx_t k = nei_ptr[i]; k < nei_ptr[i + 1]; ++k) {
        idx_t f = nei_face[k];
        double a = upper[f];
        double dj = d[own[f]];
        if (fabs(dj) > 1e-30) {
          double t = (a * a) / dj;
          d[i] = d[i] - t;
        }
      }
    }
  }
  for (idx_t c = 0; c < n; ++c) d[c] = clamp_abs(d[c]);
}

/* ------------------------------------------------------------------------ */
/* DILU factorisation: solvers/preconditioners.py:228-272                    */
/* for faces ascending: d_p, d_n captured first; d[p] -= l*u/d_n;            */
/* d[n] -= u*l/d_p (each guarded by |.| > 1e-30); then clamp(|d|)            */
/* ------------------------------------------------------------------------ */
void orc_dilu_build_f64(idx_t n, idx_t nf, const idx_t* own, const idx_t* nei,
                        const double* diag, const double* lower, const double* upper,
                        double* d) {
  memcpy(d, diag, sizeof(double) * (size_t)n);
  for (idx_t f = 0; f < nf; ++f) {
    idx_t p = own[f], q = nei[f];
    double l = lower[f], u = upper[f];
    double dp = d[p], dn = d[q];
    if (fabs(dn) > 1e-30) { double t = (l * u) / dn; d[p] = d[p] - t; }
    if (fabs(dp) > 1e-30) { double t = (u * l) / dp; d[q] = d[q] - t; }
  }
  for (idx_t c = 0; c < n; ++c) d[c] = clamp_abs(d[c]);
}

/* ------------------------------------------------------------------------ */
/* Full sweeps: DIC apply_full preconditioners.py:153-201, DILU :290-337     */
/* ------------------------------------------------------------------------ */
void orc_dic_apply_full_f64(idx_t n, idx_t nf, const idx_t* own, const idx_t* nei,
                            const double* upper, const double* pd, const double* r,
                            double* z) {
  memcpy(z, r, sizeof(double) * (size_t)n);
  for (idx_t f = 0; f < nf; ++f) {
    idx_t p = own[f], q = nei[f];
    if (p < q) {
      double dp = pd[p];
      if (fabs(dp) > 1e-30) { double t = upper[f] * z[p]; t = t / dp; z[q] = z[q] - t; }
    }
  }
  for (idx_t c = 0; c < n; ++c) z[c] = z[c] / pd[c];
  for (idx_t f = nf - 1; f >= 0; --f) {
    idx_t p = own[f], q = nei[f];
    if (p < q) {
      double dq = pd[q];
      if (fabs(dq) > 1e-30) { double t = upper[f] * z[q]; t = t / dq; z[p] = z[p] - t; }
    }
  }
}

void orc_dilu_apply_full_f64(idx_t n, idx_t nf, const idx_t* own, const idx_t* nei,
                             const double* lower, const double* upper, const double* pd,
                             const double* r, double* z) {
  memcpy(z, r, sizeof(double) * (size_t)n);
  for (idx_t f = 0; f < nf; ++f) {
    idx_t p = own[f], q = nei[f];
    double dp = pd[p];
    if (fabs(dp) > 1e-30) { double t = upper[f] * z[p]; t = t / dp; z[q] = z[q] - t; }
  }
  for (idx_t c = 0; c < n; ++c) z[c] = z[c] / pd[c];
  for (idx_t f = nf - 1; f >= 0; --f) {
    idx_t p = own[f], q = nei[f];
    double dq = pd[q];
    if (fabs(dq) > 1e-30) { double t = lower[f] * z[q]; t = t / dq; z[p] = z[p] - t; }
  }
}

/* ------------------------------------------------------------------------ */
/* Vector helpers (serial or OpenMP)                                        */
/* ------------------------------------------------------------------------ */
typedef struct {
  idx_t n, nf;
  const idx_t *own, *nei;
  const double *diag, *lower, *upper;
  int threads;                 /* 1 = serial reference order */
  idx_t *own_ptr, *own_face, *nei_ptr, *nei_face; /* threaded Amul lists */
  double* work;                /* 2n for the serial scatter */
} orc_mat;

static void mat_ax(const orc_mat* A, const double* x, double* y) {
  if (A->threads <= 1)
    orc_amul_f64(A->n, A->nf, A->own, A->nei, A->diag, A->lower, A->upper, x, y, 0, A->work);
  else
    orc_amul_csr_f64(A->n, A->nf, A->own, A->nei, A->own_ptr, A->own_face, A->nei_ptr,
                     A->nei_face, A->diag, A->lower, A->upper, x, y);
}

static double vdot(const orc_mat* A, const double* a, const double* b) {
  double s = 0.0;
  idx_t n = A->n;
  if (A->threads <= 1) {
    for (idx_t i = 0; i < n; ++i) s = s + a[i] * b[i];
  } else {
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (idx_t i = 0; i < n; ++i) s = s + a[i] * b[i];
  }
  return s;
}

/* residual.py:112-145 -- ResidualMonitor.update */
typedef struct {
  double tol, rel_tol, res0;
  int min_iter, have0;
  double* hist;
  int n_hist;
} orc_mon;

static int mon_update(orc_mon* m, double res, int iteration) {
  m->hist[m->n_hist++] = res;
  if (!m->have0) { m->res0 = res; m->have0 = 1; }
  if (iteration >= m->min_iter) {
    if (res < m->tol) return 1;
    if (m->res0 > 0.0 && res / m->res0 < m->rel_tol) return 1;
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* PCG: solvers/pcg.py:97-187 (z = r / d_factored when pd != NULL,          */
/* z = r otherwise).  Returns 1 converged, 0 not converged (max iterations  */
/* or breakdown); *n_hist = reported iteration count = len(history).        */
/* ------------------------------------------------------------------------ */
int orc_pcg_f64(idx_t n, idx_t nf, const idx_t* own, const idx_t* nei,
                const double* diag, const double* lower, const double* upper,
                const double* pd, const double* b, double* x, double tol, double rel_tol,
                int max_iter, int min_iter, int threads, double* hist, int* n_hist) {
#ifdef _OPENMP
  if (threads > 1) omp_set_num_threads(threads);
#endif
  orc_mat A = {n, nf, own, nei, diag, lower, upper, threads, 0, 0, 0, 0, 0};
  double* buf = (double*)malloc(sizeof(double) * (size_t)n * 6 + 16);
  double *r = buf, *z = buf + n, *p = buf + 2 * n, *Ap = buf + 3 * n, *w = buf + 4 * n;
  A.work = w;
  if (threads > 1) {
    A.own_ptr = (idx_t*)malloc(sizeof(idx_t) * (size_t)(n + 1));
    A.nei_ptr = (idx_t*)malloc(sizeof(idx_t) * (size_t)(n + 1));
    A.own_face = (idx_t*)malloc(sizeof(idx_t) * (size_t)(nf + 1));
    A.nei_face = (idx_t*)malloc(sizeof(idx_t) * (size_t)(nf + 1));
    orc_build_csr(n, nf, own, nei, A.own_ptr, A.own_face, A.nei_ptr, A.nei_face);
  }
  orc_mon M = {tol, rel_tol, 0.0, min_iter, 0, hist, 0};
  int conv = 0;
  mat_ax(&A, x, Ap);
#pragma omp parallel for if (threads > 1) schedule(static)
  for (idx_t i = 0; i < n; ++i) r[i] = b[i] - Ap[i];
  if (mon_update(&M, sqrt(vdot(&A, r, r)), 0)) { conv = 1; goto done; }
#pragma omp parallel for if (threads > 1) schedule(static)
  for (idx_t i = 0; i < n; ++i) { z[i] = pd ? r[i] / pd[i] : r[i]; p[i] = z[i]; }
  double rz = vdot(&A, r, z);
  for (int it = 1; it <= max_iter; ++it) {
    mat_ax(&A, p, Ap);
    double pAp = vdot(&A, p, Ap);
    if (fabs(pAp) < 1e-30) { conv = 0; goto done; }
    double alpha = rz / pAp;
#pragma omp parallel for if (threads > 1) schedule(static)
    for (idx_t i = 0; i < n; ++i) {
      double t = alpha * p[i]; x[i] = x[i] + t;
      double u = alpha * Ap[i]; r[i] = r[i] - u;
    }
    if (mon_update(&M, sqrt(vdot(&A, r, r)), it)) { conv = 1; goto done; }
#pragma omp parallel for if (threads > 1) schedule(static)
    for (idx_t i = 0; i < n; ++i) z[i] = pd ? r[i] / pd[i] : r[i];
    double rzn = vdot(&A, r, z);
    double beta = rzn / rz;
    rz = rzn;
#pragma omp parallel for if (threads > 1) schedule(static)
    for (idx_t i = 0; i < n; ++i) { double t = beta * p[i]; p[i] = z[i] + t; }
  }
done:
  *n_hist = M.n_hist;
  if (threads > 1) { free(A.own_ptr); free(A.nei_ptr); free(A.own_face); free(A.nei_face); }
  free(buf);
  return conv;
}

/* ------------------------------------------------------------------------ */
/* PBiCGStab: solvers/pbicgstab.py:103-239                                   */
/* ------------------------------------------------------------------------ */
int orc_pbicgstab_f64(idx_t n, idx_t nf, const idx_t* own, const idx_t* nei,
                      const double* diag, const double* lower, const double* upper,
                      const double* pd, const double* b, double* x, double tol,
                      double rel_tol, int max_iter, int min_iter, int threads,
                      double* hist, int* n_hist, int standard_omega) {
#ifdef _OPENMP
  if (threads > 1) omp_set_num_threads(threads);
#endif
  orc_mat A = {n, nf, own, nei, diag, lower, upper, threads, 0, 0, 0, 0, 0};
  double* buf = (double*)malloc(sizeof(double) * (size_t)n * 10 + 16);
  double *r = buf, *rt = buf + n, *p = buf + 2 * n, *v = buf + 3 * n, *y = buf + 4 * n;
  double *s = buf + 5 * n, *z = buf + 6 * n, *t = buf + 7 * n, *w = buf + 8 * n;
  A.work = w;
  if (threads > 1) {
    A.own_ptr = (idx_t*)malloc(sizeof(idx_t) * (size_t)(n + 1));
    A.nei_ptr = (idx_t*)malloc(sizeof(idx_t) * (size_t)(n + 1));
    A.own_face = (idx_t*)malloc(sizeof(idx_t) * (size_t)(nf + 1));
    A.nei_face = (idx_t*)malloc(sizeof(idx_t) * (size_t)(nf + 1));
    orc_build_csr(n, nf, own, nei, A.own_ptr, A.own_face, A.nei_ptr, A.nei_face);
  }
  orc_mon M = {tol, rel_tol, 0.0, min_iter, 0, hist, 0};
  int conv = 0;
  mat_ax(&A, x, v);
#pragma omp parallel for if (threads > 1) schedule(static)
  for (idx_t i = 0; i < n; ++i) r[i] = b[i] - v[i];
  if (mon_update(&M, sqrt(vdot(&A, r, r)), 0)) { conv = 1; goto done; }
  memcpy(rt, r, sizeof(double) * (size_t)n);
  double rho = vdot(&A, rt, r);
  memcpy(p, r, sizeof(double) * (size_t)n);
  memset(v, 0, sizeof(double) * (size_t)n);
  for (int it = 1; it <= max_iter; ++it) {
    if (fabs(rho) < 1e-30) { conv = 0; goto done; }
#pragma omp parallel for if (threads > 1) schedule(static)
    for (idx_t i = 0; i < n; ++i) y[i] = pd ? p[i] / pd[i] : p[i];
    mat_ax(&A, y, v);
    double rtv = vdot(&A, rt, v);
    if (fabs(rtv) < 1e-30) { conv = 0; goto done; }
    double alpha = rho / rtv;
#pragma omp parallel for if (threads > 1) schedule(static)
    for (idx_t i = 0; i < n; ++i) { double q = alpha * v[i]; s[i] = r[i] - q; }
    if (mon_update(&M, sqrt(vdot(&A, s, s)), it)) {
#pragma omp parallel for if (threads > 1) schedule(static)
      for (idx_t i = 0; i < n; ++i) { double q = alpha * y[i]; x[i] = x[i] + q; }
      conv = 1;
      goto done;
    }
#pragma omp parallel for if (threads > 1) schedule(static)
    for (idx_t i = 0; i < n; ++i) z[i] = pd ? s[i] / pd[i] : s[i];
    mat_ax(&A, z, t);
    double tt = vdot(&A, t, t);
    if (fabs(tt) < 1e-30) {
#pragma omp parallel for if (threads > 1) schedule(static)
      for (idx_t i = 0; i < n; ++i) { double q = alpha * y[i]; x[i] = x[i] + q; r[i] = s[i]; }
      if (mon_update(&M, sqrt(vdot(&A, r, r)), it)) { conv = 1; goto done; }
      double rho_new = vdot(&A, rt, r);
      double beta = (rho_new / rho) * alpha;
      rho = rho_new;
#pragma omp parallel for if (threads > 1) schedule(static)
      for (idx_t i = 0; i < n; ++i) { double q = p[i] - v[i]; q = beta * q; p[i] = r[i] + q; }
      continue;
    }
    /* pbicgstab.py:210 uses (t.z); standard_omega selects (t.s) */
    double omega = vdot(&A, t, standard_omega ? s : z) / tt;
#pragma omp parallel for if (threads > 1) schedule(static)
    for (idx_t i = 0; i < n; ++i) {
      double q1 = alpha * y[i];
      double q2 = omega * z[i];
      double xi = x[i] + q1;
      x[i] = xi + q2;
      double q3 = omega * t[i];
      r[i] = s[i] - q3;
    }
    if (mon_update(&M, sqrt(vdot(&A, r, r)), it)) { conv = 1; goto done; }
    double rho_new = vdot(&A, rt, r);
    if (fabs(omega) < 1e-30) { conv = 0; goto done; }
    double beta = (rho_new / rho) * (alpha / omega);
    rho = rho_new;
#pragma omp parallel for if (threads > 1) schedule(static)
    for (idx_t i = 0; i < n; ++i) {
      double q = omega * v[i];
      q = p[i] - q;
      q = beta * q;
      p[i] = r[i] + q;
    }
  }
done:
  *n_hist = M.n_hist;
  if (threads > 1) { free(A.own_ptr); free(A.nei_ptr); free(A.own_face); free(A.nei_face); }
  free(buf);
  return conv;
}

/* ------------------------------------------------------------------------ */
/* fvm.laplacian assembly: discretisation/operators.py:432-518               */
/* |S| = ATen's CPU p=2 norm over a length-3 row, which accumulates with a   */
/* fused multiply-add: sqrt(fma(z,z, fma(y,y, x*x)))                         */
/* c_f = (D_f*|S_f|)*delta_f; lower = -c/V_P; upper = -c/V_N;                */
/* diag = ((0 + sum_own c/V_P) + sum_nei c/V_N) + sum_bnd c_b/V_P            */
/* ------------------------------------------------------------------------ */
static double smag3(const double* a) {
  double x = a[0], y = a[1], z = a[2];
  return sqrt(fma(z, z, fma(y, y, x * x)));
}

void orc_laplacian_f64(idx_t n, idx_t nint, idx_t nfaces, const idx_t* own /* nfaces */,
                       const idx_t* nei /* nint */, const double* areas /* nfaces*3 */,
                       const double* delta /* nfaces */, const double* D /* nfaces */,
                       const double* V /* n */, double* lower, double* upper, double* diag,
                       double* work /* 3n */) {
  double *s1 = work, *s2 = work + n, *s3 = work + 2 * n;
  for (idx_t c = 0; c < n; ++c) { s1[c] = 0.0; s2[c] = 0.0; s3[c] = 0.0; }
  for (idx_t f = 0; f < nint; ++f) {
    double cf = D[f] * smag3(areas + 3 * f);
    cf = cf * delta[f];
    double vp = V[own[f]], vn = V[nei[f]];
    lower[f] = (-cf) / vp;
    upper[f] = (-cf) / vn;
    s1[own[f]] = s1[own[f]] + cf / vp;
  }
  for (idx_t f = 0; f < nint; ++f) {
    double cf = D[f] * smag3(areas + 3 * f);
    cf = cf * delta[f];
    s2[nei[f]] = s2[nei[f]] + cf / V[nei[f]];
  }
  for (idx_t c = 0; c < n; ++c) diag[c] = 0.0 + s1[c];
  for (idx_t c = 0; c < n; ++c) diag[c] = diag[c] + s2[c];
  if (nfaces > nint) {
    for (idx_t f = nint; f < nfaces; ++f) {
      double cb = D[f] * smag3(areas + 3 * f);
      cb = cb * delta[f];
      s3[own[f]] = s3[own[f]] + cb / V[own[f]];
    }
    for (idx_t c = 0; c < n; ++c) diag[c] = diag[c] + s3[c];
  }
}

/* fvm.div, "Gauss upwind": discretisation/operators.py:351-429              */
/* lower = F-/V_P, upper = F+/V_N, diag = (0 + sum_own -F+/V_P)              */
/*                                        + sum_nei |F-|/V_N                 */
void orc_div_upwind_f64(idx_t n, idx_t nint, const idx_t* own, const idx_t* nei,
                        const double* flux, const double* V, double* lower, double* upper,
                        double* diag, double* work /* 2n */) {
  double *s1 = work, *s2 = work + n;
  for (idx_t c = 0; c < n; ++c) { s1[c] = 0.0; s2[c] = 0.0; }
  for (idx_t f = 0; f < nint; ++f) {
    double F = flux[f];
    double fp = (F >= 0.0) ? F : 0.0;
    double fn = (F >= 0.0) ? 0.0 : F;
    lower[f] = fn / V[own[f]];
    upper[f] = fp / V[nei[f]];
    s1[own[f]] = s1[own[f]] + (-fp) / V[own[f]];
    s2[nei[f]] = s2[nei[f]] + fabs(fn) / V[nei[f]];
  }
  for (idx_t c = 0; c < n; ++c) diag[c] = 0.0 + s1[c];
  for (idx_t c = 0; c < n; ++c) diag[c] = diag[c] + s2[c];
}

/* ------------------------------------------------------------------------ */
/* DifferentiableLinearSolve.backward gradients:                             */
/* differentiable/linear_solver.py:139-149                                   */
/* ------------------------------------------------------------------------ */
void orc_dls_grads_f64(idx_t n, idx_t nf, const idx_t* own, const idx_t* nei,
                       const double* lam, const double* x, double* gdiag, double* glower,
                       double* gupper) {
  for (idx_t c = 0; c < n; ++c) gdiag[c] = (-lam[c]) * x[c];
  for (idx_t f = 0; f < nf; ++f) {
    glower[f] = (-lam[own[f]]) * x[nei[f]];
    gupper[f] = (-lam[nei[f]]) * x[own[f]];
  }
}

/* assemble_pressure_equation: solvers/pressure_equation.py:49-148          */
/* inv = 1/max(|A_p|,1e-30); inv_f = w*inv_P + (1-w)*inv_N;                   */
/* fc = (inv_f*|S|)*delta; lower = -fc/V_P; upper = -fc/V_N;                 */
/* diag = (0 + sum_own fc/V_P) + sum_nei fc/V_N;                             */
/* source = (((0 + sum_own -phi) + sum_nei phi) [+ sum_bnd -phi]) / V        */
/* ------------------------------------------------------------------------ */
static double inv_abs(double a) {
  double v = fabs(a);
  return 1.0 / (v < 1e-30 ? 1e-30 : v);
}

void orc_pressure_assemble_f64(idx_t n, idx_t nint, idx_t nfaces, const idx_t* own,
                               const idx_t* nei, const double* areas, const double* delta,
                               const double* w, const double* Ap, const double* V,
                               const double* phi, double* lower, double* upper, double* diag,
                               double* source, double* work /* 3n */) {
  double *s1 = work, *s2 = work + n, *s3 = work + 2 * n;
  for (idx_t c = 0; c < n; ++c) { s1[c] = 0.0; s2[c] = 0.0; s3[c] = 0.0; }
  for (idx_t f = 0; f < nint; ++f) {
    double inv_f = w[f] * inv_abs(Ap[own[f]]) + (1.0 - w[f]) * inv_abs(Ap[nei[f]]);
    double fc = inv_f * smag3(areas + 3 * f);
    fc = fc * delta[f];
    lower[f] = (-fc) / V[own[f]];
    upper[f] = (-fc) / V[nei[f]];
    s1[own[f]] = s1[own[f]] + fc / V[own[f]];
    s2[nei[f]] = s2[nei[f]] + fc / V[nei[f]];
  }
  for (idx_t c = 0; c < n; ++c) diag[c] = (0.0 + s1[c]) + s2[c];
  for (idx_t c = 0; c < n; ++c) { s1[c] = 0.0; s2[c] = 0.0; }
  for (idx_t f = 0; f < nint; ++f) s1[own[f]] = s1[own[f]] + (-phi[f]);
  for (idx_t f = 0; f < nint; ++f) s2[nei[f]] = s2[nei[f]] + phi[f];
  for (idx_t c = 0; c < n; ++c) source[c] = (0.0 + s1[c]) + s2[c];
  if (nfaces > nint) {
    for (idx_t f = nint; f < nfaces; ++f) s3[own[f]] = s3[own[f]] + (-phi[f]);
    for (idx_t c = 0; c < n; ++c) source[c] = source[c] + s3[c];
  }
  for (idx_t c = 0; c < n; ++c) source[c] = source[c] / V[c];
}

/* Linear-interpolation weights: discretisation/weights.py:21-85            */
/* w_f = |f_c - C_N| / (|f_c - C_P| + |f_c - C_N|) on internal faces (the    */
/* denominator replaced by 1 when it is not > 1e-30), 1 on boundary faces.   */
/* ------------------------------------------------------------------------ */
void orc_centre_weights_f64(idx_t nint, idx_t nfaces, const idx_t* own, const idx_t* nei,
                            const double* cc, const double* fc, double* w) {
  for (idx_t f = 0; f < nfaces; ++f) w[f] = 1.0;
  for (idx_t f = 0; f < nint; ++f) {
    double a[3], b[3];
    for (int k = 0; k < 3; ++k) {
      a[k] = fc[3 * f + k] - cc[3 * own[f] + k];
      b[k] = fc[3 * f + k] - cc[3 * nei[f] + k];
    }
    double dp = smag3(a), dn = smag3(b);
    double den = dp + dn;
    w[f] = dn / (den > 1e-30 ? den : 1.0);
  }
}

/* ------------------------------------------------------------------------ */
/* DifferentiableLaplacian (differentiable/operators.py:409-643)             */
/* forward (:421-522): flux_f = ((D_f*(phi_N - phi_P))*|S_f|)*delta_f;       */
/*   lap = ((0 + sum_own flux) + sum_nei (-flux)) [+ sum_bnd               */
/*         ((D_b*|S_b|)*delta_b)*phi_P]  / max(V, 1e-30)                      */
/* D is given per face (the caller resolves scalars / cell values to faces). */
/* The same routine is the phi-gradient of backward (:542-567) with phi := g. */
/* ------------------------------------------------------------------------ */
static double clampv(double v) { return v < 1e-30 ? 1e-30 : v; }

void orc_explicit_laplacian_f64(idx_t n, idx_t nint, idx_t nfaces, const idx_t* own /* nfaces */,
                                const idx_t* nei /* nint */, const double* areas,
                                const double* delta, const double* D, const double* V,
                                const double* phi, double* out, double* work /* 3n */) {
  double *s1 = work, *s2 = work + n, *s3 = work + 2 * n;
  for (idx_t c = 0; c < n; ++c) { s1[c] = 0.0; s2[c] = 0.0; s3[c] = 0.0; }
  for (idx_t f = 0; f < nint; ++f) {
    double fl = D[f] * (phi[nei[f]] - phi[own[f]]);
    fl = fl * smag3(areas + 3 * f);
    fl = fl * delta[f];
    s1[own[f]] = s1[own[f]] + fl;
  }
  for (idx_t f = 0; f < nint; ++f) {
    double fl = D[f] * (phi[nei[f]] - phi[own[f]]);
    fl = fl * smag3(areas + 3 * f);
    fl = fl * delta[f];
    s2[nei[f]] = s2[nei[f]] + (-fl);
  }
  for (idx_t c = 0; c < n; ++c) out[c] = 0.0 + s1[c];
  for (idx_t c = 0; c < n; ++c) out[c] = out[c] + s2[c];
  if (nfaces > nint) {
    for (idx_t f = nint; f < nfaces; ++f) {
      double cb = D[f] * smag3(areas + 3 * f);
      cb = cb * delta[f];
      s3[own[f]] = s3[own[f]] + cb * phi[own[f]];
    }
    for (idx_t c = 0; c < n; ++c) out[c] = out[c] + s3[c];
  }
  for (idx_t c = 0; c < n; ++c) out[c] = out[c] / clampv(V[c]);
}

/* backward, D-gradient per face (:570-600):                                 */
/*   internal: (((g_P/V_P - g_N/V_N)*(phi_N - phi_P))*|S|)*delta             */
/*   boundary: (((g_P/V_P)*phi_P)*|S|)*delta                                 */
void orc_explicit_laplacian_grad_d_f64(idx_t nint, idx_t nfaces, const idx_t* own,
                                       const idx_t* nei, const double* areas,
                                       const double* delta, const double* V, const double* phi,
                                       const double* g, double* gface) {
  for (idx_t f = 0; f < nint; ++f) {
    idx_t p = own[f], q = nei[f];
    double a = g[p] / clampv(V[p]) - g[q] / clampv(V[q]);
    a = a * (phi[q] - phi[p]);
    a = a * smag3(areas + 3 * f);
    gface[f] = a * delta[f];
  }
  for (idx_t f = nint; f < nfaces; ++f) {
    idx_t p = own[f];
    double a = (g[p] / clampv(V[p])) * phi[p];
    a = a * smag3(areas + 3 * f);
    gface[f] = a * delta[f];
  }
}

/* per-cell D (:608-625): ((0 + sum_own 0.5*gf) + sum_nei 0.5*gf)           */
/*                        [+ sum_bnd gf]                                     */
void orc_face_grad_to_cells_f64(idx_t n, idx_t nint, idx_t nfaces, const idx_t* own,
                                const idx_t* nei, const double* gface, double* gcell,
                                double* work /* 3n */) {
  double *s1 = work, *s2 = work + n, *s3 = work + 2 * n;
  for (idx_t c = 0; c < n; ++c) { s1[c] = 0.0; s2[c] = 0.0; s3[c] = 0.0; }
  for (idx_t f = 0; f < nint; ++f) s1[own[f]] = s1[own[f]] + gface[f] * 0.5;
  for (idx_t f = 0; f < nint; ++f) s2[nei[f]] = s2[nei[f]] + gface[f] * 0.5;
  for (idx_t c = 0; c < n; ++c) gcell[c] = 0.0 + s1[c];
  for (idx_t c = 0; c < n; ++c) gcell[c] = gcell[c] + s2[c];
  if (nfaces > nint) {
    for (idx_t f = nint; f < nfaces; ++f) s3[own[f]] = s3[own[f]] + gface[f];
    for (idx_t c = 0; c < n; ++c) gcell[c] = gcell[c] + s3[c];
  }
}

/* ------------------------------------------------------------------------ */
/* Pressure correctors either side of the solve (serial):                    */
/*   correct_velocity, solvers/pressure_equation.py:187-266:                 */
/*     p_f = w p_P + (1-w) p_N; grad = index_add(owner, p_f S_f),            */
/*     index_add(neighbour, -p_f S_f), index_add(owner_b, p_P S_b) (in that  */
/*     order, faces ascending); U = HbyA - (alpha/max(|A|,1e-30)) (grad /    */
/*     max(V,1e-30)); rows with |U| > 1e4 scaled by 1e4/|U|                  */
/*   compute_face_flux_HbyA + rhie_chow_correction, rhie_chow.py:81-250, and */
/*   correct_face_flux, pressure_equation.py:269-332:                        */
/*     rc_f = ((ia_f (p_P - p_N)) |S_f|) delta_f,                            */
/*     ia_f = w/max(|A_P|,1e-30) + (1-w)/max(|A_N|,1e-30)                    */
/* ------------------------------------------------------------------------ */
static double lerp_w(double w, double a, double b) { return w * a + (1.0 - w) * b; }

void orc_correct_velocity_f64(idx_t n, idx_t nint, idx_t nfaces, const idx_t* own /* nfaces */,
                              const idx_t* nei, const double* areas, const double* w,
                              const double* V, const double* p, const double* A,
                              const double* HbyA, double alpha, double* U) {
  double* g = (double*)calloc((size_t)(3 * (n > 0 ? n : 1)), sizeof(double));
  for (idx_t f = 0; f < nint; ++f) {
    const double pf = lerp_w(w[f], p[own[f]], p[nei[f]]);
    for (int q = 0; q < 3; ++q) g[3 * own[f] + q] = g[3 * own[f] + q] + pf * areas[3 * f + q];
  }
  for (idx_t f = 0; f < nint; ++f) {
    const double pf = lerp_w(w[f], p[own[f]], p[nei[f]]);
    for (int q = 0; q < 3; ++q)
      g[3 * nei[f] + q] = g[3 * nei[f] + q] + (-(pf * areas[3 * f + q]));
  }
  for (idx_t f = nint; f < nfaces; ++f) {
    const double pb = p[own[f]];
    for (int q = 0; q < 3; ++q) g[3 * own[f] + q] = g[3 * own[f] + q] + pb * areas[3 * f + q];
  }
  for (idx_t c = 0; c < n; ++c) {
    const double vc = V[c] < 1e-30 ? 1e-30 : V[c];
    const double s = alpha * inv_abs(A[c]);
    double u[3];
    for (int q = 0; q < 3; ++q) u[q] = HbyA[3 * c + q] - s * (g[3 * c + q] / vc);
    double m = smag3(u);
    m = m < 1e-30 ? 1e-30 : m;
    if (m > 1e4) {
      const double r = 1e4 / m;
      for (int q = 0; q < 3; ++q) u[q] = u[q] * r;
    }
    for (int q = 0; q < 3; ++q) U[3 * c + q] = u[q];
  }
  free(g);
}

static double rc_term(idx_t f, const idx_t* own, const idx_t* nei, const double* p,
                      const double* A, const double* areas, const double* delta,
                      const double* w) {
  const double wf = w ? w[f] : 0.5;
  const double ia = lerp_w(wf, inv_abs(A[own[f]]), inv_abs(A[nei[f]]));
  const double dp = p[own[f]] - p[nei[f]];
  return ((ia * dp) * smag3(areas + 3 * f)) * delta[f];
}

/* phi_f = (w HbyA_P + (1-w) HbyA_N) . S_f on internal faces, HbyA_P . S_f on
 * boundary faces (dot = ((0 + x) + y) + z), plus the Rhie-Chow term when p
 * is given (w NULL: 0.5). */
void orc_face_flux_f64(idx_t nint, idx_t nfaces, const idx_t* own, const idx_t* nei,
                       const double* HbyA, const double* areas, const double* w,
                       const double* p, const double* A, const double* delta, double* phi) {
  for (idx_t f = 0; f < nfaces; ++f) {
    double s = 0.0;
    if (f < nint) {
      const double wf = w ? w[f] : 0.5;
      for (int q = 0; q < 3; ++q)
        s = s + lerp_w(wf, HbyA[3 * own[f] + q], HbyA[3 * nei[f] + q]) * areas[3 * f + q];
      if (p) s = s + rc_term(f, own, nei, p, A, areas, delta, w);
    } else {
      for (int q = 0; q < 3; ++q) s = s + HbyA[3 * own[f] + q] * areas[3 * f + q];
      if (p) s = s + 0.0;
    }
    phi[f] = s;
  }
}

/* correct_face_flux: phi_out = phi + rc on internal faces, phi on boundary. */
void orc_correct_face_flux_f64(idx_t nint, idx_t nfaces, const idx_t* own, const idx_t* nei,
                               const double* phi, const double* p, const double* A,
                               const double* areas, const double* delta, const double* w,
                               double* out) {
  for (idx_t f = 0; f < nfaces; ++f)
    out[f] = f < nint ? phi[f] + rc_term(f, own, nei, p, A, areas, delta, w) : phi[f];
}

/* ------------------------------------------------------------------------ */
/* Gauss-Seidel sweeps: SmoothSolver._solve_gauss_seidel,                    */
/* solvers/smooth_solver.py:133-187 (relax = 0), and GaussSeidelSmoother,    */
/* solvers/smoothers.py:63-149 (relax = 1: x_c + omega (new - x_c)).  Cells  */
/* ascending (reverse: descending); a row's off-diagonal sum runs over the   */
/* cell's faces in ascending face order: lower[f] x[nei] where the cell owns */
/* the face, upper[f] x[own] where it is the neighbour.  The per-cell face   */
/* lists are built once per call (counting sort keeps faces ascending).      */
/* ------------------------------------------------------------------------ */
void orc_gauss_seidel_f64(idx_t n, idx_t nf, const idx_t* own, const idx_t* nei,
                          const double* diag, const double* lower, const double* upper,
                          const double* b, int n_sweeps, int reverse, int relax, double omega,
                          double* x) {
  idx_t* ptr = (idx_t*)calloc((size_t)(n + 1), sizeof(idx_t));
  idx_t* fl = (idx_t*)malloc(sizeof(idx_t) * (size_t)(2 * (nf > 0 ? nf : 1)));
  for (idx_t f = 0; f < nf; ++f) { ptr[own[f] + 1]++; ptr[nei[f] + 1]++; }
  for (idx_t c = 0; c < n; ++c) ptr[c + 1] += ptr[c];
  idx_t* cur = (idx_t*)malloc(sizeof(idx_t) * (size_t)(n > 0 ? n : 1));
  for (idx_t c = 0; c < n; ++c) cur[c] = ptr[c];
  for (idx_t f = 0; f < nf; ++f) {
    fl[cur[own[f]]++] = f;
    if (nei[f] != own[f]) fl[cur[nei[f]]++] = f;
  }
  for (int sweep = 0; sweep < n_sweeps; ++sweep) {
    for (idx_t k = 0; k < n; ++k) {
      const idx_t c = reverse ? n - 1 - k : k;
      const double xc = x[c];
      double row = diag[c] * xc;
      for (idx_t i = ptr[c]; i < cur[c]; ++i) {
        const idx_t f = fl[i];
        if (own[f] == c)
          row = row + lower[f] * x[nei[f]];
        else
          row = row + upper[f] * x[own[f]];
      }
      const double off = row - diag[c] * xc;
      const double d = diag[c];
      if (fabs(d) > 1e-30) {
        const double nv = (b[c] - off) / d;
        x[c] = relax ? xc + omega * (nv - xc) : nv;
      }
    }
  }
  free(cur);
  free(fl);
  free(ptr);
}

/* ------------------------------------------------------------------------ */
/* GAMG, solvers/gamg.py:104-585 (serial).                                   */
/*   aggregation (:166-240): adjacency lists in face order (owner gets the   */
/*     neighbour, the neighbour the owner); cells ascending, an unaggregated */
/*     cell seeds a new aggregate and takes its unaggregated neighbours; at  */
/*     the target count the remaining cells join their first aggregated     */
/*     neighbour's aggregate (else aggregate 0);                            */
/*   coarse matrix (:242-335): diag = scatter_add of the fine diagonal; a   */
/*     fine face between two aggregates adds to the coarse face of the      */
/*     pair, numbered at its first occurrence with that face's orientation, */
/*     lower/upper = first value + the others in face order;                */
/*   V-cycle (:440-493): Jacobi x + (1/max(|d|,1e-30)) (b - A x), restrict  */
/*     by scatter_add, coarse correction from zero, injection, 50 sweeps on */
/*     the coarsest level.                                                   */
/* ------------------------------------------------------------------------ */
typedef struct {
  idx_t n, nf;
  idx_t *own, *nei; /* [nf] */
  double *diag, *lower, *upper;
  idx_t* f2c; /* [n], map to the next level (NULL on the coarsest) */
  idx_t n_coarse;
} orc_level;

static idx_t gamg_aggregate(idx_t n, idx_t nf, const idx_t* own, const idx_t* nei,
                            idx_t target, idx_t* f2c) {
  idx_t* ptr = (idx_t*)calloc((size_t)(n + 1), sizeof(idx_t));
  idx_t* adj = (idx_t*)malloc(sizeof(idx_t) * (size_t)(2 * (nf > 0 ? nf : 1)));
  idx_t* cur = (idx_t*)malloc(sizeof(idx_t) * (size_t)(n > 0 ? n : 1));
  for (idx_t f = 0; f < nf; ++f) { ptr[own[f] + 1]++; ptr[nei[f] + 1]++; }
  for (idx_t c = 0; c < n; ++c) ptr[c + 1] += ptr[c];
  for (idx_t c = 0; c < n; ++c) cur[c] = ptr[c];
  for (idx_t f = 0; f < nf; ++f) {
    adj[cur[own[f]]++] = nei[f];
    adj[cur[nei[f]]++] = own[f];
  }
  for (idx_t c = 0; c < n; ++c) f2c[c] = -1;
  idx_t na = 0;
  for (idx_t c = 0; c < n; ++c) {
    if (f2c[c] >= 0) continue;
    const idx_t id = na++;
    f2c[c] = id;
    for (idx_t k = ptr[c]; k < ptr[c + 1]; ++k)
      if (f2c[adj[k]] < 0) f2c[adj[k]] = id;
    if (na >= target) {
      for (idx_t r = 0; r < n; ++r) {
        if (f2c[r] >= 0) continue;
        int assigned = 0;
        for (idx_t k = ptr[r]; k < ptr[r + 1]; ++k)
          if (f2c[adj[k]] >= 0) { f2c[r] = f2c[adj[k]]; assigned = 1; break; }
        if (!assigned) f2c[r] = 0;
      }
      break;
    }
  }
  for (idx_t c = 0; c < n; ++c)
    if (f2c[c] < 0) f2c[c] = 0;
  free(cur);
  free(adj);
  free(ptr);
  return na;
}

/* Coarse level of `fine` under fine->f2c (n_coarse cells).  The pair ->
 * coarse-face map is an open-addressing hash on (min, max). */
static void gamg_coarse(const orc_level* fine, orc_level* c) {
  const idx_t nc = fine->n_coarse;
  c->n = nc;
  c->diag = (double*)calloc((size_t)(nc > 0 ? nc : 1), sizeof(double));
  for (idx_t i = 0; i < fine->n; ++i) c->diag[fine->f2c[i]] = c->diag[fine->f2c[i]] + fine->diag[i];
  idx_t cap = 16;
  while (cap < 4 * (fine->nf + 1)) cap *= 2;
  idx_t* hkey = (idx_t*)malloc(sizeof(idx_t) * (size_t)cap);
  idx_t* hval = (idx_t*)malloc(sizeof(idx_t) * (size_t)cap);
  for (idx_t i = 0; i < cap; ++i) hkey[i] = -1;
  idx_t nfc = 0;
  idx_t m = fine->nf > 0 ? fine->nf : 1;
  c->own = (idx_t*)malloc(sizeof(idx_t) * (size_t)m);
  c->nei = (idx_t*)malloc(sizeof(idx_t) * (size_t)m);
  c->lower = (double*)malloc(sizeof(double) * (size_t)m);
  c->upper = (double*)malloc(sizeof(double) * (size_t)m);
  for (idx_t f = 0; f < fine->nf; ++f) {
    const idx_t cp = fine->f2c[fine->own[f]], cn = fine->f2c[fine->nei[f]];
    if (cp == cn) continue;
    const idx_t lo = cp < cn ? cp : cn, hi = cp < cn ? cn : cp;
    const idx_t key = lo * nc + hi;
    idx_t h = (idx_t)(((uint64_t)key * 0x9E3779B97F4A7C15ull) >> 20) & (cap - 1);
    while (hkey[h] >= 0 && hkey[h] != key) h = (h + 1) & (cap - 1);
    if (hkey[h] == key) {
      const idx_t i = hval[h];
      c->lower[i] = c->lower[i] + fine->lower[f];
      c->upper[i] = c->upper[i] + fine->upper[f];
    } else {
      hkey[h] = key;
      hval[h] = nfc;
      c->own[nfc] = cp;
      c->nei[nfc] = cn;
      c->lower[nfc] = fine->lower[f];
      c->upper[nfc] = fine->upper[f];
      ++nfc;
    }
  }
  c->nf = nfc;
  c->f2c = NULL;
  c->n_coarse = 0;
  free(hkey);
  free(hval);
}

/* r = b - A x on a level (the reference's Ax order), work = 2n doubles. */
static void gamg_residual(const orc_level* L, const double* b, const double* x, double* r,
                          double* y, double* work) {
  orc_amul_f64(L->n, L->nf, L->own, L->nei, L->diag, L->lower, L->upper, x, y, 0, work);
  for (idx_t c = 0; c < L->n; ++c) r[c] = b[c] - y[c];
}

static void gamg_jacobi(const orc_level* L, double* x, const double* b, int n_it) {
  const idx_t n = L->n;
  double* r = (double*)malloc(sizeof(double) * (size_t)(4 * (n > 0 ? n : 1)));
  for (int it = 0; it < n_it; ++it) {
    gamg_residual(L, b, x, r, r + n, r + 2 * n);
    for (idx_t c = 0; c < n; ++c) x[c] = x[c] + inv_abs(L->diag[c]) * r[c];
  }
  free(r);
}

static void gamg_vcycle(const orc_level* lv, int n_levels, int i, double* x, const double* b,
                        int n_pre, int n_post) {
  const orc_level* L = &lv[i];
  if (i == n_levels - 1) {
    gamg_jacobi(L, x, b, 50);
    return;
  }
  gamg_jacobi(L, x, b, n_pre);
  const idx_t n = L->n, nc = L->n_coarse;
  double* r = (double*)malloc(sizeof(double) * (size_t)(4 * (n > 0 ? n : 1)));
  gamg_residual(L, b, x, r, r + n, r + 2 * n);
  double* rc = (double*)calloc((size_t)(2 * (nc > 0 ? nc : 1)), sizeof(double));
  double* ec = rc + nc;
  for (idx_t c = 0; c < n; ++c) rc[L->f2c[c]] = rc[L->f2c[c]] + r[c];
  gamg_vcycle(lv, n_levels, i + 1, ec, rc, n_pre, n_post);
  for (idx_t c = 0; c < n; ++c) x[c] = x[c] + ec[L->f2c[c]];
  free(rc);
  free(r);
  gamg_jacobi(L, x, b, n_post);
}

/* n_cycles V-cycles from x (in place); hist[k] = |b - A x| after cycle k
 * (summed in cell order); level_sizes[0..*n_levels) = the hierarchy's cell
 * counts (at most max_levels + 1 entries). */
void orc_gamg_f64(idx_t n, idx_t nf, const idx_t* own, const idx_t* nei, const double* diag,
                  const double* lower, const double* upper, const double* b, double* x,
                  int n_cycles, int n_pre, int n_post, int max_levels, int min_cells_coarse,
                  double* hist, idx_t* level_sizes, int* n_levels_out) {
  orc_level* lv = (orc_level*)calloc((size_t)(max_levels + 1), sizeof(orc_level));
  lv[0].n = n;
  lv[0].nf = nf;
  lv[0].own = (idx_t*)own;
  lv[0].nei = (idx_t*)nei;
  lv[0].diag = (double*)diag;
  lv[0].lower = (double*)lower;
  lv[0].upper = (double*)upper;
  int nl = 1;
  for (int k = 0; k < max_levels; ++k) {
    orc_level* cur = &lv[nl - 1];
    if (cur->n <= min_cells_coarse) break;
    idx_t target = cur->n / 2;
    if (target < min_cells_coarse) target = min_cells_coarse;
    cur->f2c = (idx_t*)malloc(sizeof(idx_t) * (size_t)(cur->n > 0 ? cur->n : 1));
    cur->n_coarse = gamg_aggregate(cur->n, cur->nf, cur->own, cur->nei, target, cur->f2c);
    if (cur->n_coarse >= cur->n) {
      free(cur->f2c);
      cur->f2c = NULL;
      cur->n_coarse = 0;
      break;
    }
    gamg_coarse(cur, &lv[nl]);
    ++nl;
  }
  double* r = (double*)malloc(sizeof(double) * (size_t)(4 * (n > 0 ? n : 1)));
  for (int k = 0; k < n_cycles; ++k) {
    gamg_vcycle(lv, nl, 0, x, b, n_pre, n_post);
    gamg_residual(&lv[0], b, x, r, r + n, r + 2 * n);
    double ss = 0.0;
    for (idx_t c = 0; c < n; ++c) ss = ss + r[c] * r[c];
    hist[k] = sqrt(ss);
  }
  free(r);
  for (int k = 0; k < nl; ++k) {
    level_sizes[k] = lv[k].n;
    free(lv[k].f2c);
    if (k > 0) {
      free(lv[k].own);
      free(lv[k].nei);
      free(lv[k].diag);
      free(lv[k].lower);
      free(lv[k].upper);
    }
  }
  *n_levels_out = nl;
  free(lv);
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
