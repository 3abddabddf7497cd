"""Python face of the CPU oracle (``ldu_oracle.c``) -- TEST INFRASTRUCTURE ONLY.

The oracle restates pyOpenFOAM's linear-solve path on the CPU so that tests,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` can check
the CUDA path against it.  The product package never imports this module.

Routines (reference citations are in ``ldu_oracle.c``):

* ``amul`` / ``amul_T``           -- ``LduMatrix.Ax`` / ``Ax_T``
* ``dic_build`` / ``dilu_build``  -- DIC / DILU factorised diagonals
* ``dic_apply_full`` / ``dilu_apply_full`` -- the full triangular sweeps
* ``pcg`` / ``pbicgstab``         -- the solvers with ``ResidualMonitor`` rules
* ``laplacian`` / ``div_upwind``  -- ``fvm.laplacian`` / ``fvm.div`` assembly
* ``dls_grads``                   -- ``DifferentiableLinearSolve.backward``
* ``pressure_assemble``           -- ``assemble_pressure_equation``
* ``centre_weights``              -- linear-interpolation weights
* ``explicit_laplacian`` / ``explicit_laplacian_grad_d`` /
  ``face_grad_to_cells``          -- ``DifferentiableLaplacian`` forward and
  backward
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "ldu_oracle.c")
_OUT = os.path.join(_HERE, "_build", "liboracle.so")

_lib = None


def build(force: bool = False) -> str:
    """Compile ``ldu_oracle.c`` (gcc, OpenMP, no FP contraction)."""
    if not force and os.path.exists(_OUT) and os.path.getmtime(_OUT) >= os.path.getmtime(_SRC):
        return _OUT
    os.makedirs(os.path.dirname(_OUT), exist_ok=True)
    tmp = _OUT + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", _SRC, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _OUT)
    return _OUT


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _i64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a), dtype=np.int64)


def _f(a, dt=np.float64) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a), dtype=dt)


def amul(owner, neighbour, diag, lower, upper, x, transpose=False, float_accumulate=False):
    """y = A x (or A^T x) in the reference's summation order.

    For float32 inputs the reference accumulates in float64 and returns
    float64; ``float_accumulate=True`` instead gives the all-float variant
    used as the specification of the mixed solver's inner FP32 Amul."""
    dt = np.asarray(diag).dtype
    dt = np.float32 if dt == np.float32 else np.float64
    own, nei = _i64(owner), _i64(neighbour)
    d, lo, up, xx = _f(diag, dt), _f(lower, dt), _f(upper, dt), _f(x, dt)
    n, nf = d.shape[0], nei.shape[0]
    acc = np.float32 if (dt == np.float32 and float_accumulate) else np.float64
    y = np.empty(n, acc)
    w = np.empty(2 * n + 1, acc)
    if dt == np.float64:
        fn = lib().orc_amul_f64
    else:
        fn = lib().orc_amul_f32acc if float_accumulate else lib().orc_amul_f32
    fn(ctypes.c_int64(n), ctypes.c_int64(nf), _p(own), _p(nei), _p(d), _p(lo), _p(up), _p(xx),
       _p(y), ctypes.c_int(1 if transpose else 0), _p(w))
    return y


def amul_T(owner, neighbour, diag, lower, upper, x):
    return amul(owner, neighbour, diag, lower, upper, x, transpose=True)


def dic_build(owner, neighbour, diag, upper):
    own, nei = _i64(owner), _i64(neighbour)
    d0, up = _f(diag), _f(upper)
    n, nf = d0.shape[0], nei.shape[0]
    d = np.empty(n)
    wp = np.empty(n + 1, np.int64)
    wf = np.empty(nf + 1, np.int64)
    lib().orc_dic_build_f64(ctypes.c_int64(n), ctypes.c_int64(nf), _p(own), _p(nei), _p(d0),
                            _p(up), _p(d), _p(wp), _p(wf))
    return d


def dilu_build(owner, neighbour, diag, lower, upper):
    own, nei = _i64(owner), _i64(neighbour)
    d0, lo, up = _f(diag), _f(lower), _f(upper)
    n, nf = d0.shape[0], nei.shape[0]
    d = np.empty(n)
    lib().orc_dilu_build_f64(ctypes.c_int64(n), ctypes.c_int64(nf), _p(own), _p(nei), _p(d0),
                             _p(lo), _p(up), _p(d))
    return d


def dic_apply_full(owner, neighbour, upper, pd, r):
    own, nei = _i64(owner), _i64(neighbour)
    up, pdd, rr = _f(upper), _f(pd), _f(r)
    z = np.empty_like(rr)
    lib().orc_dic_apply_full_f64(ctypes.c_int64(rr.shape[0]), ctypes.c_int64(nei.shape[0]),
                                 _p(own), _p(nei), _p(up), _p(pdd), _p(rr), _p(z))
    return z


def dilu_apply_full(owner, neighbour, lower, upper, pd, r):
    own, nei = _i64(owner), _i64(neighbour)
    lo, up, pdd, rr = _f(lower), _f(upper), _f(pd), _f(r)
    z = np.empty_like(rr)
    lib().orc_dilu_apply_full_f64(ctypes.c_int64(rr.shape[0]), ctypes.c_int64(nei.shape[0]),
                                  _p(own), _p(nei), _p(lo), _p(up), _p(pdd), _p(rr), _p(z))
    return z


@dataclass
class SolveResult:
    x: np.ndarray
    iterations: int
    final_residual: float
    converged: bool
    history: np.ndarray


def _solve(fn, owner, neighbour, diag, lower, upper, b, x0, precond_diag, tolerance, rel_tol,
           max_iter, min_iter, threads, *extra):
    own, nei = _i64(owner), _i64(neighbour)
    d, lo, up, bb = _f(diag), _f(lower), _f(upper), _f(b)
    x = _f(x0).copy()
    pd = None if precond_diag is None else _f(precond_diag)
    hist = np.zeros(2 * max_iter + 4)
    nh = ctypes.c_int(0)
    conv = fn(ctypes.c_int64(d.shape[0]), ctypes.c_int64(nei.shape[0]), _p(own), _p(nei), _p(d),
              _p(lo), _p(up), None if pd is None else _p(pd), _p(bb), _p(x),
              ctypes.c_double(tolerance), ctypes.c_double(rel_tol), ctypes.c_int(max_iter),
              ctypes.c_int(min_iter), ctypes.c_int(threads), _p(hist), ctypes.byref(nh), *extra)
    h = hist[: nh.value].copy()
    return SolveResult(x, nh.value, float(h[-1]) if nh.value else 0.0, bool(conv), h)


def pcg(owner, neighbour, diag, lower, upper, b, x0, precond_diag=None, tolerance=1e-6,
        rel_tol=0.01, max_iter=1000, min_iter=0, threads=1) -> SolveResult:
    """PCG exactly as ``solvers/pcg.py:97-187``; ``precond_diag`` is the
    factorised DIC/DILU diagonal (``None`` = no preconditioner)."""
    return _solve(lib().orc_pcg_f64, owner, neighbour, diag, lower, upper, b, x0, precond_diag,
                  tolerance, rel_tol, max_iter, min_iter, threads)


def pbicgstab(owner, neighbour, diag, lower, upper, b, x0, precond_diag=None, tolerance=1e-6,
              rel_tol=0.01, max_iter=1000, min_iter=0, threads=1,
              omega: str = "reference") -> SolveResult:
    """PBiCGStab exactly as ``solvers/pbicgstab.py:103-239`` (omega =
    (t.z)/(t.t)); ``omega="standard"`` uses (t.s)/(t.t) instead."""
    return _solve(lib().orc_pbicgstab_f64, owner, neighbour, diag, lower, upper, b, x0,
                  precond_diag, tolerance, rel_tol, max_iter, min_iter, threads,
                  ctypes.c_int(1 if omega == "standard" else 0))


def laplacian(n_cells, owner_all, neighbour, face_areas, delta, D_face, volumes):
    """``fvm.laplacian`` coefficients (lower, upper, diag) for per-face D."""
    own, nei = _i64(owner_all), _i64(neighbour)
    fa, dl, D, V = _f(face_areas).reshape(-1, 3), _f(delta), _f(D_face), _f(volumes)
    nint, nfaces = nei.shape[0], own.shape[0]
    lo, up, dg = np.empty(nint), np.empty(nint), np.empty(n_cells)
    w = np.empty(3 * n_cells + 1)
    lib().orc_laplacian_f64(ctypes.c_int64(n_cells), ctypes.c_int64(nint), ctypes.c_int64(nfaces),
                            _p(own), _p(nei), _p(fa), _p(dl), _p(D), _p(V), _p(lo), _p(up),
                            _p(dg), _p(w))
    return lo, up, dg


def div_upwind(n_cells, owner, neighbour, flux, volumes):
    """``fvm.div(phi, U, "Gauss upwind")`` coefficients (lower, upper, diag)."""
    own, nei = _i64(owner), _i64(neighbour)
    F, V = _f(flux), _f(volumes)
    nint = nei.shape[0]
    lo, up, dg = np.empty(nint), np.empty(nint), np.empty(n_cells)
    w = np.empty(2 * n_cells + 1)
    lib().orc_div_upwind_f64(ctypes.c_int64(n_cells), ctypes.c_int64(nint), _p(own), _p(nei),
                             _p(F), _p(V), _p(lo), _p(up), _p(dg), _p(w))
    return lo, up, dg


def dls_grads(owner, neighbour, lam, x):
    own, nei = _i64(owner), _i64(neighbour)
    la, xx = _f(lam), _f(x)
    n, nf = la.shape[0], nei.shape[0]
    gd, gl, gu = np.empty(n), np.empty(nf), np.empty(nf)
    lib().orc_dls_grads_f64(ctypes.c_int64(n), ctypes.c_int64(nf), _p(own), _p(nei), _p(la),
                            _p(xx), _p(gd), _p(gl), _p(gu))
    return gd, gl, gu


def pressure_assemble(n_cells, owner_all, neighbour, face_areas, delta, weights, A_p, volumes,
                      phiHbyA):
    """``assemble_pressure_equation``: (lower, upper, diag, source)."""
    own, nei = _i64(owner_all), _i64(neighbour)
    fa, dl, w, ap, V, ph = (_f(face_areas).reshape(-1, 3), _f(delta), _f(weights), _f(A_p),
                            _f(volumes), _f(phiHbyA))
    nint, nfaces = nei.shape[0], own.shape[0]
    lo, up, dg, src = np.empty(nint), np.empty(nint), np.empty(n_cells), np.empty(n_cells)
    wk = np.empty(3 * n_cells + 1)
    lib().orc_pressure_assemble_f64(ctypes.c_int64(n_cells), ctypes.c_int64(nint),
                                    ctypes.c_int64(nfaces), _p(own), _p(nei), _p(fa), _p(dl),
                                    _p(w), _p(ap), _p(V), _p(ph), _p(lo), _p(up), _p(dg), _p(src),
                                    _p(wk))
    return lo, up, dg, src


def centre_weights(owner_all, neighbour, cell_centres, face_centres):
    own, nei = _i64(owner_all), _i64(neighbour)
    cc, fc = _f(cell_centres).reshape(-1, 3), _f(face_centres).reshape(-1, 3)
    w = np.empty(own.shape[0])
    lib().orc_centre_weights_f64(ctypes.c_int64(nei.shape[0]), ctypes.c_int64(own.shape[0]),
                                 _p(own), _p(nei), _p(cc), _p(fc), _p(w))
    return w


def face_values(owner_all, neighbour, D_cell, weights):
    """``LinearInterpolation.interpolate`` (interpolation.py:101-145):
    w*D_P + (1 - w)*D_N on internal faces, D_P on boundary faces."""
    own, nei = _i64(owner_all), _i64(neighbour)
    D, w = _f(D_cell), _f(weights)
    nint = nei.shape[0]
    out = D[own].copy()
    wi = w[:nint]
    out[:nint] = wi * D[own[:nint]] + (1.0 - wi) * D[nei]
    return out


def explicit_laplacian(n_cells, owner_all, neighbour, face_areas, delta, D_face, volumes, phi):
    """``DifferentiableLaplacian.forward`` for a per-face D (and the
    phi-gradient of its backward, with phi := grad_output)."""
    own, nei = _i64(owner_all), _i64(neighbour)
    fa, dl, D, V, ph = (_f(face_areas).reshape(-1, 3), _f(delta), _f(D_face), _f(volumes),
                        _f(phi))
    out = np.empty(n_cells)
    w = np.empty(3 * n_cells + 1)
    lib().orc_explicit_laplacian_f64(ctypes.c_int64(n_cells), ctypes.c_int64(nei.shape[0]),
                                     ctypes.c_int64(own.shape[0]), _p(own), _p(nei), _p(fa),
                                     _p(dl), _p(D), _p(V), _p(ph), _p(out), _p(w))
    return out


def explicit_laplacian_grad_d(owner_all, neighbour, face_areas, delta, volumes, phi, g):
    own, nei = _i64(owner_all), _i64(neighbour)
    fa, dl, V, ph, gg = (_f(face_areas).reshape(-1, 3), _f(delta), _f(volumes), _f(phi), _f(g))
    out = np.empty(own.shape[0])
    lib().orc_explicit_laplacian_grad_d_f64(ctypes.c_int64(nei.shape[0]),
                                            ctypes.c_int64(own.shape[0]), _p(own), _p(nei),
                                            _p(fa), _p(dl), _p(V), _p(ph), _p(gg), _p(out))
    return out


def face_grad_to_cells(n_cells, owner_all, neighbour, g_face):
    own, nei = _i64(owner_all), _i64(neighbour)
    gf = _f(g_face)
    out = np.empty(n_cells)
    w = np.empty(3 * n_cells + 1)
    lib().orc_face_grad_to_cells_f64(ctypes.c_int64(n_cells), ctypes.c_int64(nei.shape[0]),
                                     ctypes.c_int64(own.shape[0]), _p(own), _p(nei), _p(gf),
                                     _p(out), _p(w))
    return out


def correct_velocity(n_cells, owner_all, neighbour, face_areas, weights, volumes, p, A_p, HbyA,
                     alpha=1.0):
    """``correct_velocity`` (solvers/pressure_equation.py:187-266), serial."""
    own, nei = _i64(owner_all), _i64(neighbour)
    fa, w, V = _f(face_areas).reshape(-1, 3), _f(weights), _f(volumes)
    pp, A, H = _f(p), _f(A_p), _f(HbyA).reshape(-1, 3)
    U = np.empty((n_cells, 3))
    lib().orc_correct_velocity_f64(ctypes.c_int64(n_cells), ctypes.c_int64(nei.shape[0]),
                                   ctypes.c_int64(own.shape[0]), _p(own), _p(nei), _p(fa),
                                   _p(w), _p(V), _p(pp), _p(A), _p(H), ctypes.c_double(alpha),
                                   _p(U))
    return U


def face_flux(owner_all, neighbour, HbyA, face_areas, weights=None, p=None, A_p=None,
              delta=None):
    """``compute_face_flux_HbyA`` (rhie_chow.py:81-133) and, with p,
    ``compute_face_flux`` = that + ``rhie_chow_correction`` (rhie_chow.py:
    136-250); weights None means 0.5."""
    own, nei = _i64(owner_all), _i64(neighbour)
    H, fa = _f(HbyA).reshape(-1, 3), _f(face_areas).reshape(-1, 3)
    w = None if weights is None else _f(weights)
    pp = None if p is None else _f(p)
    A = None if A_p is None else _f(A_p)
    dl = None if delta is None else _f(delta)
    phi = np.empty(own.shape[0])
    lib().orc_face_flux_f64(ctypes.c_int64(nei.shape[0]), ctypes.c_int64(own.shape[0]),
                            _p(own), _p(nei), _p(H), _p(fa), None if w is None else _p(w),
                            None if pp is None else _p(pp), None if A is None else _p(A),
                            None if dl is None else _p(dl), _p(phi))
    return phi


def correct_face_flux(owner_all, neighbour, phi, p, A_p, face_areas, delta, weights):
    """``correct_face_flux`` (solvers/pressure_equation.py:269-332)."""
    own, nei = _i64(owner_all), _i64(neighbour)
    ph, pp, A = _f(phi), _f(p), _f(A_p)
    fa, dl, w = _f(face_areas).reshape(-1, 3), _f(delta), _f(weights)
    out = np.empty(own.shape[0])
    lib().orc_correct_face_flux_f64(ctypes.c_int64(nei.shape[0]), ctypes.c_int64(own.shape[0]),
                                    _p(own), _p(nei), _p(ph), _p(pp), _p(A), _p(fa), _p(dl),
                                    _p(w), _p(out))
    return out


def gauss_seidel(owner, neighbour, diag, lower, upper, b, x0, n_sweeps=1, reverse=False,
                 relax=False, omega=1.0):
    """``n_sweeps`` Gauss-Seidel sweeps from x0 (smooth_solver.py:133-187;
    ``relax``: GaussSeidelSmoother's x_c + omega (new - x_c),
    smoothers.py:63-149); returns x."""
    own, nei = _i64(owner), _i64(neighbour)
    x = _f(x0).copy()
    lib().orc_gauss_seidel_f64(ctypes.c_int64(x.shape[0]), ctypes.c_int64(own.shape[0]),
                               _p(own), _p(nei), _p(_f(diag)), _p(_f(lower)), _p(_f(upper)),
                               _p(_f(b)), ctypes.c_int(n_sweeps), ctypes.c_int(int(reverse)),
                               ctypes.c_int(int(relax)), ctypes.c_double(omega), _p(x))
    return x


def gamg(owner, neighbour, diag, lower, upper, b, x0, n_cycles, n_pre_smooth=2, n_post_smooth=2,
         max_levels=10, min_cells_coarse=10):
    """``n_cycles`` V-cycles of GAMGSolver (solvers/gamg.py:104-585) from x0,
    serial; returns (x, residual norm after each cycle, level cell counts)."""
    own, nei = _i64(owner), _i64(neighbour)
    x = _f(x0).copy()
    hist = np.empty(max(n_cycles, 1))
    sizes = np.empty(max_levels + 1, np.int64)
    nl = ctypes.c_int(0)
    lib().orc_gamg_f64(ctypes.c_int64(x.shape[0]), ctypes.c_int64(own.shape[0]), _p(own),
                       _p(nei), _p(_f(diag)), _p(_f(lower)), _p(_f(upper)), _p(_f(b)), _p(x),
                       ctypes.c_int(n_cycles), ctypes.c_int(n_pre_smooth),
                       ctypes.c_int(n_post_smooth), ctypes.c_int(max_levels),
                       ctypes.c_int(min_cells_coarse), _p(hist), _p(sizes), ctypes.byref(nl))
    return x, hist[:n_cycles], sizes[: nl.value]


def num_threads() -> int:
    return int(lib().orc_num_threads())
