"""ctypes binding of libgbfoam.so (the C ABI declared in include/gbfoam.h).

This is the whole bridge between the Python classes and the CUDA kernels:
torch owns the memory and the stream, the kernels get raw device pointers.
There is no CPU fallback: if the library cannot be loaded, every operation
raises.
"""

from __future__ import annotations

import ctypes
import os
import threading

import torch

from . import build as _build

__all__ = [
    "lib",
    "check",
    "Layout",
    "Batch",
    "SolveParams",
    "SolveResult",
    "ptr",
    "stream_ptr",
    "EXPORTED",
    "GBF_CONVERGED",
    "GBF_BREAKDOWN",
    "GBF_MAX_ITER",
    "GBF_DEVICE_TIMEOUT",
]

GBF_RUNNING, GBF_CONVERGED, GBF_BREAKDOWN, GBF_MAX_ITER, GBF_DEVICE_TIMEOUT = 0, 1, 2, 3, 4

_c_i32 = ctypes.c_int32
_c_i64 = ctypes.c_int64
_c_vp = ctypes.c_void_p
_c_dbl = ctypes.c_double
_c_size = ctypes.c_size_t


class Layout(ctypes.Structure):
    """``gbf_layout``: cell-sliced LDU addressing (device pointers)."""

    _fields_ = [
        ("n_cells", _c_i32),
        ("n_faces", _c_i32),
        ("n_slices", _c_i32),
        ("max_width", _c_i32),
        ("uniform_wo", _c_i32),
        ("uniform_wn", _c_i32),
        ("all_uniform", _c_i32),
        ("reserved", _c_i32),
        ("n_slots", _c_i64),
        ("slice_off", _c_vp),
        ("slice_w", _c_vp),
        ("slot_col", _c_vp),
        ("slot_face", _c_vp),
        ("owner", _c_vp),
        ("neighbour", _c_vp),
        ("slot_dm", _c_vp),
        ("slot_mirror", _c_vp),
    ]


class SolveParams(ctypes.Structure):
    _fields_ = [
        ("tolerance", _c_dbl),
        ("rel_tol", _c_dbl),
        ("max_iter", _c_i32),
        ("min_iter", _c_i32),
        ("check_every", _c_i32),
        ("variant", _c_i32),
    ]


class SolveResult(ctypes.Structure):
    _fields_ = [
        ("iterations", _c_i32),
        ("status", _c_i32),
        ("final_residual", _c_dbl),
        ("initial_residual", _c_dbl),
        ("inner_iterations", _c_i32),
        ("outer_updates", _c_i32),
        ("launches", _c_i32),
        ("reserved", _c_i32),
    ]


class Batch(ctypes.Structure):
    """``gbf_batch``: tile map of a block-diagonal batch (device pointers)."""

    _fields_ = [
        ("n_systems", _c_i32),
        ("n_tiles", _c_i32),
        ("tile_sys", _c_vp),
        ("tile_begin", _c_vp),
        ("tile_end", _c_vp),
        ("sys_tile0", _c_vp),
    ]


_P = ctypes.POINTER
_L = _P(Layout)

# name -> (restype, argtypes); the complete exported surface of gbfoam.h
EXPORTED: dict[str, tuple] = {
    "gbf_last_error": (ctypes.c_char_p, []),
    "gbf_version": (ctypes.c_int, []),
    "gbf_device_sm_count": (ctypes.c_int, [_P(_c_i32)]),
    "gbf_selftest_bounded_waits": (ctypes.c_int, [_c_vp]),
    "gbf_timing_enable": (ctypes.c_int, [_c_i32, _c_i32]),
    "gbf_timing_read": (ctypes.c_int, [_c_i32, _P(_c_i32), _P(_c_dbl)]),
    "gbf_layout_plan": (ctypes.c_int, [_c_i32, _c_i32, _c_vp, _c_vp, _c_i32, _P(_c_i32),
                                       _P(_c_i64), _P(_c_i32), _P(_c_i32)]),
    "gbf_layout_fill": (ctypes.c_int, [_c_i32, _c_i32, _c_vp, _c_vp, _c_i32, _c_vp, _c_vp, _c_vp,
                                       _c_vp]),
    "gbf_layout_compress": (ctypes.c_int, [_c_i32, _c_vp, _c_vp, _c_vp, _c_vp, _P(_c_i64)]),
    "gbf_layout_mirror": (ctypes.c_int, [_c_i32, _c_i32, _c_i32, _c_i32, _c_vp, _c_vp, _c_vp,
                                         _c_vp, _P(_c_i32)]),
    "gbf_pack_sym_f64_to_f32": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_amul_sym_f32": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_fv_relax_f64": (ctypes.c_int, [_c_i32, _c_dbl, _c_dbl, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_xpay_f64": (ctypes.c_int, [_c_i32, _c_vp, _c_dbl, _c_vp, _c_vp, _c_vp]),
    "gbf_dot_f64": (ctypes.c_int, [_c_i32, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_diagonal_solve_f64": (ctypes.c_int, [_c_i32, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_gamg_aggregate": (ctypes.c_int, [_c_i32, _c_i32, _c_vp, _c_vp, _c_i32, _c_vp,
                                          _P(_c_i32)]),
    "gbf_gamg_coarse_faces": (ctypes.c_int, [_c_i32, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp,
                                             _P(_c_i32)]),
    "gbf_gamg_restrict_f64": (ctypes.c_int, [_c_i32, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_gamg_coarse_coeffs_f64": (ctypes.c_int, [_c_i32, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp,
                                                  _c_vp, _c_vp]),
    "gbf_gamg_prolong_add_f64": (ctypes.c_int, [_c_i32, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_gs_schedule": (ctypes.c_int, [_c_i32, _c_i32, _c_vp, _c_vp, _c_i32, _c_vp, _c_vp,
                                       _P(_c_i32), _P(_c_i32)]),
    "gbf_gauss_seidel_f64": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_i32,
                                            _c_dbl, _c_i32, _c_vp, _c_vp, _c_vp]),
    "gbf_residual_f64": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_relax_f64": (ctypes.c_int, [_c_i32, _c_dbl, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_norm2_workspace_bytes": (_c_size, []),
    "gbf_norm2_f64": (ctypes.c_int, [_c_i32, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_hbya_f64": (ctypes.c_int, [_c_i32, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_inv_abs_clamped_f64": (ctypes.c_int, [_c_i32, _c_vp, _c_vp, _c_vp]),
    "gbf_face_flux_f64": (ctypes.c_int, [_c_i32, _c_i32, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp,
                                         _c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_rhie_chow_f64": (ctypes.c_int, [_c_i32, _c_i32, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp,
                                         _c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_correct_velocity_f64": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp,
                                                _c_vp, _c_vp, _c_dbl, _c_vp, _c_vp]),
    "gbf_boundary_flux_sum_f64": (ctypes.c_int, [_c_i32, _c_i32, _c_vp, _c_vp, _c_vp]),
    "gbf_adjust_phi_f64": (ctypes.c_int, [_c_i32, _c_i32, _c_vp, _c_vp, _c_vp]),
    "gbf_face_geometry_f64": (ctypes.c_int, [_c_i32, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_cell_faces": (ctypes.c_int, [_c_i32, _c_i32, _c_i32, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_cell_geometry_f64": (ctypes.c_int, [_c_i32, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp,
                                             _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_face_interp_f64": (ctypes.c_int, [_c_i32, _c_i32, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp,
                                           _c_vp, _c_vp, _c_vp]),
    "gbf_dic_schedule": (ctypes.c_int, [_c_i32, _c_i32, _c_vp, _c_vp, _c_vp, _c_vp, _P(_c_i32), _P(_c_i32)]),
    "gbf_dilu_schedule": (ctypes.c_int, [_c_i32, _c_i32, _c_vp, _c_vp, _c_vp, _c_vp, _P(_c_i32), _P(_c_i32)]),
    "gbf_dilu_flow_links": (ctypes.c_int, [_c_i32, _c_i32, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_sweep_flow_links": (ctypes.c_int, [_c_i32, _c_i32, _c_vp, _c_vp, _c_i32, _c_i32, _c_vp,
                                            _c_vp, _c_vp]),
    "gbf_sweep_schedule": (ctypes.c_int, [_c_i32, _c_i32, _c_vp, _c_vp, _c_i32, _c_i32, _c_vp,
                                          _c_vp, _P(_c_i32), _P(_c_i32)]),
    "gbf_sweep_f64": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp, _c_i32, _c_i32, _c_i32,
                                     _c_vp, _c_vp, _c_vp]),
    "gbf_boundary_lists": (ctypes.c_int, [_c_i32, _c_i32, _c_i32, _c_vp, _c_vp, _c_vp]),
    "gbf_laplacian_assemble_f64": (ctypes.c_int, [_L, _c_i32, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp,
                                                  _c_i32, _c_dbl, _c_vp, _c_vp, _c_vp, _c_vp,
                                                  _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_div_upwind_assemble_f64": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_centre_weights_f64": (ctypes.c_int, [_c_i32, _c_i32, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp,
                                              _c_vp]),
    "gbf_laplacian_grad_gamma_f64": (ctypes.c_int, [_L, _c_i32, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp,
                                                    _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_dls_grads_f64": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_adjoint_face_grad_f64": (ctypes.c_int, [_L, _c_i32, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp,
                                                 _c_vp, _c_dbl, _c_i32, _c_vp, _c_vp]),
    "gbf_pressure_assemble_f64": (ctypes.c_int, [_L, _c_i32, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp,
                                                 _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp,
                                                 _c_vp, _c_vp]),
    "gbf_explicit_laplacian_f64": (ctypes.c_int, [_L, _c_i32, _c_vp, _c_vp, _c_vp, _c_vp, _c_i32,
                                                  _c_dbl, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp,
                                                  _c_vp, _c_vp]),
    "gbf_explicit_laplacian_grad_d_f64": (ctypes.c_int, [_L, _c_i32, _c_vp, _c_vp, _c_vp, _c_vp,
                                                         _c_vp, _c_vp, _c_vp, _c_vp, _c_vp,
                                                         _c_vp, _c_vp, _c_vp]),
    "gbf_stream_fault": (ctypes.c_int, [_c_vp]),
    "gbf_pack_f64": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_pack_f32": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_pack_f64_to_f32": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_amul_f64": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp, _c_i32, _c_vp]),
    "gbf_amul_f32_f64out": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp, _c_i32, _c_vp]),
    "gbf_amul_f32": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp, _c_i32, _c_vp]),
    "gbf_wavefront_barrier_bytes": (_c_size, []),
    "gbf_selftest_wavefront_fault": (ctypes.c_int, [_P(_c_i32)]),
    "gbf_selftest_flow_fault": (ctypes.c_int, [_P(_c_i32)]),
    "gbf_copy_from_host": (ctypes.c_int, [_c_vp, _c_vp, _c_size, _c_vp]),
    "gbf_copy_to_host": (ctypes.c_int, [_c_vp, _c_vp, _c_size, _c_vp]),
    "gbf_wavefront_fault": (ctypes.c_int, [_c_vp, _P(_c_i32), _c_vp]),
    "gbf_dic_build_f64": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp, _c_i32, _c_i32, _c_vp,
                                         _c_vp, _c_vp]),
    "gbf_dilu_build_f64": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_i32, _c_i32,
                                          _c_vp, _c_vp, _c_vp]),
    "gbf_gauss_seidel_flow_f64": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp, _c_i32, _c_dbl,
                                                 _c_i32, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_sweep_flow_f64": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_i32, _c_vp, _c_vp, _c_i32,
                                          _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_dic_build_flow_f64": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_dilu_flow_slots_bytes": (_c_size, [_c_i32]),
    "gbf_dilu_build_flow_f64": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp,
                                               _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_diag_apply_f64": (ctypes.c_int, [_c_i32, _c_vp, _c_vp, _c_vp, _c_vp]),
    "gbf_pcg_workspace_bytes": (_c_size, [_c_i32]),
    "gbf_pcg_solve_f64": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp,
                                         _P(SolveParams), _P(SolveResult), _c_vp, _c_size, _c_vp]),
    "gbf_pcg_solve_f64_noalloc": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp,
                                                 _P(SolveParams), _P(SolveResult), _c_vp]),
    "gbf_mixed_pcg_workspace_bytes": (_c_size, [_c_i32]),
    "gbf_mixed_pcg_solve": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_i32, _c_vp, _c_vp, _c_vp,
                                           _c_dbl, _c_vp, _c_i32, _P(SolveParams),
                                           _P(SolveResult), _c_vp, _c_size, _c_vp]),
    "gbf_mixed_pbicgstab_workspace_bytes": (_c_size, [_c_i32]),
    "gbf_mixed_pbicgstab_solve": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp,
                                                 _c_dbl, _c_vp, _c_i32, _P(SolveParams),
                                                 _P(SolveResult), _c_vp, _c_size, _c_vp]),
    "gbf_batched_mixed_pcg_workspace_bytes": (_c_size, [_c_i32, _c_i32, _c_i32]),
    "gbf_batched_mixed_pcg_solve": (ctypes.c_int, [_L, _P(Batch), _c_vp, _c_vp, _c_vp, _c_vp,
                                                   _c_vp, _c_vp, _c_dbl, _P(SolveParams), _c_i32,
                                                   _c_i32, _c_vp, _c_vp, _c_size, _c_vp]),
    "gbf_pbicgstab_workspace_bytes": (_c_size, [_c_i32]),
    "gbf_pbicgstab_solve_f64": (ctypes.c_int, [_L, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp, _c_vp,
                                               _P(SolveParams), _P(SolveResult), _c_vp, _c_size,
                                               _c_vp]),
}

_lock = threading.Lock()
_handle = None


def lib() -> ctypes.CDLL:
    """Load (building first if needed) libgbfoam.so."""
    global _handle
    if _handle is None:
        with _lock:
            if _handle is None:
                path = _build.LIB_PATH
                if not os.path.exists(path) or os.environ.get("GBFOAM_REBUILD"):
                    path = _build.build()
                h = ctypes.CDLL(path)
                for name, (res, args) in EXPORTED.items():
                    fn = getattr(h, name)
                    fn.restype = res
                    fn.argtypes = args
                _handle = h
    return _handle


class GbfError(RuntimeError):
    """A libgbfoam entry point returned a non-zero status."""


def check(rc: int, what: str = "") -> None:
    if rc != 0:
        msg = lib().gbf_last_error().decode(errors="replace")
        raise GbfError(f"{what or 'libgbfoam'} failed (status {rc}): {msg}")


def ptr(t: torch.Tensor | None) -> int | None:
    """Raw device pointer of a contiguous tensor (None passes NULL)."""
    if t is None:
        return None
    return t.data_ptr()


def stream_ptr(device: torch.device) -> int:
    """cudaStream_t of torch's current stream on ``device``."""
    return torch.cuda.current_stream(device).cuda_stream


def wavefront_barrier(device) -> torch.Tensor:
    """Device memory for the grid barrier of one cooperative wavefront call
    (gbf_wavefront_barrier_bytes; the call zeroes it)."""
    return torch.empty(int(lib().gbf_wavefront_barrier_bytes()), dtype=torch.uint8,
                       device=device)


def check_wavefront(barrier, what: str, device) -> None:
    """Raises if the cooperative wavefront call that used `barrier` gave up
    on a grid-barrier wait (synchronises the stream)."""
    fault = ctypes.c_int32(0)
    check(lib().gbf_wavefront_fault(barrier.data_ptr(), ctypes.byref(fault), stream_ptr(device)),
          "gbf_wavefront_fault")
    if fault.value:
        raise RuntimeError(f"{what}: a grid-barrier wait ran out; the result is invalid")
