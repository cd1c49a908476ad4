"""ctypes binding of ``libpointrix_gb300.so`` (the C ABI in
``include/pointrix_gb300.h``).

The library is built in-tree by :mod:`pointrix_gb300.build`.  There is no
fallback: if the library is missing or fails to load, every operator raises.
"""
from __future__ import annotations

import ctypes as C
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

i32, i64, f32, szt = C.c_int, C.c_int64, C.c_float, C.c_size_t
vp = C.c_void_p

# name -> argtypes (restype int unless listed in _RESTYPES)
SIGNATURES = {
    "pgb_status_string": [i32],
    "pgb_abi_version": [],
    "pgb_compute_sh_forward": [vp, i64, i32, i64, i64, i64, vp, vp, vp],
    "pgb_compute_sh_backward": [vp, i64, i32, i64, i64, i64, vp, vp, vp, vp, vp],
    "pgb_camera_grad_scratch_bytes": [],
    "pgb_project_point_forward": [vp, i64, vp, vp, i32, i32, f32, f32, vp, vp, vp],
    "pgb_project_point_backward": [vp, i64, vp, vp, i32, i32, f32, f32, vp, vp, vp, vp, vp, vp, szt, vp],
    "pgb_compute_cov3d_forward": [vp, vp, vp, i64, vp, vp],
    "pgb_compute_cov3d_backward": [vp, vp, vp, i64, vp, vp, vp, vp],
    "pgb_ewa_project_forward": [vp, vp, vp, vp, vp, vp, i64, i32, i32, vp, vp, vp, vp],
    "pgb_ewa_project_backward": [vp, vp, vp, vp, vp, i64, i32, i32, vp, vp, vp, vp, vp, vp, szt, vp],
    "pgb_sort_scratch_bytes": [i64, i64, i32, i32, C.POINTER(szt), C.POINTER(szt)],
    "pgb_sort_gaussian_begin": [vp, vp, vp, i64, i32, i32, vp, szt, vp, vp],
    "pgb_sort_gaussian_begin_views": [vp, vp, vp, i64, i32, vp, szt, vp, vp],
    "pgb_camera_pose_forward": [vp, vp, vp, vp, vp],
    "pgb_camera_pose_backward": [vp, vp, vp, vp, vp, vp, vp],
    "pgb_sort_gaussian_finish": [vp, vp, vp, i64, i32, i32, i64, vp, szt, vp, szt, vp, vp, vp, vp],
    "pgb_sort_gaussian_finish_capacity": [vp, vp, vp, i64, i32, i32, i64, vp, szt, vp, szt, vp, vp,
                                          vp, vp],
    "pgb_sort_gaussian_noalloc": [vp, vp, vp, vp, i64, i32, i32, vp, i64, vp, C.POINTER(i64), vp],
    "pgb_sort_gaussian_finish_views": [vp, vp, vp, i64, vp, i32, i64, vp, szt, vp, szt, vp, vp, vp, vp],
    "pgb_sort_gaussian_finish_views_capacity": [vp, vp, vp, i64, vp, i32, i64, vp, szt, vp, szt, vp,
                                                vp, vp, vp],
    "pgb_alpha_blending_forward_views": [vp, vp, vp, vp, i64, i32, vp, i64, vp, f32, vp, i32, vp, vp, vp, vp, vp, vp],
    "pgb_alpha_blending_backward_views": [vp, i64, i32, vp, i64, vp, f32, vp, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp],
    "pgb_blend_record_floats": [i32],
    "pgb_blend_grad_record_floats": [i32],
    "pgb_alpha_blending_forward": [vp, vp, vp, vp, i64, i32, vp, i64, vp, f32, i32, i32, vp, vp, vp, vp, vp, vp],
    "pgb_alpha_blending_backward": [vp, i64, i32, vp, i64, vp, f32, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp],
    "pgb_alpha_blending_forward_with_batch": [vp, vp, vp, vp, i64, i32, vp, i64, vp, f32, i32, i32, vp, vp,
                                              vp, vp, vp, vp, i32],
    "pgb_alpha_blending_backward_with_batch": [vp, i64, i32, vp, i64, vp, f32, i32, i32, vp, vp, vp, vp,
                                               vp, vp, vp, vp, vp, vp, i32],
    "pgb_alpha_blending_forward_views_with_batch": [vp, vp, vp, vp, i64, i32, vp, i64, vp, f32, vp, i32,
                                                    vp, vp, vp, vp, vp, vp, i32],
    "pgb_alpha_blending_backward_views_with_batch": [vp, i64, i32, vp, i64, vp, f32, vp, i32, vp, vp, vp,
                                                     vp, vp, vp, vp, vp, vp, vp, i32],
    "pgb_blend_batches": [i32, vp],
    "pgb_blend_pair_census": [vp, i32, i64, vp, i64, vp, i32, i32, vp, vp, vp],
    "pgb_band_tiles": [vp, vp, i64, i32, i32, i32, i32, vp, vp],
    "pgb_tile_counts_views": [vp, vp, i64, vp, i32, i32, vp, vp],
    "pgb_sort_gaussian_finish_views_h": [vp, vp, vp, i64, vp, i32, i32, i64, i32, vp, szt, vp, szt,
                                         vp, vp, vp, vp],
    "pgb_alpha_blending_forward_views_h": [vp, vp, vp, vp, i64, i32, vp, i64, vp, f32, vp, i32, i32,
                                           vp, vp, vp, vp, vp, vp, vp, i32],
    "pgb_alpha_blending_backward_views_h": [vp, i64, i32, vp, i64, vp, f32, vp, i32, i32, vp, vp,
                                            vp, vp, vp, vp, vp, vp, vp, vp, vp, i32],
    "pgb_blend_batches_h": [i32, i32, vp],
    "pgb_band_counts": [vp, vp, i64, i32, i32, vp, i32, vp, vp],
    "pgb_sort_gaussian_rebegin": [vp, vp, i64, vp, szt, vp, vp],
    "pgb_sort_gaussian_finish_band": [vp, vp, vp, i64, i32, i32, i32, i32, i64, vp, szt, vp, szt,
                                      vp, vp, vp, vp],
    "pgb_band_lists_scratch_bytes": [i64, i32],
    "pgb_band_lists_count": [vp, vp, i64, i32, i32, vp, i32, vp, szt, vp, szt, vp, vp],
    "pgb_band_lists_write": [vp, vp, i64, i32, i32, vp, i32, vp, szt, vp, szt, vp, vp, vp],
    "pgb_sort_gaussian_finish_band_list": [vp, vp, i64, i32, i32, i32, i32, i64, vp, i64, vp, szt,
                                           vp, szt, vp, vp, vp, vp],
    "pgb_alpha_blending_forward_band": [vp, vp, vp, vp, i64, i32, vp, i64, vp, f32, i32, i32, i32,
                                        i32, i32, vp, vp, vp, vp, vp, vp, i32],
    "pgb_alpha_blending_backward_band": [vp, i64, i32, vp, i64, vp, f32, i32, i32, i32, i32, vp,
                                         vp, vp, vp, i32, i32, vp, vp, vp, vp, vp, vp, i32],
    "pgb_alpha_blending_forward_pieces": [vp, vp, vp, vp, vp, i32, i64, vp, i64, vp, f32, i32, i32,
                                          vp, vp, vp, vp, vp, vp, i32],
    "pgb_alpha_blending_backward_pieces": [vp, i64, vp, i32, vp, i64, vp, f32, i32, i32, vp, vp, vp,
                                           vp, vp, vp, vp, vp, vp, vp, i32],
}
class AdamSegment(C.Structure):
    """``pgb_adam_segment`` of include/pointrix_gb300.h."""
    _fields_ = [("param", vp), ("grad", vp), ("exp_avg", vp), ("exp_avg_sq", vp),
                ("n", i64), ("lr", f32), ("bias_correction1", f32), ("bias_correction2", f32)]


SIGNATURES["pgb_adam_step"] = [C.POINTER(AdamSegment), i32, f32, f32, f32, vp]
SIGNATURES["pgb_adam_step_device"] = [C.POINTER(AdamSegment), i32, C.c_double, C.c_double, f32, vp,
                                      vp, vp]
SIGNATURES.update({
    "pgb_gaussian_activate_forward": [vp, vp, vp, i64, vp, vp, vp, vp, vp],
    "pgb_gaussian_activate_backward": [vp, vp, vp, i64, vp, vp, vp, vp, vp, vp, vp, vp],
    "pgb_sh_rgb_scratch_floats": [i64],
    "pgb_sh_rgb_forward": [vp, i64, i32, i32, vp, vp, vp, vp],
    "pgb_sh_rgb_backward": [vp, i64, i32, i32, vp, vp, vp, vp, vp, vp, vp, i64, vp],
    "pgb_sh_rgb_views_scratch_floats": [i64],
    "pgb_sh_rgb_views_forward": [vp, i64, i32, i32, vp, vp, i32, vp, vp],
    "pgb_sh_rgb_views_backward": [vp, i64, i32, i32, vp, vp, i32, vp, vp, vp, vp, vp, i64, vp],
    "pgb_l1_l2_loss_scratch_doubles": [i64],
    "pgb_l1_l2_loss_forward": [vp, vp, i64, f32, vp, i64, vp, vp],
    "pgb_l1_l2_loss_backward": [vp, vp, i64, f32, vp, vp, vp],
    "pgb_l1_l2_loss_forward_grad": [vp, vp, i64, f32, vp, i64, vp, vp, vp],
    "pgb_l1_l2_loss_backward_unit": [vp, vp, i64, f32, vp, vp, vp],
    "pgb_densify_accumulate": [vp, i64, vp, f32, f32, vp, vp, vp, vp],
    "pgb_ssim_scratch_doubles": [i32, i32, i32],
    "pgb_preprocess_forward": [vp, vp, vp, i64, vp, vp, i32, i32, f32, f32, vp, vp, vp, vp, vp, vp],
    "pgb_preprocess_backward": [vp, vp, vp, i64, vp, vp, i32, i32, f32, f32, vp, vp, vp, vp, vp, vp,
                                vp, vp, vp, vp, szt, vp],
    "pgb_ssim_forward": [vp, vp, i32, i32, i32, vp, i64, vp, vp],
    "pgb_camera_grad_views_scratch_bytes": [i32],
    "pgb_preprocess_views_forward": [vp, vp, vp, i64, vp, vp, vp, i32, f32, f32, vp, vp, vp, vp,
                                     vp, vp],
    "pgb_preprocess_views_backward": [vp, vp, vp, i64, vp, vp, vp, i32, f32, f32, vp, vp, vp, vp,
                                      vp, vp, vp, vp, vp, vp, szt, vp],
    "pgb_ssim_backward": [vp, vp, i32, i32, i32, vp, vp, vp],
})

_RESTYPES = {"pgb_status_string": C.c_char_p, "pgb_camera_grad_scratch_bytes": szt,
             "pgb_camera_grad_views_scratch_bytes": szt, "pgb_band_lists_scratch_bytes": szt,
             "pgb_ssim_scratch_doubles": i64}


class PgbError(RuntimeError):
    """A non-zero status from the GB300 kernel library."""


def lib():
    """The loaded library (built first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            handle = C.CDLL(str(path))
            for name, args in SIGNATURES.items():
                fn = getattr(handle, name)
                fn.argtypes = args
                fn.restype = _RESTYPES.get(name, i32)
            _lib = handle
    return _lib


def check(status: int, what: str) -> None:
    if status != 0:
        msg = lib().pgb_status_string(status).decode()
        raise PgbError(f"{what}: {msg} (status {status})")


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args), name)
