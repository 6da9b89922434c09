"""Loads libctbb_gb300.so (built in-tree by ctbangbang_gb300.build) and declares
the C ABI of include/ctbb_gb300.h for ctypes.

There is no fallback: if the library is missing the import fails with the
command that builds it, and every compute entry point of the library returns
CTBB_ERR_NO_DEVICE when no CUDA device is present.
"""
import ctypes as C
import os

from .structs import ReconMetadata, ReconParams

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libctbb_gb300.so")

STORAGE_FP32, STORAGE_FP16 = 0, 1

STATUS = {
    0: "CTBB_OK", 1: "CTBB_ERR_ARGUMENT", 2: "CTBB_ERR_CONFIG", 3: "CTBB_ERR_RANGE",
    4: "CTBB_ERR_IO", 5: "CTBB_ERR_CUDA", 6: "CTBB_ERR_NO_DEVICE", 7: "CTBB_ERR_ALLOC",
    8: "CTBB_ERR_STATE",
}

_MR = C.POINTER(ReconMetadata)
_F = C.POINTER(C.c_float)
_VP = C.c_void_p

# name -> (restype, argtypes); every symbol include/ctbb_gb300.h declares.
PROTOTYPES = {
    "ctbb_last_error": (C.c_char_p, []),
    "ctbb_version": (C.c_char_p, []),
    "ctbb_set_stream": (C.c_int, [_VP]),
    "ctbb_configure_recon_params": (C.c_int, [C.c_char_p, C.POINTER(ReconParams)]),
    "ctbb_configure_ct_geom": (C.c_int, [_MR]),
    "ctbb_configure_reconstruction": (C.c_int, [_MR]),
    "ctbb_update_block_info": (C.c_int, [_MR]),
    "ctbb_extract_projections": (C.c_int, [_MR]),
    "ctbb_finish_and_cleanup": (C.c_int, [_MR]),
    "ctbb_n_slices_final": (C.c_int, [_MR]),
    "ctbb_load_filter": (C.c_int, [_MR, _F]),
    "ctbb_ramp_filter_taps": (C.c_int, [C.c_int, C.c_float, C.c_float, C.c_float, _F]),
    "ctbb_adaptive_filter_kk": (C.c_int, [_MR]),
    "ctbb_rebin_filter": (C.c_int, [_MR]),
    "ctbb_backproject": (C.c_int, [_MR]),
    "ctbb_finalize_image_stack": (C.c_int, [_MR]),
    "ctbb_finalize_image_stack_hu": (C.c_int, [_MR, C.c_float]),
    "ctbb_adaptive_filter_device": (C.c_int, [_MR, _VP, _VP]),
    "ctbb_adaptive_filter_device_noalloc": (C.c_int, [_MR, _VP, _VP]),
    "ctbb_rebin_device": (C.c_int, [_MR, _VP, _VP]),
    "ctbb_ramp_filter_device": (C.c_int, [_VP, C.c_size_t, C.c_int, _F]),
    "ctbb_ramp_filter_fp16_device": (C.c_int, [_VP, C.c_size_t, C.c_int, _F, C.c_int, _VP, _VP]),
    "ctbb_set_storage": (C.c_int, [C.c_int]),
    "ctbb_reconstruct_batch_device": (C.c_int, [C.c_int, C.POINTER(_MR), C.POINTER(_VP), C.POINTER(_VP), C.c_float]),
    "ctbb_set_autotune": (C.c_int, [C.c_int]),
    "ctbb_batch_begin": (C.c_int, []),
    "ctbb_batch_add_device": (C.c_int, [_MR, _VP, _VP, C.c_float]),
    "ctbb_batch_run": (C.c_int, []),
    "ctbb_autotune_report": (C.c_int, [C.c_char_p, C.c_size_t]),
    "ctbb_context_set_storage": (C.c_int, [C.c_void_p, C.c_int]),
    "ctbb_backproject_device": (C.c_int, [_MR, _VP, _VP]),
    "ctbb_backproject_fp16_device": (C.c_int, [_MR, _VP, _VP, _VP]),
    "ctbb_scan_workspace_bytes": (C.c_size_t, [_MR]),
    "ctbb_server_create": (C.c_int, [C.c_int, C.c_size_t, C.POINTER(C.c_void_p)]),
    "ctbb_server_submit": (C.c_int, [C.c_void_p, _MR, _F, _F, C.c_float, C.POINTER(C.c_uint64)]),
    "ctbb_server_wait": (C.c_int, [C.c_void_p, C.c_uint64, _VP]),
    "ctbb_server_destroy": (C.c_int, [C.c_void_p]),
    "ctbb_server_configure": (C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    "ctbb_server_passed_count": (C.c_uint64, [C.c_void_p]),
    "ctbb_context_create": (C.c_int, [C.POINTER(C.c_void_p)]),
    "ctbb_context_destroy": (C.c_int, [C.c_void_p]),
    "ctbb_context_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ctbb_context_release_workspace": (C.c_int, [C.c_void_p]),
    "ctbb_context_device_bytes": (C.c_size_t, [C.c_void_p]),
    "ctbb_context_reconstruct_scan_device": (C.c_int, [C.c_void_p, _MR, _VP, _VP, C.c_float]),
    "ctbb_context_reconstruct_scan_host": (C.c_int, [C.c_void_p, _MR, _F, _F, C.c_float]),
    "ctbb_context_reconstruct_scan_file": (C.c_int, [C.c_void_p, _MR, _F, C.c_float]),
    "ctbb_context_reconstruct_device": (C.c_int, [C.c_void_p, _MR, _VP, _VP, C.c_float]),
    "ctbb_context_reconstruct_host": (C.c_int, [C.c_void_p, _MR, _F, _F, C.c_float]),
    "ctbb_write_dicom_series": (C.c_int, [_MR, _F, C.c_int, C.c_float, C.c_char_p]),
    "ctbb_finalize_device": (C.c_int, [_MR, _VP, _VP, C.c_float]),
    "ctbb_reconstruct_device": (C.c_int, [_MR, _VP, _VP, C.c_float]),
    "ctbb_reconstruct_scan_device": (C.c_int, [_MR, _VP, _VP, C.c_float]),
    "ctbb_reconstruct_scan_host": (C.c_int, [_MR, _F, _F, C.c_float]),
    "ctbb_reconstruct_scan_file": (C.c_int, [_MR, _F, C.c_float]),
    "ctbb_reconstruct_host": (C.c_int, [_MR, _F, _F, C.c_float]),
    "ctbb_profile_enable": (C.c_int, [C.c_int]),
    "ctbb_profile_read": (C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_uint64), C.c_int, C.c_int]),
    "ctbb_workspace_bytes": (C.c_size_t, [_MR]),
    "ctbb_release_workspace": (C.c_int, []),
    "ctbb_kernel_launch_count": (C.c_uint64, []),
    "ctbb_struct_layout": (C.c_int, [C.POINTER(C.c_size_t), C.c_int]),
}


class CtbbError(RuntimeError):
    def __init__(self, func, status, text):
        self.status = status
        self.status_name = STATUS.get(status, str(status))
        super().__init__("%s -> %s: %s" % (func, self.status_name, text))


_lib = None


def load():
    """Returns the loaded library (loads it on first use)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            "libctbb_gb300.so is not built (%s); run `python -c \"import __graft_entry__ as g; "
            "g.build()\"` or `python -m ctbangbang_gb300.build`" % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(func_name, status):
    """Raises CtbbError for a non-zero status of the named entry point."""
    if status != 0:
        text = load().ctbb_last_error().decode(errors="replace")
        raise CtbbError(func_name, status, text)
    return status


def call(name, *args):
    return check(name, getattr(load(), name)(*args))
