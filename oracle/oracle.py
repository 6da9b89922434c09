"""Loaders of the oracle libraries (TEST INFRASTRUCTURE).

  oracle()     -> ctypes handle of oracle/_build/libctbb_oracle.so, this
                  project's CPU restatement of the reference path (built with
                  `make -C oracle` on first use; plain g++).
  reference()  -> ctypes handle of oracle/_ref/libctbb_ref.so, the reference's
                  own CPU sources compiled with oracle/ref/Makefile, or None when
                  the reference tree is not available on this machine and
                  nothing was built.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and reference
arm import this module.  The product never does.
"""
import ctypes as C
import os
import subprocess

from ctbangbang_gb300.structs import ReconMetadata, ReconParams

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "_build", "libctbb_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libctbb_ref.so")
# The reference source tree, named by the environment (no default: the
# reference build is made only where its sources are present).
REFERENCE_TREE = os.environ.get("CTBB_REFERENCE_TREE")

_MR = C.POINTER(ReconMetadata)
_F = C.POINTER(C.c_float)
_D = C.POINTER(C.c_double)

_oracle = None
_ref = None


def build_oracle():
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return ORACLE_LIB


def build_reference():
    """Compiles the reference CPU path if its sources are present; returns the
    library path or None."""
    if not REFERENCE_TREE or not os.path.isdir(os.path.join(REFERENCE_TREE, "src")):
        return REF_LIB if os.path.exists(REF_LIB) else None
    subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), "REF=" + REFERENCE_TREE], check=True)
    return REF_LIB


def oracle():
    global _oracle
    if _oracle is None:
        srcs = [os.path.join(HERE, f) for f in ("ctbb_oracle.cpp", "ctbb_oracle_plan.cpp")]
        if not os.path.exists(ORACLE_LIB) or any(os.path.getmtime(ORACLE_LIB) < os.path.getmtime(f) for f in srcs):
            build_oracle()
        lib = C.CDLL(ORACLE_LIB)
        protos = {
            "oracle_load_filter": (C.c_int, [_MR, _F]),
            "oracle_adaptive_filter": (C.c_int, [_MR]),
            "oracle_rebin": (C.c_int, [_MR]),
            "oracle_filter_rows": (C.c_int, [_F, C.c_size_t, C.c_int, _F]),
            "oracle_rebin_filter": (C.c_int, [_MR]),
            "oracle_backproject_range": (C.c_int, [_MR, _F, C.c_int, C.c_int, _F]),
            "oracle_backproject": (C.c_int, [_MR]),
            "oracle_finalize": (C.c_int, [_MR]),
            "oracle_n_half_turns": (C.c_int, [_MR]),
            "oracle64_block": (C.c_int, [_MR, _F, C.c_int, _F, _D]),
            "oracle64_finalize": (C.c_int, [_MR, _D, _D]),
            "oracle64_backproject_range": (C.c_int, [_MR, _F, C.c_int, C.c_int, _D]),
            "oracle_rebin_views": (C.c_int, [_MR, _F, C.c_int, C.c_int, _F]),
            "oracle_backproject_patch": (C.c_int, [_MR, _F, C.c_int, C.c_int, C.c_int, C.c_int, _F]),
            "oracle64_adaptive_filter": (C.c_int, [_MR, _F, _D]),
            "oracle64_rebin_views": (C.c_int, [_MR, _D, C.c_int, C.c_int, _D]),
            "oracle64_filter_rows": (C.c_int, [_D, C.c_size_t, C.c_int, _F]),
            "oracle64_backproject_patch": (C.c_int, [_MR, _D, C.c_int, C.c_int, C.c_int, C.c_int, _D]),
            "oracle_n_slices_final": (C.c_int, [_MR]),
            "oracle64_finalize_weights": (C.c_int, [_MR, C.c_int, _D, C.POINTER(C.c_int)]),
            "oracle_configure_recon_params": (C.c_int, [C.c_char_p, C.POINTER(ReconParams)]),
            "oracle_configure_ct_geom": (C.c_int, [_MR]),
            "oracle_configure_reconstruction": (C.c_int, [_MR]),
            "oracle_update_block_info": (C.c_int, [_MR]),
            "oracle_free_plan": (C.c_int, [_MR]),
            "oracle_ramp_taps": (C.c_int, [C.c_int, C.c_float, C.c_float, C.c_float, _F]),
            "oracle_interp2": (C.c_float, [_F, C.c_int, C.c_int, C.c_float, C.c_float]),
            "oracle_interp3": (C.c_float, [_F, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float]),
        }
        for name, (res, args) in protos.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _oracle = lib
    return _oracle


def reference():
    global _ref
    if _ref is None:
        path = REF_LIB if os.path.exists(REF_LIB) else build_reference()
        if not path or not os.path.exists(path):
            return None
        lib = C.CDLL(path)
        protos = {
            "ref_sizeof_recon_metadata": (C.c_size_t, []),
            "ref_offsetof": (C.c_size_t, [C.c_int]),
            "ref_configure_recon_params": (C.c_int, [C.c_char_p, C.POINTER(ReconParams)]),
            "ref_configure_ct_geom": (C.c_int, [_MR]),
            "ref_configure_reconstruction": (C.c_int, [_MR]),
            "ref_update_block_info": (C.c_int, [_MR]),
            "ref_extract_projections": (C.c_int, [_MR]),
            "ref_adaptive_filter_kk": (C.c_int, [_MR]),
            "ref_adaptive_thresholds": (C.c_int, [_MR, _F]),
            "ref_rebin_filter_cpu": (C.c_int, [_MR]),
            "ref_backproject_cpu": (C.c_int, [_MR]),
            "ref_finalize_image_stack_cpu": (C.c_int, [_MR]),
            "ref_load_filter": (C.c_int, [_MR, _F]),
            "ref_free": (C.c_int, [_MR]),
            "ref_interp2": (C.c_float, [_F, C.c_int, C.c_int, C.c_float, C.c_float]),
            "ref_interp3": (C.c_float, [_F, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float]),
        }
        for name, (res, args) in protos.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _ref = lib
    return _ref
