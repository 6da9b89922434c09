"""CPU tests of the boundary: struct layout, exported symbols, the host
planner against the reference planner's golden tables, the .prm parser, the
ramp-kernel generator against the reference's kernel files, and the loud
failure of compute entry points without a GPU."""
import ctypes as C
import glob
import hashlib
import json
import os
import re

import numpy as np
import pytest

from ctbangbang_gb300 import lib as L
from ctbangbang_gb300 import scans, structs
from tests.conftest import HAS_GPU, REPO

GOLDEN = os.path.join(REPO, "tests", "golden")


def test_struct_layout_matches_header(lib):
    arr = (C.c_size_t * 12)()
    n = lib.ctbb_struct_layout(arr, 12)
    assert n == 12
    assert arr[0] == C.sizeof(structs.ReconMetadata)
    assert list(arr)[1:] == structs.layout_offsets()


def test_struct_layout_matches_reference(lib, ref_lib):
    assert ref_lib.ref_sizeof_recon_metadata() == C.sizeof(structs.ReconMetadata)
    assert [ref_lib.ref_offsetof(i) for i in range(11)] == structs.layout_offsets()


def test_every_declared_symbol_is_exported(lib):
    header = open(os.path.join(REPO, "include", "ctbb_gb300.h")).read()
    declared = set(re.findall(r"^(?:const\s+)?[a-z_0-9]+\s*\*?\s*(ctbb_[a-z0-9_]+)\s*\(", header, re.M))
    assert len(declared) >= 29
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    # the Python prototypes cover every declared entry point
    assert declared <= set(L.PROTOTYPES) | {"ctbb_struct_layout"}
    # the C++-linkage drop-ins of the reference signatures
    out = os.popen("nm -D --defined-only %s" % L.LIB_PATH).read()
    for mangled in ("_Z18adaptive_filter_kkP14recon_metadata", "_Z12rebin_filterP14recon_metadata",
                    "_Z11backprojectP14recon_metadata", "_Z20finalize_image_stackP14recon_metadata"):
        assert mangled in out


def test_integration_guide_lists_every_entry_point():
    """The integration guide's entry-point index names every function the
    header declares (a binding author starts from that index)."""
    header = open(os.path.join(REPO, "include", "ctbb_gb300.h")).read()
    declared = set(re.findall(r"^(?:const\s+)?[a-z_0-9]+\s*\*?\s*(ctbb_[a-z0-9_]+)\s*\(", header, re.M))
    guide = open(os.path.join(REPO, "INTEGRATION.md")).read()
    listed = set(re.findall(r"`(ctbb_[a-z0-9_]+)`", guide))
    assert not declared - listed, sorted(declared - listed)


def test_version(lib):
    assert b"sm_103a" in lib.ctbb_version()


@pytest.mark.skipif(HAS_GPU, reason="checks the no-device error path")
def test_compute_entry_points_fail_loudly_without_gpu(lib, tmp_path):
    spec = scans.tiny(0, 0)
    mr = scans.plan_spec(spec, str(tmp_path))
    lib.ctbb_update_block_info(C.byref(mr))
    for name in ("ctbb_adaptive_filter_kk", "ctbb_rebin_filter", "ctbb_finalize_image_stack"):
        st = getattr(lib, name)(C.byref(mr))
        assert L.STATUS[st] == "CTBB_ERR_NO_DEVICE", name
        assert b"no CUDA device" in lib.ctbb_last_error()
    with pytest.raises(L.CtbbError):
        L.call("ctbb_rebin_filter", C.byref(mr))
    dummy = C.c_void_p(1 << 20)  # never dereferenced: the device check comes first
    st = lib.ctbb_batch_add_device(C.byref(mr), dummy, dummy, C.c_float(0.0))
    assert L.STATUS[st] == "CTBB_ERR_NO_DEVICE", lib.ctbb_last_error()
    assert L.STATUS[lib.ctbb_batch_run()] == "CTBB_ERR_NO_DEVICE"
    taps = (C.c_float * 256)()
    st = lib.ctbb_ramp_filter_fp16_device(dummy, 1, 128, taps, 0, dummy, dummy)
    assert L.STATUS[st] == "CTBB_ERR_NO_DEVICE"
    # argument checks come before the device check
    st = lib.ctbb_ramp_filter_fp16_device(dummy, 1, 100, taps, 0, dummy, dummy)
    assert L.STATUS[st] == "CTBB_ERR_ARGUMENT" and b"multiple of 64" in lib.ctbb_last_error()
    st = lib.ctbb_ramp_filter_fp16_device(dummy, 1, 128, taps, 48, dummy, dummy)
    assert L.STATUS[st] == "CTBB_ERR_ARGUMENT"
    assert L.STATUS[lib.ctbb_set_storage(3)] == "CTBB_ERR_ARGUMENT"
    assert lib.ctbb_set_storage(L.STORAGE_FP16) == 0 and lib.ctbb_set_storage(L.STORAGE_FP32) == 0
    h = C.c_void_p()
    assert L.STATUS[lib.ctbb_context_create(C.byref(h))] == "CTBB_ERR_NO_DEVICE" and not h.value
    assert L.STATUS[lib.ctbb_server_create(2, C.c_size_t(1 << 30), C.byref(h))] == "CTBB_ERR_NO_DEVICE"
    assert not h.value
    scans.free_plan(mr)


def test_scan_workspace_bytes_counts_the_union_window(lib, tmp_path):
    """The whole-scan footprint (the request server's admission unit): two
    copies of the union window's raw frames, its rebinned rows, the image
    and final stacks; more than one block's window, less than two scans."""
    spec = scans.tiny(1, 1, n_slices=14, slice_thickness=2.5, seed=3)
    mr = scans.plan_spec(spec, str(tmp_path))
    need = lib.ctbb_scan_workspace_bytes(C.byref(mr))
    assert mr.ri.n_blocks >= 2
    frame = mr.cg.n_rows_raw * mr.cg.n_channels * 4
    block_ws = lib.ctbb_workspace_bytes(C.byref(mr))
    assert need > 2 * mr.ri.n_proj_pull * frame
    assert need < 4 * spec.n_readings * frame + block_ws + (16 << 20)
    assert lib.ctbb_scan_workspace_bytes(None) == 0
    scans.free_plan(mr)


# ---------------------------------------------------------------- planner

def _plan_fixtures():
    return sorted(glob.glob(os.path.join(GOLDEN, "plan_*.json")))


def _ri(mr):
    ri = {f: getattr(mr.ri, f) for f, _ in structs.ReconInfo._fields_ if f != "cb"}
    ri.update({"cb." + f: getattr(mr.ri.cb, f) for f, _ in structs.BlockInfo._fields_})
    return ri


def _spec_from(d):
    keep = {k: v for k, v in d.items() if k in scans.ScanSpec.__dataclass_fields__}
    return scans.ScanSpec(**keep)


@pytest.mark.parametrize("path", _plan_fixtures(), ids=lambda p: os.path.basename(p))
def test_planner_bit_exact_vs_reference_golden(lib, tmp_path, path):
    """configure_ct_geom / configure_reconstruction / update_block_info of this
    library reproduce the reference planner's integers and float tables exactly."""
    fx = json.load(open(path))
    spec = _spec_from(fx["spec"])
    mr = scans.plan_spec(spec, str(tmp_path))
    n = spec.n_readings
    for k, v in fx["geom"].items():
        assert getattr(mr.cg, k) == pytest.approx(v, abs=0) or np.float32(getattr(mr.cg, k)) == np.float32(v), k
    assert np.float32(mr.rp.end_pos) == np.float32(fx["rp_end_pos"])
    got = _ri(mr)
    for k, v in fx["plan"].items():
        assert np.float32(got[k]) == np.float32(v) if isinstance(v, float) else got[k] == v, k
    assert hashlib.sha256(C.string_at(mr.tube_angles, 4 * n)).hexdigest() == fx["tube_angles_sha256"]
    assert hashlib.sha256(C.string_at(mr.table_positions, 8 * n)).hexdigest() == fx["table_positions_sha256"]
    assert len(fx["blocks"]) == mr.ri.n_blocks
    for blk in fx["blocks"]:
        lib.ctbb_update_block_info(C.byref(mr))
        got = _ri(mr)
        for k, v in blk.items():
            assert np.float32(got[k]) == np.float32(v) if isinstance(v, float) else got[k] == v, (k, got[k], v)
    scans.free_plan(mr)


def test_planner_rejects_out_of_range(lib, tmp_path):
    spec = scans.tiny(0, 0)
    spec.start_pos = -50.0
    prm, inst = scans.prepare(spec, str(tmp_path))
    with pytest.raises(L.CtbbError) as e:
        scans.plan(prm, inst)
    assert e.value.status_name == "CTBB_ERR_RANGE"


def test_prm_missing_key_is_an_error_not_exit(lib, tmp_path):
    p = tmp_path / "bad.prm"
    p.write_text("Nrows:\t16\n% no CollSlicewidth\n")
    rp = structs.ReconParams()
    st = lib.ctbb_configure_recon_params(str(p).encode(), C.byref(rp))
    assert L.STATUS[st] == "CTBB_ERR_CONFIG"
    assert rp.n_rows == 16


@pytest.mark.parametrize("key,value", [
    ("SliceThickness:", "-2.0"), ("CollSlicewidth:", "inf"), ("PitchValue:", "nan"), ("ReconFOV:", "-1"),
    ("Xorigin:", "nan"), ("Nx:", "-512"), ("Ny:", "100000"), ("Zffs:", "2"), ("Readings:", "-5"),
])
def test_prm_out_of_range_values_are_config_errors(lib, tmp_path, key, value):
    """Values the reference would carry into planning (negative or non-finite
    sizes, a negative side parsed as a huge unsigned, FFS flags other than 0/1)
    are rejected by the parser with a status, never by exit() or a crash."""
    prm, _ = scans.prepare(scans.tiny(0, 0), str(tmp_path))
    txt = open(prm).read()
    assert re.search(r"^%s\s" % re.escape(key), txt, flags=re.M), key
    open(prm, "w").write(re.sub(r"^%s\s.*$" % re.escape(key), "%s\t%s" % (key, value), txt, flags=re.M))
    rp = structs.ReconParams()
    st = lib.ctbb_configure_recon_params(prm.encode(), C.byref(rp))
    assert L.STATUS[st] == "CTBB_ERR_CONFIG", (key, value, lib.ctbb_last_error())
    assert key[:-1].encode() in lib.ctbb_last_error() or b"Nx/Ny" in lib.ctbb_last_error()


def test_missing_raw_file_is_an_io_error(lib, tmp_path):
    spec = scans.tiny(0, 0)
    mr = scans.plan_spec(spec, str(tmp_path))
    mr.rp.raw_data_file = b"not_there.raw"
    L.call("ctbb_update_block_info", C.byref(mr))
    st = lib.ctbb_extract_projections(C.byref(mr))
    assert L.STATUS[st] == "CTBB_ERR_IO", lib.ctbb_last_error()
    scans.free_plan(mr)


def test_prm_parser_matches_reference(lib, ref_lib, tmp_path):
    spec = scans.CONFIGS["config2"]
    prm, _ = scans.prepare(spec, str(tmp_path))
    with open(prm, "a") as f:
        f.write("TableFeed:\t12.5 % overrides PitchValue\nNSlices:\t7\n")
    a, b = structs.ReconParams(), structs.ReconParams()
    L.call("ctbb_configure_recon_params", prm.encode(), C.byref(a))
    ref_lib.ref_configure_recon_params(prm.encode(), C.byref(b))
    assert bytes(a) == bytes(b)


def test_builtin_scanners_match_reference(lib, ref_lib, tmp_path):
    for scanner in ("0", "1", "2"):
        spec = scans.CONFIGS["config2"]
        prm, inst = scans.prepare(spec, str(tmp_path))
        mr_a, mr_b = structs.ReconMetadata(), structs.ReconMetadata()
        for mr in (mr_a, mr_b):
            L.call("ctbb_configure_recon_params", prm.encode(), C.byref(mr.rp))
            mr.rp.scanner = scanner.encode()
            mr.install_dir = inst.encode()
        L.call("ctbb_configure_ct_geom", C.byref(mr_a))
        ref_lib.ref_configure_ct_geom(C.byref(mr_b))
        assert bytes(mr_a.cg) == bytes(mr_b.cg), scanner
        assert mr_a.rp.file_subtype == mr_b.rp.file_subtype


# ---------------------------------------------------------------- filter taps

def test_ramp_taps_equal_reference_sharp_kernels(lib):
    """KAT: the reference's f_<N>_sharp files are the ramp formula of
    resources/ramp.m with c = 1, a = 1, ds = r_f sin(fai/2)."""
    kat = json.load(open(os.path.join(GOLDEN, "ramp_kat.json")))
    geo = {"f_736_sharp": (595.0, 0.067864 * 3.1415926535897 / 180.0),   # Definition AS
           "f_672_sharp": (570.0, 0.07758621 * 3.1415926535897 / 180.0)}  # Sensation 64
    for name, fx in kat.items():
        r_f, fai = geo[name]
        n_os = fx["n_os"]
        taps = (C.c_float * (2 * n_os))()
        ds = np.float32(r_f * np.sin(np.float32(fai) / 2.0))
        L.call("ctbb_ramp_filter_taps", n_os, C.c_float(float(ds)), 1.0, 1.0, taps)
        t = np.frombuffer(taps, np.float32)
        np.testing.assert_allclose(t[n_os - 8:n_os + 9], fx["centre_taps"], rtol=0, atol=2e-7)
        assert abs(t.astype(np.float64).sum() - fx["sum"]) < 1e-5


def test_load_filter_generates_missing_ramp(lib, tmp_path):
    spec = scans.tiny(0, 0)
    mr = scans.plan_spec(spec, str(tmp_path))
    for f in glob.glob(str(tmp_path / "resources" / "filters" / "*")):
        os.remove(f)
    n = 2 * mr.cg.n_channels_oversampled
    t = (C.c_float * n)()
    L.call("ctbb_load_filter", C.byref(mr), t)
    taps = np.frombuffer(t, np.float32)
    ds = mr.cg.r_f * np.sin(mr.cg.fan_angle_increment / 2.0)
    assert taps[n // 2] == pytest.approx(1.0 / (4.0 * ds), rel=1e-6)
    mr.rp.recon_kernel = 2  # "medium" is not present: a clear error, not exit()
    with pytest.raises(L.CtbbError) as e:
        L.call("ctbb_load_filter", C.byref(mr), t)
    assert e.value.status_name == "CTBB_ERR_IO"
    scans.free_plan(mr)


def test_finalize_with_a_table_that_does_not_move_is_a_config_error(lib, tmp_path):
    """The reference takes the table's direction as dtp / |dtp| with dtp the
    distance between table positions 0 and 1000 (finalize_image_stack_cpu.cu:35),
    undefined for an axial scan; the library returns CTBB_ERR_CONFIG instead
    of ordering the slices by garbage, before it looks for a device."""
    spec = scans.tiny(0, 0)
    mr = scans.plan_spec(spec, str(tmp_path))
    tp = np.ctypeslib.as_array(mr.table_positions, (spec.n_readings,))
    tp[:] = tp[0]
    st = lib.ctbb_finalize_image_stack(C.byref(mr))
    assert L.STATUS[st] == "CTBB_ERR_CONFIG", lib.ctbb_last_error()
    assert b"does not move" in lib.ctbb_last_error()
    scans.free_plan(mr)
