"""GPU parity tests: the CUDA path, called through the C ABI, against the
oracle (the reference CPU path's arithmetic) and the reference's golden
fixtures.

Bars (float32 image work in HU, 1 HU = 0.019/1000 per mm):
  adaptive filter, unfiltered rebin, finalize:  bit-exact
  ramp filter (FP32 FFT vs the reference's double FFT): |err| <= 2e-5 * max|row|
  backprojection / end to end:                   <= 1 HU max, <= 0.1 HU RMS
  device whole-scan path vs drop-in calls:       bit-exact
"""
import ctypes as C
import os

import numpy as np
import pytest

from ctbangbang_gb300 import lib as L
from ctbangbang_gb300 import scans

import ctbb_synth
from tests import helpers as H
from tests.test_cpu_oracle import GoldenScan, assert_rebin_matches_golden, golden_block_files, load_case

pytestmark = pytest.mark.gpu

MODES = [(0, 0), (0, 1), (1, 0), (1, 1)]
FILTER_RTOL = 2e-5
HU_MAX, HU_RMS = 1.0, 0.1


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def ptr(t):
    return C.c_void_p(t.data_ptr())


def fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def assert_filter_close(got, want):
    scale = float(np.abs(want).max())
    err = float(np.abs(got.astype(np.float64) - want).max())
    assert err <= FILTER_RTOL * scale, (err, scale)


def assert_hu(got, want):
    mx, rms = H.hu_errors(got, want)
    assert mx <= HU_MAX and rms <= HU_RMS, (mx, rms)
    return mx, rms


@pytest.fixture(params=MODES, ids=lambda m: "z%d_p%d" % m)
def mode_scan(request, lib, tmp_path):
    z, p = request.param
    spec = scans.tiny(z, p, adaptive_filtration=3.0, seed=200 + 2 * z + p)
    s = H.Scan(spec, str(tmp_path))
    yield s
    s.close()


def test_adaptive_filter_bit_exact(torch_cuda, oracle_lib, mode_scan):
    mr = mode_scan.mr
    raw = mode_scan.next_block()
    want = H.oracle_block(oracle_lib, mode_scan, raw)["adaptive"]
    assert (want != raw).sum() > 0
    L.call("ctbb_adaptive_filter_kk", C.byref(mr))
    got = H.view(mr.ctd.raw, H.dims(mr)["n_raw"]).copy()
    np.testing.assert_array_equal(got, want)


def test_rebin_bit_exact_and_filter(torch_cuda, oracle_lib, mode_scan):
    torch = torch_cuda
    mr = mode_scan.mr
    raw = mode_scan.next_block()
    st = H.oracle_block(oracle_lib, mode_scan, raw)
    d = H.dims(mr)
    d_raw = dev(torch, st["adaptive"])
    d_rb = torch.empty(d["n_rebin"], dtype=torch.float32, device="cuda")
    L.call("ctbb_rebin_device", C.byref(mr), ptr(d_raw), ptr(d_rb))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d_rb.cpu().numpy(), st["rebin"])
    taps = H.taps_of(mr)
    L.call("ctbb_ramp_filter_device", ptr(d_rb), d["n_views"] * mr.cg.n_rows, mr.cg.n_channels_oversampled, fptr(taps))
    torch.cuda.synchronize()
    assert_filter_close(d_rb.cpu().numpy(), st["filtered"])


def test_backproject_hu(torch_cuda, oracle_lib, mode_scan):
    torch = torch_cuda
    mr = mode_scan.mr
    raw = mode_scan.next_block()
    st = H.oracle_block(oracle_lib, mode_scan, raw)
    d = H.dims(mr)
    d_rb = dev(torch, st["filtered"])
    d_blk = torch.empty(d["n_block"], dtype=torch.float32, device="cuda")
    L.call("ctbb_backproject_device", C.byref(mr), ptr(d_rb), ptr(d_blk))
    torch.cuda.synchronize()
    assert_hu(d_blk.cpu().numpy(), st["block"])


def fp64_block(oracle_lib, mr, raw):
    """The FP64 oracle's block (adaptive filter always, as main.cu:222 calls it)."""
    taps = H.taps_of(mr)
    out = np.zeros(H.dims(mr)["n_block"], np.float64)
    oracle_lib.oracle64_block(C.byref(mr), fptr(np.ascontiguousarray(raw, np.float32)), 1, fptr(taps),
                              out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def test_end_to_end_vs_fp64_oracle(torch_cuda, oracle_lib, mode_scan):
    """The drop-in chain (adaptive filter, rebin + ramp filter,
    backprojection) against the FP64 oracle of the same block: the bars of the
    FP32 reference path apply (the reference's own FP32 path is within
    0.02 HU of FP64 on these scans)."""
    mr = mode_scan.mr
    raw = mode_scan.next_block()
    want = fp64_block(oracle_lib, mr, raw)
    mode_scan.set_raw(raw)
    L.call("ctbb_adaptive_filter_kk", C.byref(mr))
    L.call("ctbb_rebin_filter", C.byref(mr))
    L.call("ctbb_backproject", C.byref(mr))
    d = H.dims(mr)
    got = H.view(mr.ctd.image, d["n_image"])[:d["n_block"]].astype(np.float64)
    assert np.abs(want).max() > 0.01
    mx, rms = assert_hu(got, want)
    print("GPU vs FP64 oracle: max %.4f HU, rms %.5f HU" % (mx, rms))


def run_dropin(scan):
    """main.cu's block loop and finalize through the drop-in entry points."""
    mr = scan.mr
    for _ in range(mr.ri.n_blocks):
        scan.next_block()
        L.call("ctbb_adaptive_filter_kk", C.byref(mr))
        L.call("ctbb_rebin_filter", C.byref(mr))
        L.call("ctbb_backproject", C.byref(mr))
    L.call("ctbb_finalize_image_stack", C.byref(mr))
    d = H.dims(mr)
    n_final = L.load().ctbb_n_slices_final(C.byref(mr))
    img = H.view(mr.ctd.image, d["n_image"]).copy()
    fin = H.view(mr.ctd.final_image_stack, n_final * d["plane"]).copy()
    return img, fin


def run_oracle(orc, scan):
    mr = scan.mr
    for _ in range(mr.ri.n_blocks):
        raw = scan.next_block()
        scan.set_raw(raw)
        orc.oracle_adaptive_filter(C.byref(mr))
        orc.oracle_rebin_filter(C.byref(mr))
        orc.oracle_backproject(C.byref(mr))
    orc.oracle_finalize(C.byref(mr))
    d = H.dims(mr)
    n_final = L.load().ctbb_n_slices_final(C.byref(mr))
    return (H.view(mr.ctd.image, d["n_image"]).copy(),
            H.view(mr.ctd.final_image_stack, n_final * d["plane"]).copy())


def reset_blocks(scan):
    scan.mr.ri.cb.block_idx = 0


@pytest.mark.parametrize("variant", ["multi_block_in", "reverse_rows", "strength0"])
def test_dropin_pipeline_vs_oracle(torch_cuda, oracle_lib, lib, tmp_path, variant):
    if variant == "multi_block_in":
        spec = scans.tiny(0, 1, adaptive_filtration=2.0, n_slices=14, slice_thickness=2.5, table_dir="in", seed=31)
    elif variant == "reverse_rows":
        spec = scans.tiny(1, 1, adaptive_filtration=2.0, reverse_row_interleave=1, seed=32)
    else:
        spec = scans.tiny(1, 0, adaptive_filtration=0.0, seed=33)
    scan = H.Scan(spec, str(tmp_path))
    img_g, fin_g = run_dropin(scan)
    reset_blocks(scan)
    scan.mr.ctd.final_image_stack = None  # the drop-in's stack stays allocated (test only)
    img_o, fin_o = run_oracle(oracle_lib, scan)
    assert_hu(img_g, img_o)
    assert_hu(fin_g, fin_o)
    # finalize alone is bit-exact given the same image
    H.view(scan.mr.ctd.image, img_o.size)[:] = img_o
    L.call("ctbb_finalize_image_stack", C.byref(scan.mr))
    np.testing.assert_array_equal(H.view(scan.mr.ctd.final_image_stack, fin_o.size), fin_o)
    scan.close()


def shape_spec(variant):
    if variant == "odd_image":  # neither side a multiple of the 32 x 4 CTA or 8 x 4 warp tile
        return scans.tiny(0, 1, adaptive_filtration=2.0, nx=37, ny=29, seed=61)
    if variant == "pitch_0.6":  # more half turns in the pull window, two blocks
        return scans.tiny(1, 1, adaptive_filtration=2.0, pitch=0.6, n_slices=14, slice_thickness=2.5, seed=62)
    if variant == "pitch_1.4":
        return scans.tiny(1, 0, adaptive_filtration=2.0, pitch=1.4, seed=63)
    if variant == "wide_detector":  # 4096 oversampled channels: 8192-point filter, runtime row stride
        return scans.tiny(0, 1, adaptive_filtration=2.0, n_channels=2048, seed=71)
    spec = scans.tiny(1, 1, adaptive_filtration=2.0, nx=40, ny=40, seed=64)
    spec.x_origin, spec.y_origin, spec.tube_start_angle = 7.5, -4.0, 30.0
    return spec


@pytest.mark.parametrize("variant", ["odd_image", "pitch_0.6", "pitch_1.4", "offset_origin", "wide_detector"])
def test_image_shapes_and_helices_vs_oracle(torch_cuda, oracle_lib, lib, tmp_path, variant):
    """Image sides off the thread tiling, other pitches, an off-centre field
    of view with a rotated tube start: the drop-in block loop against the
    oracle, end to end."""
    scan = H.Scan(shape_spec(variant), str(tmp_path))
    img_g, fin_g = run_dropin(scan)
    reset_blocks(scan)
    scan.mr.ctd.final_image_stack = None  # the drop-in's stack stays allocated (test only)
    img_o, fin_o = run_oracle(oracle_lib, scan)
    assert float(np.abs(img_o).max()) > 0.01
    assert_hu(img_g, img_o)
    assert_hu(fin_g, fin_o)
    scan.close()


def test_zero_scan_reconstructs_to_zero(torch_cuda, oracle_lib, lib, tmp_path):
    """An empty scan (no attenuation: every line integral 0, so the adaptive
    filter's per-frame maxima are 0 and its eccentricity 0/0): every stage
    stays finite and the stack is exactly 0, as in the reference arithmetic,
    through the drop-in chain and the whole-scan path."""
    torch = torch_cuda
    spec = scans.tiny(1, 1, adaptive_filtration=2.0, n_slices=14, slice_thickness=2.5, seed=53)
    scan = H.Scan(spec, str(tmp_path))
    scan.frames[:] = 0
    raw = scan.next_block()
    st = H.oracle_block(oracle_lib, scan, raw)
    assert not st["block"].any()
    reset_blocks(scan)
    img, fin = run_dropin(scan)
    assert np.isfinite(img).all() and not img.any()
    assert np.isfinite(fin).all() and not fin.any()
    d_scan = dev(torch, scan.frames.reshape(-1))
    d_fin = torch.full((fin.size,), float("nan"), dtype=torch.float32, device="cuda")
    L.call("ctbb_reconstruct_scan_device", C.byref(scan.mr), ptr(d_scan), ptr(d_fin), 0.0)
    out = d_fin.cpu().numpy()
    assert np.isfinite(out).all() and not out.any()
    scan.close()


def test_large_image_backprojection_patches(torch_cuda, oracle_lib, lib, tmp_path):
    """A 1024^2 image (a 512 x 256 CTA grid): the GPU backprojection of the
    oracle's filtered rows against the oracle's on a corner and a centre patch."""
    torch = torch_cuda
    scan = H.Scan(scans.tiny(1, 1, adaptive_filtration=2.0, nx=1024, ny=1024, seed=72), str(tmp_path))
    mr = scan.mr
    scan.next_block()
    d = H.dims(mr)
    # the oracle's filtered rows (its backprojection of the whole image would
    # take minutes; only the patches below are backprojected)
    oracle_lib.oracle_adaptive_filter(C.byref(mr))
    oracle_lib.oracle_rebin(C.byref(mr))
    rows = H.view(mr.ctd.rebin, d["n_rebin"]).copy()
    oracle_lib.oracle_filter_rows(fptr(rows), d["n_views"] * mr.cg.n_rows, mr.cg.n_channels_oversampled,
                                  fptr(H.taps_of(mr)))
    d_blk = torch.empty(d["n_block"], dtype=torch.float32, device="cuda")
    L.call("ctbb_backproject_device", C.byref(mr), ptr(dev(torch, rows)), ptr(d_blk))
    torch.cuda.synchronize()
    got = d_blk.cpu().numpy().reshape(mr.ri.n_slices_block, 1024, 1024)
    want = np.zeros(d["n_block"], np.float32)
    for x0, y0 in ((0, 0), (496, 504), (992, 960)):
        oracle_lib.oracle_backproject_patch(C.byref(mr), fptr(rows), x0, x0 + 32, y0, y0 + 32, fptr(want))
        w = want.reshape(got.shape)[:, y0:y0 + 32, x0:x0 + 32]
        assert_hu(got[:, y0:y0 + 32, x0:x0 + 32], w)
    assert np.abs(want).max() > 0.005
    scan.close()


def test_reconstruct_device_equals_dropin(torch_cuda, lib, tmp_path):
    torch = torch_cuda
    spec = scans.tiny(1, 1, adaptive_filtration=2.0, n_slices=14, slice_thickness=2.5, seed=41)
    scan = H.Scan(spec, str(tmp_path))
    _, fin_g = run_dropin(scan)
    d_scan = dev(torch, scan.frames.reshape(-1))
    d_fin = torch.empty(fin_g.size, dtype=torch.float32, device="cuda")
    L.call("ctbb_reconstruct_device", C.byref(scan.mr), ptr(d_scan), ptr(d_fin), 0.0)
    np.testing.assert_array_equal(d_fin.cpu().numpy(), fin_g)
    # HU output: 1000 (mu - mu_w) / mu_w of the same stack
    L.call("ctbb_reconstruct_device", C.byref(scan.mr), ptr(d_scan), ptr(d_fin), scans.MU_WATER)
    hu = d_fin.cpu().numpy()
    np.testing.assert_allclose(hu, 1000.0 * (fin_g - scans.MU_WATER) / scans.MU_WATER, rtol=1e-5, atol=1e-3)
    scan.close()


@pytest.mark.parametrize("path", golden_block_files(), ids=lambda p: os.path.basename(p)[6:-4])
def test_gpu_vs_reference_golden(torch_cuda, lib, tmp_path, path):
    """The CUDA path against outputs of the reference's own CPU code."""
    torch = torch_cuda
    z, meta, spec, frames = load_case(path)
    scan = GoldenScan(spec, frames, str(tmp_path))
    mr = scan.mr
    step = meta["view_step"]
    for b in range(meta["n_blocks"]):
        raw = scan.next_block()
        d = H.dims(mr)
        L.call("ctbb_adaptive_filter_kk", C.byref(mr))
        got = H.view(mr.ctd.raw, d["n_raw"]).copy()
        changed = np.nonzero(got != raw)[0]
        np.testing.assert_array_equal(changed, z["adaptive_idx_b%d" % b])
        np.testing.assert_array_equal(got[changed], z["adaptive_val_b%d" % b])
        d_raw = dev(torch, got)
        d_rb = torch.empty(d["n_rebin"], dtype=torch.float32, device="cuda")
        L.call("ctbb_rebin_device", C.byref(mr), ptr(d_raw), ptr(d_rb))
        torch.cuda.synchronize()
        vs = mr.cg.n_rows * mr.cg.n_channels_oversampled
        assert_rebin_matches_golden(d_rb.cpu().numpy().reshape(-1, vs)[::step], z["rebin_b%d" % b])
        L.call("ctbb_rebin_filter", C.byref(mr))
        L.call("ctbb_backproject", C.byref(mr))
    d = H.dims(mr)
    assert_hu(H.view(mr.ctd.image, d["n_image"]), z["image"])
    L.call("ctbb_finalize_image_stack", C.byref(mr))
    assert_hu(H.view(mr.ctd.final_image_stack, z["final"].size), z["final"])
    scan.close()


def test_rebin_filter_testing_flag_copies_filtered_rows(torch_cuda, oracle_lib, lib, tmp_path):
    """flags.testing: the drop-in rebin_filter also fills host ctd.rebin (the
    reference's rebin.ct_test checkpoint)."""
    scan = H.Scan(scans.tiny(0, 1, seed=51), str(tmp_path))
    mr = scan.mr
    raw = scan.next_block()
    st = H.oracle_block(oracle_lib, scan, raw, adaptive=False)
    mr.flags.testing = 1
    L.call("ctbb_rebin_filter", C.byref(mr))
    assert_filter_close(H.view(mr.ctd.rebin, H.dims(mr)["n_rebin"]).copy(), st["filtered"])
    L.call("ctbb_backproject", C.byref(mr))
    assert not mr.ctd.d_rebin
    scan.close()


def test_backproject_without_rebin_is_a_state_error(torch_cuda, lib, tmp_path):
    scan = H.Scan(scans.tiny(0, 0, seed=52), str(tmp_path))
    scan.next_block()
    st = L.load().ctbb_backproject(C.byref(scan.mr))
    assert L.STATUS[st] == "CTBB_ERR_STATE"
    scan.close()


def test_config1_geometry_reduced_image(torch_cuda, oracle_lib, lib, tmp_path):
    """Config-1 scanner and helix (672 ch x 16 rows, 1152 views/turn, pitch 1,
    3 turns, pull window past the end of the data) on a 48^2 image."""
    spec = scans.ScanSpec(**{**scans.CONFIGS["config1"].__dict__})
    spec.nx = spec.ny = 48
    spec.recon_fov = 48 * 0.68 * 4
    spec.n_slices = 4
    scan = H.Scan(spec, str(tmp_path))
    mr = scan.mr
    raw = scan.next_block()
    assert mr.ri.idx_pull_start + mr.ri.n_proj_pull > spec.n_readings  # frames past the end read 0
    st = H.oracle_block(oracle_lib, scan, raw)
    scan.set_raw(raw)
    L.call("ctbb_adaptive_filter_kk", C.byref(mr))
    np.testing.assert_array_equal(H.view(mr.ctd.raw, H.dims(mr)["n_raw"]), st["adaptive"])
    L.call("ctbb_rebin_filter", C.byref(mr))
    L.call("ctbb_backproject", C.byref(mr))
    d = H.dims(mr)
    assert_hu(H.view(mr.ctd.image, d["n_block"]), st["block"])
    scan.close()


def test_config2_block_adaptive_filter_and_rebin_bit_exact(torch_cuda, oracle_lib, lib, tmp_path):
    """Block 0 of the config-2 scan at full size (11264 frames of 32 x 736,
    phi+z FFS, adaptive filter on: 18 and 180 degree statistics windows of
    ~230 and ~2300 frames): the device adaptive filter against the oracle on
    every sample, and the device rebin against the oracle on views at the
    start, middle and end of the block -- bit for bit."""
    torch = torch_cuda
    from ctbangbang_gb300 import structs
    spec = scans.ScanSpec(**{**scans.CONFIGS["config2"].__dict__})
    spec.nx = spec.ny = 64
    mr = scans.plan_spec(spec, str(tmp_path))
    L.call("ctbb_update_block_info", C.byref(mr))
    m = structs.ReconMetadata()
    C.memmove(C.byref(m), C.byref(mr), C.sizeof(m))
    n = spec.n_readings
    frame = m.cg.n_rows_raw * m.cg.n_channels
    P = m.ri.n_proj_pull
    d = H.dims(mr)
    ta = dev(torch, np.ctypeslib.as_array(mr.tube_angles, (n,)).copy())
    tp = dev(torch, np.ctypeslib.as_array(mr.table_positions, (n,)).copy())
    objs = ctbb_synth.phantom_objects(spec)
    d_raw = torch.empty(P * frame, dtype=torch.float32, device="cuda")
    ctbb_synth.project_device(m, objs, ta.data_ptr(), tp.data_ptr(), int(m.ri.idx_pull_start), P, spec.i0,
                         spec.seed, d_raw.data_ptr(), torch.cuda.current_stream().cuda_stream)
    d_filt = torch.empty_like(d_raw)
    L.call("ctbb_adaptive_filter_device", C.byref(m), ptr(d_raw), ptr(d_filt))
    d_rb = torch.empty(d["n_rebin"], dtype=torch.float32, device="cuda")
    L.call("ctbb_rebin_device", C.byref(m), ptr(d_filt), ptr(d_rb))
    torch.cuda.synchronize()
    raw = d_raw.cpu().numpy()
    got_filt = d_filt.cpu().numpy()
    del d_raw, d_filt
    H.view(mr.ctd.raw, d["n_raw"])[:] = raw
    oracle_lib.oracle_adaptive_filter(C.byref(mr))
    want_filt = H.view(mr.ctd.raw, d["n_raw"]).copy()
    assert (want_filt != raw).sum() > 1000  # the filter changed samples
    np.testing.assert_array_equal(got_filt, want_filt)
    nv = d["n_views"]
    view = mr.cg.n_rows * mr.cg.n_channels_oversampled
    want = np.zeros(d["n_rebin"], np.float32)
    got = d_rb.cpu().numpy()
    for v0 in (0, nv // 2 - 4, nv - 8):
        oracle_lib.oracle_rebin_views(C.byref(mr), fptr(want_filt), v0, v0 + 8, fptr(want))
        np.testing.assert_array_equal(got[v0 * view:(v0 + 8) * view], want[v0 * view:(v0 + 8) * view])
    scans.free_plan(mr)


def test_config2_block_backprojection_512_patches(torch_cuda, oracle_lib, lib, tmp_path):
    """The benchmark's own image, config 2's block 0 at 512^2 over the full
    field (a warp then covers 8 x 4 mm, so the flat / inner / other classes
    mix as in the benchmark): the GPU block against the oracle on a 32 x 32
    patch at the centre and one at the edge of the field, all 32 slices."""
    torch = torch_cuda
    from ctbangbang_gb300 import structs
    spec = scans.ScanSpec(**{**scans.CONFIGS["config2"].__dict__})
    mr = scans.plan_spec(spec, str(tmp_path))
    L.call("ctbb_update_block_info", C.byref(mr))
    m = structs.ReconMetadata()
    C.memmove(C.byref(m), C.byref(mr), C.sizeof(m))
    n = spec.n_readings
    frame = m.cg.n_rows_raw * m.cg.n_channels
    P = m.ri.n_proj_pull
    d = H.dims(mr)
    ta = dev(torch, np.ctypeslib.as_array(mr.tube_angles, (n,)).copy())
    tp = dev(torch, np.ctypeslib.as_array(mr.table_positions, (n,)).copy())
    objs = ctbb_synth.phantom_objects(spec)
    d_raw = torch.empty(P * frame, dtype=torch.float32, device="cuda")
    ctbb_synth.project_device(m, objs, ta.data_ptr(), tp.data_ptr(), int(m.ri.idx_pull_start), P, spec.i0,
                         spec.seed, d_raw.data_ptr(), torch.cuda.current_stream().cuda_stream)
    d_filt = torch.empty_like(d_raw)
    L.call("ctbb_adaptive_filter_device", C.byref(m), ptr(d_raw), ptr(d_filt))
    del d_raw
    d_rb = torch.empty(d["n_rebin"], dtype=torch.float32, device="cuda")
    L.call("ctbb_rebin_device", C.byref(m), ptr(d_filt), ptr(d_rb))
    del d_filt
    taps = H.taps_of(m)
    L.call("ctbb_ramp_filter_device", ptr(d_rb), d["n_views"] * m.cg.n_rows, m.cg.n_channels_oversampled, fptr(taps))
    d_blk = torch.empty(d["n_block"], dtype=torch.float32, device="cuda")
    L.call("ctbb_backproject_device", C.byref(m), ptr(d_rb), ptr(d_blk))
    torch.cuda.synchronize()
    rows = d_rb.cpu().numpy()
    got = d_blk.cpu().numpy().reshape(m.ri.n_slices_block, m.rp.ny, m.rp.nx)
    want = np.zeros(d["n_block"], np.float32)
    for x0, y0 in ((240, 240), (0, 240)):
        oracle_lib.oracle_backproject_patch(C.byref(m), fptr(rows), x0, x0 + 32, y0, y0 + 32, fptr(want))
        w = want.reshape(got.shape)[:, y0:y0 + 32, x0:x0 + 32]
        assert np.abs(w).max() > 0.005
        assert_hu(got[:, y0:y0 + 32, x0:x0 + 32], w)
    scans.free_plan(mr)


GEOMETRY_CASES = {
    "config2": ("config2", {}),
    "config3": ("config3", {"turns": 6.0, "n_slices": 32}),  # block 0 only
    # 6 half turns per window: the pi' drift of p grows with the half turn
    "config2_pitch0.5": ("config2", {"pitch": 0.5, "turns": 14.0}),
    "config2_in_offset": ("config2", {"table_dir": "in", "x_origin": 40.0, "y_origin": -25.0,
                                      "tube_start_angle": 45.0}),
}


@pytest.mark.parametrize("case", list(GEOMETRY_CASES))
def test_config_geometry_backprojection(torch_cuda, oracle_lib, lib, tmp_path, case):
    """Backprojection of block 0 with the config-2 scanner and helix (1472 x 64
    rebinned rows, 1152 views/turn, phi+z FFS, pitch 0.8, 4 half turns per
    window), config 3's (1472 x 128 rows, 3 half turns), config 2 at pitch 0.5
    (6 half turns) or with the table moving in, an off-centre field and a 45
    degree tube start, over the full 500 mm field at 64^2 pixels: the rows
    the benchmarks read, including the flat (|q| <= Q) chunks that only
    detectors of 8 or more rows take.  The filtered rows come from the device
    stages (checked against the oracle on the small scans above); the oracle
    backprojects the same rows."""
    torch = torch_cuda
    from ctbangbang_gb300 import structs
    config, changes = GEOMETRY_CASES[case]
    spec = scans.ScanSpec(**{**scans.CONFIGS[config].__dict__})
    spec.nx = spec.ny = 64
    for k, v in changes.items():
        setattr(spec, k, v)
    mr = scans.plan_spec(spec, str(tmp_path))
    L.call("ctbb_update_block_info", C.byref(mr))
    m = structs.ReconMetadata()
    C.memmove(C.byref(m), C.byref(mr), C.sizeof(m))
    n = spec.n_readings
    frame = m.cg.n_rows_raw * m.cg.n_channels
    P = m.ri.n_proj_pull
    nv = P // m.ri.n_ffs - 2 * m.cg.add_projections
    ta = dev(torch, np.ctypeslib.as_array(mr.tube_angles, (n,)).copy())
    tp = dev(torch, np.ctypeslib.as_array(mr.table_positions, (n,)).copy())
    objs = ctbb_synth.phantom_objects(spec)
    d_raw = torch.empty(P * frame, dtype=torch.float32, device="cuda")
    ctbb_synth.project_device(m, objs, ta.data_ptr(), tp.data_ptr(), int(m.ri.idx_pull_start), P, spec.i0,
                         spec.seed, d_raw.data_ptr(), torch.cuda.current_stream().cuda_stream)
    d_filt = torch.empty_like(d_raw)
    L.call("ctbb_adaptive_filter_device", C.byref(m), ptr(d_raw), ptr(d_filt))
    del d_raw
    d_rb = torch.empty(nv * m.cg.n_rows * m.cg.n_channels_oversampled, dtype=torch.float32, device="cuda")
    L.call("ctbb_rebin_device", C.byref(m), ptr(d_filt), ptr(d_rb))
    del d_filt
    taps = H.taps_of(m)
    L.call("ctbb_ramp_filter_device", ptr(d_rb), nv * m.cg.n_rows, m.cg.n_channels_oversampled, fptr(taps))
    n_block = m.rp.nx * m.rp.ny * m.ri.n_slices_block
    d_blk = torch.empty(n_block, dtype=torch.float32, device="cuda")
    L.call("ctbb_backproject_device", C.byref(m), ptr(d_rb), ptr(d_blk))
    torch.cuda.synchronize()
    rows = d_rb.cpu().numpy()
    want = np.zeros(n_block, np.float32)
    oracle_lib.oracle_backproject_range(C.byref(m), fptr(rows), 0, m.cg.n_proj_turn // 2, fptr(want))
    got = d_blk.cpu().numpy()
    assert np.abs(want).max() > 0.01  # the phantom is in the field
    assert_hu(got, want)
    scans.free_plan(mr)


@pytest.mark.parametrize("n_os", [1025, 1472, 2048])
def test_ramp_filter_4096_point_rows(torch_cuda, oracle_lib, n_os):
    """Row lengths 1025..2048 take the 4096-point transform: the edge lengths
    and the config-2 length, an odd number of rows (the last transform carries
    one row), against the oracle's double-precision FFT convolution."""
    torch = torch_cuda
    rng = np.random.default_rng(n_os)
    n_lines = 301
    rows = rng.standard_normal((n_lines, n_os)).astype(np.float32)
    taps = np.zeros(2 * n_os, np.float32)
    L.call("ctbb_ramp_filter_taps", n_os, C.c_float(0.3), C.c_float(1.0), C.c_float(1.0), fptr(taps))
    d = dev(torch, rows.ravel())
    L.call("ctbb_ramp_filter_device", ptr(d), n_lines, n_os, fptr(taps))
    torch.cuda.synchronize()
    want = rows.copy()
    oracle_lib.oracle_filter_rows(fptr(want), n_lines, n_os, fptr(taps))
    assert_filter_close(d.cpu().numpy().reshape(n_lines, n_os), want)


@pytest.mark.parametrize("strength", [0.0, 2.0])
def test_whole_scan_path_vs_block_loop(torch_cuda, lib, tmp_path, strength):
    """ctbb_reconstruct_scan_device (one resident rebinned scan) against the
    block loop on a multi-block scan.  The views each block reads from frames
    near its window's ends are re-made from the block's own window (the
    adaptive filter's statistics stop there), so with or without the filter
    the two differ only by the rounding of the rebin's view coordinate (the
    union's split form against each block's float expression)."""
    torch = torch_cuda
    spec = scans.tiny(1, 1, adaptive_filtration=strength, n_slices=14, slice_thickness=2.5, seed=43)
    scan = H.Scan(spec, str(tmp_path))
    mr = scan.mr
    assert mr.ri.n_blocks >= 2
    n_final = lib.ctbb_n_slices_final(C.byref(mr))
    plane = mr.rp.nx * mr.rp.ny
    d_scan = dev(torch, scan.frames.reshape(-1))
    d_a = torch.empty(n_final * plane, dtype=torch.float32, device="cuda")
    d_b = torch.empty_like(d_a)
    L.call("ctbb_reconstruct_device", C.byref(mr), ptr(d_scan), ptr(d_a), 0.0)
    L.call("ctbb_reconstruct_scan_device", C.byref(mr), ptr(d_scan), ptr(d_b), 0.0)
    mx, rms = H.hu_errors(d_b.cpu().numpy(), d_a.cpu().numpy())
    print("whole scan vs block loop, adaptive %.1f: max %.4f HU, rms %.5f HU" % (strength, mx, rms))
    assert mx <= 0.02 and rms <= 0.002, (mx, rms)
    scan.close()


def test_whole_scan_streamed_from_host_equals_device_path(torch_cuda, lib, tmp_path):
    """The streamed host path runs the same kernels on the same data as the
    device whole-scan path, only scheduled as the chunks arrive: bit-exact.
    Another scan runs first so that no work buffer holds this scan's data."""
    torch = torch_cuda
    other = H.Scan(scans.tiny(1, 1, adaptive_filtration=2.0, n_slices=14, slice_thickness=2.5, seed=44),
                   str(tmp_path / "other"))
    spec = scans.tiny(1, 1, adaptive_filtration=2.0, n_slices=14, slice_thickness=2.5, seed=45)
    scan = H.Scan(spec, str(tmp_path / "scan"))
    mr = scan.mr
    assert mr.ri.n_blocks >= 2
    n_final = lib.ctbb_n_slices_final(C.byref(mr))
    plane = mr.rp.nx * mr.rp.ny
    d_other = dev(torch, other.frames.reshape(-1))
    d_junk = torch.empty(lib.ctbb_n_slices_final(C.byref(other.mr)) * plane, dtype=torch.float32, device="cuda")
    L.call("ctbb_reconstruct_scan_device", C.byref(other.mr), ptr(d_other), ptr(d_junk), 0.0)
    torch.cuda.synchronize()
    h_scan = np.ascontiguousarray(scan.frames.reshape(-1), dtype=np.float32)
    h_final = np.zeros(n_final * plane, np.float32)
    L.call("ctbb_reconstruct_scan_host", C.byref(mr), fptr(h_scan), fptr(h_final), 0.0)
    d_scan = dev(torch, h_scan)
    d_fin = torch.empty(n_final * plane, dtype=torch.float32, device="cuda")
    L.call("ctbb_reconstruct_scan_device", C.byref(mr), ptr(d_scan), ptr(d_fin), 0.0)
    np.testing.assert_array_equal(h_final, d_fin.cpu().numpy())
    other.close()
    scan.close()


def test_release_workspace_then_reconstruct_again(torch_cuda, lib, tmp_path):
    """ctbb_release_workspace frees every cached buffer, table, stream and
    event and unbinds the device; the next call rebuilds them and gives the
    same stack, on the block loop and on the streamed whole-scan path."""
    torch = torch_cuda
    spec = scans.tiny(1, 1, adaptive_filtration=2.0, n_slices=14, slice_thickness=2.5, seed=46)
    scan = H.Scan(spec, str(tmp_path))
    mr = scan.mr
    n_final = lib.ctbb_n_slices_final(C.byref(mr))
    plane = mr.rp.nx * mr.rp.ny
    d_scan = dev(torch, scan.frames.reshape(-1))
    h_scan = np.ascontiguousarray(scan.frames.reshape(-1), dtype=np.float32)
    first = torch.empty(n_final * plane, dtype=torch.float32, device="cuda")
    L.call("ctbb_reconstruct_device", C.byref(mr), ptr(d_scan), ptr(first), 0.0)
    h_first = np.zeros(n_final * plane, np.float32)
    L.call("ctbb_reconstruct_scan_host", C.byref(mr), fptr(h_scan), fptr(h_first), 0.0)
    torch.cuda.synchronize()
    L.call("ctbb_release_workspace")
    again = torch.empty_like(first)
    L.call("ctbb_reconstruct_device", C.byref(mr), ptr(d_scan), ptr(again), 0.0)
    h_again = np.zeros_like(h_first)
    L.call("ctbb_reconstruct_scan_host", C.byref(mr), fptr(h_scan), fptr(h_again), 0.0)
    np.testing.assert_array_equal(again.cpu().numpy(), first.cpu().numpy())
    np.testing.assert_array_equal(h_again, h_first)
    scan.close()


def test_whole_scan_from_raw_file_equals_device_path(torch_cuda, lib, tmp_path):
    """ctbb_reconstruct_scan_file reads the plan's raw file in chunks on a
    reader thread while the earlier chunks are processed: the same stack as
    the device whole-scan path on the same frames, bit for bit.  The file is
    cut 700 frames short, inside the last pull window, so the frames past its
    end must read as zeros."""
    torch = torch_cuda
    spec = scans.tiny(1, 1, adaptive_filtration=2.0, n_slices=14, slice_thickness=2.5, seed=47)
    scan = H.Scan(spec, str(tmp_path))
    mr = scan.mr
    frames = scan.frames.reshape(spec.n_readings, -1).copy()
    keep = spec.n_readings - 700
    scans.write_raw(os.path.join(str(tmp_path), "scan.raw"), frames[:keep])
    frames[keep:] = 0.0
    n_final = lib.ctbb_n_slices_final(C.byref(mr))
    plane = mr.rp.nx * mr.rp.ny
    h_file = np.zeros(n_final * plane, np.float32)
    L.call("ctbb_reconstruct_scan_file", C.byref(mr), fptr(h_file), 0.0)
    s_last = int(mr.ri.idx_pull_start)  # the last block's window after the call
    assert s_last < keep < s_last + mr.ri.n_proj_pull
    d_scan = dev(torch, frames.reshape(-1))
    d_fin = torch.empty(n_final * plane, dtype=torch.float32, device="cuda")
    L.call("ctbb_reconstruct_scan_device", C.byref(mr), ptr(d_scan), ptr(d_fin), 0.0)
    np.testing.assert_array_equal(h_file, d_fin.cpu().numpy())
    # a second call reuses the staging buffers
    h_again = np.zeros_like(h_file)
    L.call("ctbb_reconstruct_scan_file", C.byref(mr), fptr(h_again), 0.0)
    np.testing.assert_array_equal(h_again, h_file)
    scan.close()
