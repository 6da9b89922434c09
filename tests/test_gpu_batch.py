"""Many whole scans, one backprojection launch (ctbb_batch_* /
ctbb_reconstruct_batch_device): every stack equals its scan reconstructed
alone (ctbb_reconstruct_scan_device), within the rounding of another launch
shape -- the autotuner may pick a different slice chunking than the single
scan's default, and per-slice sums then run in another order (the launch-shape
test of the single-scan path bounds that at 0.01 HU)."""
import ctypes as C

import numpy as np
import pytest

from ctbangbang_gb300 import lib as L
from ctbangbang_gb300 import scans
from tests import helpers as H

pytestmark = pytest.mark.gpu

SHAPE_HU = 0.01


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _uneven_scans(tmp_path):
    """Scans differing in FFS mode, rows, image size, slices and turns: four
    whose pull windows (17-19 half turns at 96 views per turn) only the
    slice-chunk form holds, and three at 192 views per turn whose windows of
    3, 6 and 7 half turns run the column form (32 slices per thread at 3, 16
    from 5 by default; the autotuner may pick others)."""
    specs = [
        scans.tiny(0, 0, n_rows_raw=8, nx=32, ny=32, n_slices=8, seed=61, adaptive_filtration=1.0),
        scans.tiny(1, 1, n_rows_raw=4, nx=48, ny=48, n_slices=14, slice_thickness=2.5, seed=62,
                   adaptive_filtration=2.0),
        scans.tiny(0, 1, n_rows_raw=8, nx=32, ny=32, n_slices=40, seed=63, pitch=0.8),
        scans.tiny(1, 0, n_rows_raw=4, nx=64, ny=64, n_slices=6, seed=64),
        scans.tiny(1, 1, n_rows_raw=64, n_proj_turn=192, nx=32, ny=32, n_slices=14, slice_thickness=2.5,
                   seed=66, adaptive_filtration=2.0),
        scans.tiny(0, 1, n_rows_raw=32, n_proj_turn=192, nx=48, ny=48, n_slices=40, seed=67, pitch=0.8),
        scans.tiny(1, 0, n_rows_raw=16, n_proj_turn=192, nx=64, ny=64, n_slices=10, seed=68),
    ]
    return [H.Scan(sp, str(tmp_path / ("s%d" % i))) for i, sp in enumerate(specs)]


def _alone(torch, lib, scan):
    mr = scan.mr
    n_final = lib.ctbb_n_slices_final(C.byref(mr))
    d = torch.from_numpy(np.ascontiguousarray(scan.frames.reshape(-1))).cuda()
    out = torch.empty(n_final * mr.rp.nx * mr.rp.ny, dtype=torch.float32, device="cuda")
    L.call("ctbb_reconstruct_scan_device", C.byref(mr), C.c_void_p(d.data_ptr()), C.c_void_p(out.data_ptr()),
           C.c_float(0.0))
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("storage", ["fp32", "fp16"])
def test_batch_equals_each_scan_alone(torch_cuda, lib, tmp_path, storage):
    torch = torch_cuda
    mode = L.STORAGE_FP32 if storage == "fp32" else L.STORAGE_FP16
    batch = _uneven_scans(tmp_path)
    L.call("ctbb_set_storage", mode)
    try:
        alone = [_alone(torch, lib, s) for s in batch]
        d_scans = [torch.from_numpy(np.ascontiguousarray(s.frames.reshape(-1))).cuda() for s in batch]
        d_finals = [torch.empty(a.size, dtype=torch.float32, device="cuda") for a in alone]
        n = len(batch)
        mrs = (C.POINTER(type(batch[0].mr)) * n)(*[C.pointer(s.mr) for s in batch])
        scans_p = (C.c_void_p * n)(*[t.data_ptr() for t in d_scans])
        finals_p = (C.c_void_p * n)(*[t.data_ptr() for t in d_finals])
        L.call("ctbb_reconstruct_batch_device", n, mrs, scans_p, finals_p, C.c_float(0.0))
        torch.cuda.synchronize()
        for i, (a, d) in enumerate(zip(alone, d_finals)):
            mx, rms = H.hu_errors(d.cpu().numpy(), a)
            print("%s scan %d: batch vs alone max %.5f HU rms %.6f HU" % (storage, i, mx, rms))
            assert mx <= SHAPE_HU, (i, mx, rms)
        # the step form, twice in a row (slots reused), gives the same stacks
        for _ in range(2):
            L.call("ctbb_batch_begin")
            outs = [torch.full_like(t, -1.0) for t in d_finals]
            for s, d, o in zip(batch, d_scans, outs):
                L.call("ctbb_batch_add_device", C.byref(s.mr), C.c_void_p(d.data_ptr()), C.c_void_p(o.data_ptr()),
                       C.c_float(0.0))
            L.call("ctbb_batch_run")
            torch.cuda.synchronize()
            for o, d in zip(outs, d_finals):
                assert torch.equal(o, d)
    finally:
        L.call("ctbb_set_storage", L.STORAGE_FP32)
        for s in batch:
            s.close()
    buf = C.create_string_buffer(1 << 16)
    n_report = lib.ctbb_autotune_report(buf, len(buf))
    assert n_report > 0 and b"zpt" in buf.value


def test_autotuned_single_scan_path_matches_default_shape(torch_cuda, lib, tmp_path):
    """ctbb_set_autotune(1): the single-scan device path takes the tuned shape
    per geometry class; the stack stays within the shape-rounding bar.  The
    window (4 half turns at 192 views per turn) lets every candidate run."""
    torch = torch_cuda
    scan = H.Scan(scans.tiny(1, 1, n_rows_raw=32, n_proj_turn=192, nx=48, ny=48, n_slices=14, slice_thickness=2.5,
                             seed=65, adaptive_filtration=1.0), str(tmp_path))
    ref = _alone(torch, lib, scan)
    L.call("ctbb_set_autotune", 1)
    try:
        tuned = _alone(torch, lib, scan)
        again = _alone(torch, lib, scan)
    finally:
        L.call("ctbb_set_autotune", 0)
    mx, rms = H.hu_errors(tuned, ref)
    assert mx <= SHAPE_HU, (mx, rms)
    np.testing.assert_array_equal(tuned, again)
    scan.close()
