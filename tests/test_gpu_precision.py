"""The reduced-storage path: the ramp filter as an FP16 hi/lo Toeplitz
contraction on the tensor cores with FP16 output rows and a per-row scale,
checked against the FP64 oracle's filter (the reference's convolution,
src/rebin_filter_cpu.cu:647-709, in double).

Bar per sample: |y - y64| <= 2^-10 |y64| + 1e-4 max|y64 of the row| -- the
FP16 rounding of the stored value (at most 2^-11 relative) plus the hi/lo
products' and the tensor cores' FP32 accumulation error."""
import ctypes as C

import numpy as np
import pytest

from ctbangbang_gb300 import lib as L

pytestmark = pytest.mark.gpu

REL, ROW = 2.0 ** -10, 1e-4


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def tc_filter(torch, rows, taps, rows_per_view=0):
    """(filtered rows as float64, stored FP16 values, scales)."""
    n_lines, n = rows.shape
    d = torch.from_numpy(np.ascontiguousarray(rows, np.float32)).cuda()
    width = 4 if rows_per_view else 1
    out = torch.empty(n_lines * n * width, dtype=torch.float16, device="cuda")
    scale = torch.empty(n_lines, dtype=torch.float32, device="cuda")
    L.call("ctbb_ramp_filter_fp16_device", C.c_void_p(d.data_ptr()), n_lines, n, fptr(taps), rows_per_view,
           C.c_void_p(out.data_ptr()), C.c_void_p(scale.data_ptr()))
    torch.cuda.synchronize()
    stored = out.float().cpu().numpy().reshape(n_lines, n, width).astype(np.float64)
    sc = scale.cpu().numpy().astype(np.float64)
    assert np.all(sc > 0) and np.all(np.log2(sc) == np.round(np.log2(sc))), "scales are powers of two"
    return stored[:, :, 0] * sc[:, None], stored, sc


def fp64_filter(oracle_lib, rows, taps):
    want = np.ascontiguousarray(rows, np.float64).copy()
    oracle_lib.oracle64_filter_rows(want.ctypes.data_as(C.POINTER(C.c_double)), want.shape[0], want.shape[1],
                                    fptr(taps))
    return want


def assert_close(got, want):
    err = np.abs(got - want)
    bound = REL * np.abs(want) + ROW * np.abs(want).max(axis=1, keepdims=True)
    worst = float((err / bound).max())
    assert worst <= 1.0, ("worst error / bound", worst, float(err.max()))
    return worst


@pytest.mark.parametrize("n_os", [1472, 1344, 128])
def test_tensor_core_ramp_filter_vs_fp64(torch_cuda, lib, oracle_lib, n_os):
    """Random rows (white noise plus a smooth projection-like bump) of the
    row lengths of the built-in scanners with flying focal spot and a short
    one; 300 rows, so the last 128-row tile is partial."""
    rng = np.random.default_rng(n_os)
    n_lines = 300
    ch = np.arange(n_os)
    bump = 3.0 * np.clip(1.0 - ((ch - n_os / 2) / (0.4 * n_os)) ** 2, 0, None)
    rows = (bump[None, :] * rng.uniform(0.5, 1.5, (n_lines, 1)) +
            0.05 * rng.standard_normal((n_lines, n_os))).astype(np.float32)
    taps = np.zeros(2 * n_os, np.float32)
    L.call("ctbb_ramp_filter_taps", n_os, C.c_float(0.352), C.c_float(1.0), C.c_float(1.0), fptr(taps))
    got, _, _ = tc_filter(torch_cuda, rows, taps)
    want = fp64_filter(oracle_lib, rows, taps)
    worst = assert_close(got, want)
    print("n_os %d: worst error / bound %.3f" % (n_os, worst))


def test_tensor_core_ramp_filter_zero_and_single_rows(torch_cuda, lib, oracle_lib):
    """An all-zero row stays zero (scale 1); a single row and an impulse row
    reproduce the taps."""
    n_os = 1472
    taps = np.zeros(2 * n_os, np.float32)
    L.call("ctbb_ramp_filter_taps", n_os, C.c_float(0.352), C.c_float(1.0), C.c_float(1.0), fptr(taps))
    rows = np.zeros((3, n_os), np.float32)
    rows[1, 700] = 1.0
    rows[2] = np.linspace(0.0, 2.0, n_os, dtype=np.float32)
    got, _, _ = tc_filter(torch_cuda, rows, taps)
    assert np.all(got[0] == 0.0)
    want = fp64_filter(oracle_lib, rows, taps)
    assert_close(got[1:], want[1:])


@pytest.mark.parametrize("rpv", [64, 128])
def test_tensor_core_ramp_filter_footprint_quads(torch_cuda, lib, oracle_lib, rpv):
    """The footprint layout: every row of a view shares one scale, and word
    (r, c) holds samples (r, c), (r, c+1), (r+1, c), (r+1, c+1) of the view --
    zeros past its last row or channel -- each within the bar of the FP64
    filter."""
    n_os = 1472
    n_views = 3
    n_lines = n_views * rpv
    rng = np.random.default_rng(rpv)
    ch = np.arange(n_os)
    bump = 3.0 * np.clip(1.0 - ((ch - n_os / 2) / (0.4 * n_os)) ** 2, 0, None)
    rows = (bump[None, :] * rng.uniform(0.2, 1.5, (n_lines, 1)) +
            0.05 * rng.standard_normal((n_lines, n_os))).astype(np.float32)
    taps = np.zeros(2 * n_os, np.float32)
    L.call("ctbb_ramp_filter_taps", n_os, C.c_float(0.352), C.c_float(1.0), C.c_float(1.0), fptr(taps))
    _, q, sc = tc_filter(torch_cuda, rows, taps, rows_per_view=rpv)
    want = fp64_filter(oracle_lib, rows, taps).reshape(n_views, rpv, n_os)
    q = q.reshape(n_views, rpv, n_os, 4)
    sc = sc.reshape(n_views, rpv)
    assert np.all(sc == sc[:, :1]), "one scale per view"
    s = sc[:, 0][:, None, None]
    assert_close((q[:, :, :, 0] * s).reshape(-1, n_os), want.reshape(-1, n_os))
    assert_close((q[:, :, :-1, 1] * s).reshape(-1, n_os - 1), want[:, :, 1:].reshape(-1, n_os - 1))
    assert_close((q[:, :-1, :, 2] * s).reshape(-1, n_os), want[:, 1:, :].reshape(-1, n_os))
    assert_close((q[:, :-1, :-1, 3] * s).reshape(-1, n_os - 1), want[:, 1:, 1:].reshape(-1, n_os - 1))
    assert np.all(q[:, :, -1, 1] == 0) and np.all(q[:, -1, :, 2:] == 0)


def _whole_scan(torch, mr, frames, storage, host=False):
    from ctbangbang_gb300 import lib as LL
    lib = LL.load()
    plane = mr.rp.nx * mr.rp.ny
    n_final = lib.ctbb_n_slices_final(C.byref(mr))
    L.call("ctbb_set_storage", storage)
    try:
        if host:
            h_scan = np.ascontiguousarray(frames.reshape(-1), dtype=np.float32)
            out = np.zeros(n_final * plane, np.float32)
            L.call("ctbb_reconstruct_scan_host", C.byref(mr), fptr(h_scan), fptr(out), C.c_float(0.0))
            return out
        d_scan = torch.from_numpy(np.ascontiguousarray(frames.reshape(-1), dtype=np.float32)).cuda()
        d_fin = torch.empty(n_final * plane, dtype=torch.float32, device="cuda")
        L.call("ctbb_reconstruct_scan_device", C.byref(mr), C.c_void_p(d_scan.data_ptr()),
               C.c_void_p(d_fin.data_ptr()), C.c_float(0.0))
        torch.cuda.synchronize()
        return d_fin.cpu().numpy()
    finally:
        L.call("ctbb_set_storage", L.STORAGE_FP32)


@pytest.mark.parametrize("mode", [(0, 0), (1, 1)], ids=["no_ffs", "phi_z_ffs"])
def test_fp16_storage_whole_scan_vs_fp64_oracle(torch_cuda, lib, oracle_lib, tmp_path, mode):
    """The reduced-storage whole scan (tensor-core filter, FP16 footprint rows,
    FP32 accumulation) of a one-block scan against the FP64 oracle of that
    block, finalized in double: within 1 HU max and 0.1 HU RMS.  The float32
    whole scan of the same scan is reported beside it."""
    from ctbangbang_gb300 import scans
    from tests import helpers as H
    z, p = mode
    spec = scans.tiny(z, p, adaptive_filtration=2.0, n_rows_raw=8, seed=300 + 2 * z + p)
    scan = H.Scan(spec, str(tmp_path))
    mr = scan.mr
    assert mr.ri.n_blocks == 1
    fp16 = _whole_scan(torch_cuda, mr, scan.frames, L.STORAGE_FP16)
    fp32 = _whole_scan(torch_cuda, mr, scan.frames, L.STORAGE_FP32)
    mr.ri.cb.block_idx = 0  # the whole-scan call leaves the last block planned
    raw = scan.next_block()
    taps = H.taps_of(mr)
    d = H.dims(mr)
    block64 = np.zeros(d["n_block"], np.float64)
    oracle_lib.oracle64_block(C.byref(mr), raw.ctypes.data_as(C.POINTER(C.c_float)), 1, fptr(taps),
                              block64.ctypes.data_as(C.POINTER(C.c_double)))
    n_final = lib.ctbb_n_slices_final(C.byref(mr))
    final64 = np.zeros(n_final * d["plane"], np.float64)
    oracle_lib.oracle64_finalize(C.byref(mr), block64.ctypes.data_as(C.POINTER(C.c_double)),
                                 final64.ctypes.data_as(C.POINTER(C.c_double)))
    mx16, rms16 = H.hu_errors(fp16, final64)
    mx32, rms32 = H.hu_errors(fp32, final64)
    mxd, rmsd = H.hu_errors(fp16, fp32)
    print("FP16 rows vs FP64: max %.4f HU rms %.5f HU; FP32 rows vs FP64: max %.4f rms %.5f; FP16 vs FP32: "
          "max %.4f rms %.5f" % (mx16, rms16, mx32, rms32, mxd, rmsd))
    assert mx16 <= 1.0 and rms16 <= 0.1, (mx16, rms16)
    scan.close()


def test_fp16_storage_streamed_equals_device(torch_cuda, lib, tmp_path):
    """The streamed host path in FP16 storage filters the same rows chunk by
    chunk: the device path's stack bit for bit, on a multi-block scan."""
    from ctbangbang_gb300 import scans
    from tests import helpers as H
    spec = scans.tiny(1, 1, adaptive_filtration=2.0, n_slices=14, slice_thickness=2.5, seed=48)
    scan = H.Scan(spec, str(tmp_path))
    assert scan.mr.ri.n_blocks >= 2
    dev = _whole_scan(torch_cuda, scan.mr, scan.frames, L.STORAGE_FP16)
    host = _whole_scan(torch_cuda, scan.mr, scan.frames, L.STORAGE_FP16, host=True)
    np.testing.assert_array_equal(host, dev)
    scan.close()


def test_storage_mode_rejects_unknown_values(lib):
    st = lib.ctbb_set_storage(7)
    assert L.STATUS[st] == "CTBB_ERR_ARGUMENT"
