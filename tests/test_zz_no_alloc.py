"""The adaptive filter entry point that allocates nothing.

Some callers cannot allocate device memory while a scan is processed -- a
scanner-side service that reserves all device memory at start-up and keeps
cudaMalloc out of its per-scan path, or a process whose device memory belongs
to another allocator.  ctbb_adaptive_filter_device_noalloc serves them from a
fixed static device array.  This file is collected last (its name sorts after
the others) so a run that stops at the first failure has run everything else.
"""
import ctypes as C

import numpy as np
import pytest

from ctbangbang_gb300 import lib as L
from ctbangbang_gb300 import scans
from tests import helpers as H


def test_noalloc_rejects_windows_beyond_its_fixed_scratch(lib, tmp_path):
    scan = H.Scan(scans.tiny(0, 0, seed=71), str(tmp_path))
    scan.next_block()
    scan.mr.ri.n_proj_pull = 65536 + 128
    st = lib.ctbb_adaptive_filter_device_noalloc(C.byref(scan.mr), C.c_void_p(16), C.c_void_p(16))
    assert L.STATUS[st] == "CTBB_ERR_ARGUMENT"
    assert b"exceeds the fixed scratch" in lib.ctbb_last_error()
    scan.close()


@pytest.mark.gpu
def test_noalloc_matches_allocating_entry_point_on_consecutive_calls(lib, tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    # two different scans in a row: the second call reuses the static scratch
    # the first one filled
    for seed, (z, p) in ((72, (1, 1)), (73, (0, 1))):
        scan = H.Scan(scans.tiny(z, p, adaptive_filtration=3.0, seed=seed), str(tmp_path / str(seed)))
        raw = scan.next_block()
        mr = scan.mr
        d_in = torch.from_numpy(raw).cuda()
        want = torch.empty_like(d_in)
        got = torch.full_like(d_in, float("nan"))
        L.call("ctbb_adaptive_filter_device", C.byref(mr), C.c_void_p(d_in.data_ptr()),
               C.c_void_p(want.data_ptr()))
        L.call("ctbb_adaptive_filter_device_noalloc", C.byref(mr), C.c_void_p(d_in.data_ptr()),
               C.c_void_p(got.data_ptr()))
        torch.cuda.synchronize()
        w, g = want.cpu().numpy(), got.cpu().numpy()
        assert (w != raw).sum() > 0          # the filter changed samples
        np.testing.assert_array_equal(g, w)  # bit-exact, like every adaptive-filter test
        scan.close()
