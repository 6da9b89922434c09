"""GPU tests of concurrent scans: contexts (ctbb_context_*) and the request
server (ctbb_server_*).  Every scan's result must be the same, bit for bit,
alone and in the mix: the same kernels run on the same data whatever runs
beside them."""
import ctypes as C
import threading

import numpy as np
import pytest

from ctbangbang_gb300 import lib as L
from ctbangbang_gb300 import scans
from ctbangbang_gb300.serving import Server
from tests import helpers as H

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def mixed_specs():
    """Scans of different FFS modes, sizes and block counts."""
    yield scans.tiny(1, 1, adaptive_filtration=2.0, n_slices=14, slice_thickness=2.5, seed=301)
    yield scans.tiny(0, 1, adaptive_filtration=2.0, nx=48, ny=40, seed=302)
    yield scans.tiny(1, 0, pitch=0.6, n_channels=96, seed=303)
    yield scans.tiny(0, 0, adaptive_filtration=3.0, n_slices=20, slice_thickness=1.5, seed=304)
    yield scans.tiny(1, 1, pitch=1.4, n_rows_raw=8, seed=305)


class Req:
    def __init__(self, spec, workdir):
        self.scan = H.Scan(spec, workdir)
        self.h_scan = np.ascontiguousarray(self.scan.frames.reshape(-1), dtype=np.float32)
        n_final = L.load().ctbb_n_slices_final(C.byref(self.scan.mr))
        self.h_final = np.full(n_final * self.scan.mr.rp.nx * self.scan.mr.rp.ny, np.nan, np.float32)

    def alone(self):
        out = np.zeros_like(self.h_final)
        L.call("ctbb_reconstruct_scan_host", C.byref(self.scan.mr), fptr(self.h_scan), fptr(out), 0.0)
        return out


@pytest.fixture
def requests(lib, tmp_path):
    reqs = [Req(spec, str(tmp_path / str(i))) for i, spec in enumerate(mixed_specs())]
    yield reqs
    for r in reqs:
        r.scan.close()


def test_contexts_run_concurrently_with_the_results_alone(torch_cuda, requests):
    want = [r.alone() for r in requests]
    ctxs = []
    for _ in requests:
        h = C.c_void_p()
        L.call("ctbb_context_create", C.byref(h))
        ctxs.append(h)
    errors = []

    def run(i):
        try:
            r = requests[i]
            for _ in range(2):  # the second run reuses the context's buffers
                L.call("ctbb_context_reconstruct_scan_host", ctxs[i], C.byref(r.scan.mr), fptr(r.h_scan),
                       fptr(r.h_final), 0.0)
        except Exception as e:  # reported below
            errors.append(e)

    threads = [threading.Thread(target=run, args=(i,)) for i in range(len(requests))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for r, w in zip(requests, want):
        np.testing.assert_array_equal(r.h_final, w)
    held = [L.load().ctbb_context_device_bytes(h) for h in ctxs]
    assert all(b > 0 for b in held)
    L.call("ctbb_context_release_workspace", ctxs[0])
    assert L.load().ctbb_context_device_bytes(ctxs[0]) == 0
    for h in ctxs:
        L.call("ctbb_context_destroy", h)


def test_server_results_equal_alone(torch_cuda, requests):
    want = [r.alone() for r in requests]
    with Server(n_workers=3, device_budget_bytes=8 << 30) as srv:
        tickets = [srv.submit(r.scan.mr, fptr(r.h_scan), fptr(r.h_final)) for r in requests]
        results = [srv.wait(t) for t in tickets]
    for r, w, res in zip(requests, want, results):
        np.testing.assert_array_equal(r.h_final, w)
        assert res.status == 0 and 0 <= res.worker < 3
        assert res.latency_ms >= res.run_ms > 0 and res.queue_ms >= 0
        assert res.device_bytes == L.load().ctbb_scan_workspace_bytes(C.byref(r.scan.mr))


def run_with_budget(requests, budget, n_workers=3):
    with Server(n_workers=n_workers, device_budget_bytes=budget) as srv:
        tickets = [srv.submit(r.scan.mr, fptr(r.h_scan), fptr(r.h_final)) for r in requests]
        return [srv.wait(t) for t in tickets]


def overlapping_sets(results):
    """For each request's start, the requests running at that moment (one
    clock: ms since the server was created)."""
    spans = [(res.start_ms, res.end_ms, res.device_bytes) for res in results]
    return [[s for s in spans if s[0] <= t0 < s[1]] for t0, _, _ in spans]


def test_server_budget_bounds_what_runs_together(torch_cuda, requests):
    """Budget = the largest scan's memory: one scan at a time.  Budget = the
    two largest: never more than that in flight.  Same stacks either way."""
    want = [r.alone() for r in requests]
    needs = sorted(L.load().ctbb_scan_workspace_bytes(C.byref(r.scan.mr)) for r in requests)
    for budget in (needs[-1], needs[-1] + needs[-2]):
        results = run_with_budget(requests, budget)
        for r, w in zip(requests, want):
            np.testing.assert_array_equal(r.h_final, w)
        for running in overlapping_sets(results):
            assert sum(b for _, _, b in running) <= budget, (budget, running)
            if budget == needs[-1]:
                assert len(running) == 1, running


def test_server_ticket_is_collected_once(torch_cuda, requests):
    r = requests[1]
    with Server(n_workers=2, device_budget_bytes=8 << 30) as srv:
        t = srv.submit(r.scan.mr, fptr(r.h_scan), fptr(r.h_final))
        assert srv.wait(t).status == 0
        with pytest.raises(L.CtbbError) as e:
            srv.wait(t)
    assert e.value.status_name == "CTBB_ERR_ARGUMENT"


def test_server_refuses_a_scan_over_the_budget(torch_cuda, requests):
    r = requests[0]
    need = L.load().ctbb_scan_workspace_bytes(C.byref(r.scan.mr))
    with Server(n_workers=1, device_budget_bytes=need - 1) as srv:
        with pytest.raises(L.CtbbError) as e:
            srv.submit(r.scan.mr, fptr(r.h_scan), fptr(r.h_final))
    assert e.value.status_name == "CTBB_ERR_ALLOC"


def test_server_isolates_a_failing_request(torch_cuda, requests, tmp_path):
    """A request that fails while it runs -- its plan names the sharp
    reconstruction kernel, whose filter file the scan's install directory
    lacks, so the whole-scan call fails after its first copies were enqueued
    -- returns its error and text; the requests around it are unaffected, and
    the failed call leaves the context usable."""
    bad = Req(scans.tiny(0, 0, recon_kernel=3, seed=306), str(tmp_path / "bad"))
    try:
        want = [r.alone() for r in requests]
        mix = requests[:2] + [bad] + requests[2:]
        with Server(n_workers=2, device_budget_bytes=8 << 30) as srv:
            tickets = [srv.submit(r.scan.mr, fptr(r.h_scan), fptr(r.h_final)) for r in mix]
            results = []
            for t in tickets:
                try:
                    results.append(srv.wait(t))
                except L.CtbbError as e:
                    results.append(e)
        err = results[2]
        assert isinstance(err, L.CtbbError) and err.status_name == "CTBB_ERR_IO", err
        assert "sharp" in str(err)
        for r, w, res in zip(requests, want, results[:2] + results[3:]):
            assert not isinstance(res, L.CtbbError), res
            np.testing.assert_array_equal(r.h_final, w)
        # the same failure on the library-wide context, then a good call
        with pytest.raises(L.CtbbError) as e:
            bad.alone()
        assert e.value.status_name == "CTBB_ERR_IO"
        np.testing.assert_array_equal(requests[0].alone(), want[0])
    finally:
        bad.scan.close()
