"""The whole-scan path against the reference's block loop at the full size of
the precision workload: 736 channels x 64 raw rows with phi+z flying focal
spot (rebinned 1472 x 128), 1152 views/turn, pitch 0.8, 40 turns, 512^2 x 400
slices of 0.6 mm in 13 blocks of 32, adaptive raw filter on.

The block loop (ctbb_reconstruct_device) filters and rebins every block's own
pull window as the reference does (src/main.cu:207-245); the whole-scan path
(ctbb_reconstruct_scan_device) filters and rebins the union of the windows
once and re-makes, per block, the views whose frames lie within the adaptive
filter's statistics reach of the block's window ends.  Every one of the 13
blocks has such edges (all but the first two and last two at both ends), so
the stack covers each of them."""
import ctypes as C

import pytest

from ctbangbang_gb300 import lib as L
from ctbangbang_gb300 import scans

import ctbb_synth
from tests.helpers import HU_PER_MU

pytestmark = pytest.mark.gpu

# The two paths compute the block-interior views from the same filtered
# frames; they differ only in the float rounding of the rebin's view
# coordinate, which the union takes from its own (longer) window.
WHOLE_VS_BLOCKS_MAX_HU = 0.25
WHOLE_VS_BLOCKS_RMS_HU = 0.01


@pytest.fixture(scope="module")
def config3(tmp_path_factory):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = L.load()
    spec = scans.CONFIGS["config3"]
    wd = str(tmp_path_factory.mktemp("config3"))
    mr = scans.plan_spec(spec, wd)
    d_scan = ctbb_synth.project_scan_device(torch, mr, spec)
    torch.cuda.synchronize()
    yield torch, lib, spec, mr, d_scan
    del d_scan
    scans.free_plan(mr)
    L.call("ctbb_release_workspace")
    torch.cuda.empty_cache()


def test_config3_whole_scan_vs_block_loop_every_block(config3):
    torch, lib, spec, mr, d_scan = config3
    assert mr.ri.n_blocks == 13
    plane = mr.rp.nx * mr.rp.ny
    n_final = lib.ctbb_n_slices_final(C.byref(mr))
    d_blocks = torch.empty(n_final * plane, dtype=torch.float32, device="cuda")
    d_whole = torch.empty_like(d_blocks)
    L.call("ctbb_reconstruct_device", C.byref(mr), C.c_void_p(d_scan.data_ptr()),
           C.c_void_p(d_blocks.data_ptr()), C.c_float(0.0))
    L.call("ctbb_reconstruct_scan_device", C.byref(mr), C.c_void_p(d_scan.data_ptr()),
           C.c_void_p(d_whole.data_ptr()), C.c_float(0.0))
    torch.cuda.synchronize()
    diff = ((d_whole - d_blocks).double() * HU_PER_MU).reshape(n_final, plane)
    per_slice = diff.abs().amax(dim=1).cpu().numpy()
    mx = float(per_slice.max())
    rms = float(diff.pow(2).mean().sqrt())
    # the largest difference per group of 32 final slices (one block's slab)
    groups = [float(per_slice[k:k + 32].max()) for k in range(0, n_final, 32)]
    print("config 3 whole scan vs block loop: max %.4f HU, rms %.5f HU; per 32 slices %s"
          % (mx, rms, " ".join("%.3f" % g for g in groups)))
    assert bool(torch.isfinite(d_whole).all())
    assert mx <= WHOLE_VS_BLOCKS_MAX_HU and rms <= WHOLE_VS_BLOCKS_RMS_HU, (mx, rms)


def test_config3_streamed_host_path_equals_device_path(config3):
    """The streamed host path patches the same edge views, once each block's
    whole window has arrived: the device path's stack bit for bit."""
    torch, lib, spec, mr, d_scan = config3
    plane = mr.rp.nx * mr.rp.ny
    n_final = lib.ctbb_n_slices_final(C.byref(mr))
    d_whole = torch.empty(n_final * plane, dtype=torch.float32, device="cuda")
    L.call("ctbb_reconstruct_scan_device", C.byref(mr), C.c_void_p(d_scan.data_ptr()),
           C.c_void_p(d_whole.data_ptr()), C.c_float(0.0))
    h_scan = torch.empty(d_scan.numel(), dtype=torch.float32, pin_memory=True)
    h_scan.copy_(d_scan)
    h_final = torch.empty(n_final * plane, dtype=torch.float32, pin_memory=True)
    fptr = lambda t: t.numpy().ctypes.data_as(C.POINTER(C.c_float))
    L.call("ctbb_reconstruct_scan_host", C.byref(mr), fptr(h_scan), fptr(h_final), C.c_float(0.0))
    torch.cuda.synchronize()
    assert torch.equal(h_final.cuda(), d_whole)
