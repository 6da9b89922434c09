"""GPU tests of the environment knobs (read once per process, so each setting
runs in its own process): the streamed whole-scan path gives the device
path's stack bit for bit at any number of copy chunks, and the
backprojector's forms and launch shapes agree with the default to
rounding."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

from tests.conftest import REPO

pytestmark = pytest.mark.gpu

CHILD = r"""
import ctypes as C, sys
import numpy as np
sys.path.insert(0, REPO)
from ctbangbang_gb300 import lib as L, scans
from tests import helpers as H
out, mode = sys.argv[1], sys.argv[2]
n_proj_turn, n_rows_raw = int(sys.argv[4]), int(sys.argv[5])
fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
spec = scans.tiny(1, 1, adaptive_filtration=2.0, n_slices=14, slice_thickness=2.5, seed=91,
                  n_proj_turn=n_proj_turn, n_rows_raw=n_rows_raw)
scan = H.Scan(spec, sys.argv[3])
mr = scan.mr
n_final = L.load().ctbb_n_slices_final(C.byref(mr))
h_scan = np.ascontiguousarray(scan.frames.reshape(-1), dtype=np.float32)
fin = np.zeros(n_final * mr.rp.nx * mr.rp.ny, np.float32)
L.call("ctbb_reconstruct_scan_host", C.byref(mr), fp(h_scan), fp(fin), 0.0)
np.save(out, fin)
"""


def run_child(tmp_path, name, env_extra, n_proj_turn=96, n_rows_raw=4):
    out = str(tmp_path / (name + ".npy"))
    work = tmp_path / ("w_" + name)
    work.mkdir()
    env = dict(os.environ, **env_extra)
    code = "REPO = %r\n" % REPO + CHILD
    r = subprocess.run([sys.executable, "-c", code, out, name, str(work), str(n_proj_turn), str(n_rows_raw)],
                       env=env, capture_output=True, text=True, timeout=600, cwd=REPO)
    assert r.returncode == 0, r.stderr[-3000:]
    return np.load(out)


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_streamed_path_any_chunk_count(torch_cuda, tmp_path):
    """1, 5 and 64 copy chunks (CTBB_SCAN_CHUNKS) against the default 8: the
    adaptive filter advances, rebin view ranges and block starts move, the
    stack does not."""
    want = run_child(tmp_path, "chunks8", {})
    assert np.abs(want).max() > 0.01
    for n in (1, 5, 64):
        np.testing.assert_array_equal(run_child(tmp_path, "chunks%d" % n, {"CTBB_SCAN_CHUNKS": str(n)}), want)


def window_half_turns(n_proj_turn, n_rows_raw, tmp_path):
    """Half turns in block 0's pull window of the child's scan (planner only)."""
    from ctbangbang_gb300 import lib as L, scans
    spec = scans.tiny(1, 1, adaptive_filtration=2.0, n_slices=14, slice_thickness=2.5, seed=91,
                      n_proj_turn=n_proj_turn, n_rows_raw=n_rows_raw)
    prm, install = scans.prepare(spec, str(tmp_path))
    mr = scans.plan(prm, install)
    L.call("ctbb_update_block_info", C.byref(mr))
    n_views = mr.ri.n_proj_pull // mr.ri.n_ffs - 2 * mr.cg.add_projections
    return n_views // (mr.cg.n_proj_turn // 2)


# (views per turn, raw detector rows, half turns of the window): windows the
# column form holds (at most 8 half turns), one where its default is 32 slices
# per thread at 8 CTAs per SM and one where it is 16 slices
WINDOWS = ((192, 64, 3), (192, 16, 6))


@pytest.mark.parametrize("n_proj_turn,n_rows_raw,nht", WINDOWS)
def test_backprojector_launch_shapes_agree(torch_cuda, tmp_path, n_proj_turn, n_rows_raw, nht):
    """Both backprojector forms and their launch shapes against the default
    (column form, 16 angle chunks, slices per thread and CTAs per SM by the
    window's width): other CTA / warp
    tilings, slices per thread and angle chunks change which sub-chunks a warp
    classes as flat, inner or other (whose row coordinates round differently)
    and the order of the angle sums, not the algorithm -- and since q of every
    slice is taken from the block's slice 0 in every form, not the |q| < 1
    decisions either: within 0.01 HU of the default."""
    assert window_half_turns(n_proj_turn, n_rows_raw, tmp_path) == nht
    child = lambda name, env: run_child(tmp_path, name, env, n_proj_turn, n_rows_raw)
    want = child("default", {})
    assert np.abs(want).max() > 0.01
    hu = 1000.0 / 0.019
    for name, env in (("a1", {"CTBB_BP_ACHUNKS": "1"}),
                      ("a4", {"CTBB_BP_ACHUNKS": "4"}),
                      ("z16", {"CTBB_BP_COL_ZPT": "16"}),
                      ("m7", {"CTBB_BP_MINB": "7"}),
                      ("z32m8", {"CTBB_BP_COL_ZPT": "32", "CTBB_BP_MINB": "8"}),
                      ("z16m8", {"CTBB_BP_COL_ZPT": "16", "CTBB_BP_MINB": "8"}),
                      ("z8", {"CTBB_BP_COL_ZPT": "8"}),
                      ("c32", {"CTBB_BP_CTA_W": "32"}),
                      ("w4c32", {"CTBB_BP_WARP_W": "4", "CTBB_BP_CTA_W": "32"}),
                      ("tile", {"CTBB_BP_FORM": "tile"}),
                      ("tile_t256", {"CTBB_BP_FORM": "tile", "CTBB_BP_THREADS": "256", "CTBB_BP_MINB": "4"}),
                      ("tile_z16", {"CTBB_BP_FORM": "tile", "CTBB_BP_ZPT": "16"})):
        got = child(name, env)
        diff = np.abs((got.astype(np.float64) - want) * hu).max()
        print("window of %d half turns, launch shape %s: max %.2e HU from the default" % (nht, name, diff))
        assert diff <= 0.01, name
