"""Shared helpers of the test suite: scan set-up, numpy views of the
recon_metadata arrays, oracle and GPU block pipelines, HU error metrics."""
import ctypes as C
import os
import tempfile

import numpy as np

from ctbangbang_gb300 import lib as _lib
from ctbangbang_gb300 import scans

import ctbb_synth

HU_PER_MU = 1000.0 / scans.MU_WATER   # 1 HU = mu_water / 1000


def view(ptr, n, dtype=np.float32):
    return np.ctypeslib.as_array(ptr, (int(n),)) if n else np.zeros(0, dtype)


def dims(mr):
    P = mr.ri.n_proj_pull
    nv = P // mr.ri.n_ffs - 2 * mr.cg.add_projections
    return dict(
        P=P, n_raw=P * mr.cg.n_rows_raw * mr.cg.n_channels,
        n_views=nv, n_rebin=nv * mr.cg.n_rows * mr.cg.n_channels_oversampled,
        plane=mr.rp.nx * mr.rp.ny, n_image=mr.rp.nx * mr.rp.ny * mr.ri.n_slices_recon,
        n_block=mr.rp.nx * mr.rp.ny * mr.ri.n_slices_block,
    )


class Scan:
    """A planned scan with its projected raw data, ready for block calls."""

    def __init__(self, spec, workdir=None, noise=True):
        self.spec = spec
        self._tmp = None
        if workdir is None:
            self._tmp = tempfile.TemporaryDirectory(prefix="ctbb_test_")
            workdir = self._tmp.name
        self.workdir = workdir
        self.prm, self.install = scans.prepare(spec, workdir)
        self.mr = scans.plan(self.prm, self.install)
        self.objects = ctbb_synth.phantom_objects(spec)
        self.frames = ctbb_synth.project_host(self.mr, self.objects, 0, spec.n_readings,
                                         spec.i0 if noise else 0.0, spec.seed)
        scans.write_raw(os.path.join(workdir, "scan.raw"), self.frames)

    def next_block(self):
        """update_block_info + fill ctd.raw from the projected frames
        (frames outside the data read as zeros)."""
        _lib.call("ctbb_update_block_info", C.byref(self.mr))
        d = dims(self.mr)
        raw = view(self.mr.ctd.raw, d["n_raw"]).reshape(d["P"], -1)
        s = int(self.mr.ri.idx_pull_start)
        if s >= 2 ** 63:  # a pull window starting before frame 0 is stored wrapped
            s -= 2 ** 64
        raw[:] = 0
        lo, hi = max(s, 0), min(s + d["P"], self.spec.n_readings)
        if hi > lo:
            raw[lo - s:hi - s] = self.frames[lo:hi].reshape(hi - lo, -1)
        return raw.reshape(-1).copy()

    def set_raw(self, values):
        d = dims(self.mr)
        view(self.mr.ctd.raw, d["n_raw"])[:] = values

    def close(self):
        scans.free_plan(self.mr)
        if self._tmp is not None:
            self._tmp.cleanup()


def taps_of(mr):
    n = 2 * mr.cg.n_channels_oversampled
    t = (C.c_float * n)()
    _lib.call("ctbb_load_filter", C.byref(mr), t)
    return np.frombuffer(t, dtype=np.float32).copy()


def oracle_block(orc, scan, raw, adaptive=True):
    """Oracle (float, reference arithmetic) stages of the current block."""
    mr = scan.mr
    d = dims(mr)
    out = {}
    scan.set_raw(raw)
    if adaptive:
        orc.oracle_adaptive_filter(C.byref(mr))
    out["adaptive"] = view(mr.ctd.raw, d["n_raw"]).copy()
    orc.oracle_rebin(C.byref(mr))
    out["rebin"] = view(mr.ctd.rebin, d["n_rebin"]).copy()
    taps = taps_of(mr)
    rows = view(mr.ctd.rebin, d["n_rebin"])
    orc.oracle_filter_rows(rows.ctypes.data_as(C.POINTER(C.c_float)), d["n_views"] * mr.cg.n_rows,
                           mr.cg.n_channels_oversampled, taps.ctypes.data_as(C.POINTER(C.c_float)))
    out["filtered"] = rows.copy()
    img = view(mr.ctd.image, d["n_image"])
    off = (mr.ri.cb.block_idx - 1) * d["n_block"]
    img[off:off + d["n_block"]] = 0
    orc.oracle_backproject(C.byref(mr))
    out["block"] = img[off:off + d["n_block"]].copy()
    scan.set_raw(raw)
    return out


def hu_errors(a, b):
    """(max, rms) of a - b in HU."""
    diff = (np.asarray(a, np.float64) - np.asarray(b, np.float64)) * HU_PER_MU
    return float(np.abs(diff).max()), float(np.sqrt(np.mean(diff ** 2)))
