"""Benchmark of the helical weighted-FBP hot path on one (or N replica) GB300s.

A step is one full reconstruction of the config-2 scan (736 channels x 32
raw rows, phi+z flying focal spot rebinned to 1472 x 64, 1152 views/turn,
pitch 0.8, 10 turns, 512^2 x 96 raw slices in 3 blocks of 32, thickened to
16 final 3 mm slices): adaptive raw filter -> FFS rebin -> ramp filter ->
FP32 wFBP backprojection of every block, then reorder/thicken.  Input: a
seeded synthetic phantom scan (water cylinder + 30 ellipsoids, Poisson noise
at I0 = 5e4) generated on the device; there is no public dataset.

--path scan (default) runs the whole-scan entry points: the union of the
blocks' pull windows is filtered and rebinned once and every block is
backprojected from it.  --path blocks runs the reference's block loop (each
block's window filtered and rebinned on its own).  The line reports the other
path too ("other_path") with the HU difference between the two stacks.

  value  voxel-updates/s with the raw scan resident in HBM (device-timed with
         CUDA events on the library's stream); each step reads over 2 GB of
         raw input, more than L2, so no flush is needed between steps.
  e2e    the same metric through the host-buffer entry point from pinned host
         buffers: the raw frames are copied host->device and the final stack
         device->host inside the timed region.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import concurrent.futures as cf
import dataclasses
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import ctbb_synth  # noqa: E402  (synthetic scans and the FP32 peak probe)

FLOP_PER_VU = 13          # q FMA 2, q_idx FMA 2, bilinear 6, s += W v 2, h += W 1
STAGES = ["adaptive_filter", "rebin", "ramp_filter", "backproject", "finalize"]


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="config3",
                    help="headline workload (config3: the largest single-GPU configuration)")
    ap.add_argument("--beside", default="config2",
                    help="a second workload measured after the headline and reported beside it ('' for none)")
    ap.add_argument("--no-hu", action="store_true", help="skip the HU errors of the output against the oracle")
    ap.add_argument("--no-fp16", action="store_true",
                    help="skip the reduced-storage measurement (tensor-core ramp filter, FP16 footprint rows)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--file", action="store_true",
                    help="also time ctbb_reconstruct_scan_file on the scan written to the plan's raw file")
    ap.add_argument("--no-whole-scan", action="store_true",
                    help="skip the measurement of the other path (see --path)")
    ap.add_argument("--path", choices=["scan", "blocks"], default="scan",
                    help="scan: one resident rebinned scan for all blocks (ctbb_reconstruct_scan_*); "
                         "blocks: the reference's block loop (ctbb_reconstruct_device / _host)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-scans measurement")
    ap.add_argument("--batch-scans", type=int, default=24)
    ap.add_argument("--batch-budget-gb", type=float, default=100.0,
                    help="device bytes of rows a batch may hold before it runs")
    ap.add_argument("--no-serve", action="store_true",
                    help="skip the served-stream measurement (request server vs the plain per-scan path)")
    ap.add_argument("--serve-requests", type=int, default=600)
    ap.add_argument("--serve-scans", type=int, default=8,
                    help="distinct scans of the batched distribution the requests draw from (plus one large scan)")
    ap.add_argument("--serve-workers", type=int, default=3)
    ap.add_argument("--serve-window", type=int, default=16, help="requests in flight at most (output buffers)")
    ap.add_argument("--profile-case", action="store_true",
                    help="one block of the config through each stage once (small case for ncu captures)")
    return ap.parse_args()


# --------------------------------------------------------------------------
# plan and sizes
# --------------------------------------------------------------------------

def make_plan(spec, workdir):
    from ctbangbang_gb300 import scans
    prm, inst = scans.prepare(spec, workdir)
    return scans.plan(prm, inst)


def block_plans(mr):
    """recon_info of every block (the reference's update_block_info sequence)."""
    from ctbangbang_gb300 import lib as L
    from ctbangbang_gb300 import structs
    m = structs.ReconMetadata()
    C.memmove(C.byref(m), C.byref(mr), C.sizeof(m))
    m.ctd.raw = m.ctd.rebin = None
    m.ri.cb.block_idx = 0
    out = []
    for _ in range(mr.ri.n_blocks):
        L.call("ctbb_update_block_info", C.byref(m))
        ri = structs.ReconInfo()
        C.memmove(C.byref(ri), C.byref(m.ri), C.sizeof(ri))
        out.append(ri)
    import ctypes
    libc = ctypes.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    libc.free(C.cast(m.ctd.raw, C.c_void_p))
    libc.free(C.cast(m.ctd.rebin, C.c_void_p))
    return out


def max_over_ranks(ms, dist, device="cuda"):
    """The slowest rank's time: every replica's step ends when the last one does."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_seed(seed, rank):
    """Each replica reconstructs its own seeded scan."""
    return seed + 7919 * rank


def workload_text(name, spec, mr, n_blocks, n_final):
    """One line naming the workload by its sizes."""
    ffs = {(0, 0): "no FFS", (0, 1): "phi FFS", (1, 0): "z FFS", (1, 1): "phi+z FFS"}[(spec.z_ffs, spec.phi_ffs)]
    text = ("%s: %d ch x %d rows %s -> %d x %d, %d views/turn, pitch %.2g, %g turns, %d^2 x %d slices (%d blocks)"
            % (name, mr.cg.n_channels, mr.cg.n_rows_raw, ffs, mr.cg.n_channels_oversampled, mr.cg.n_rows,
               mr.cg.n_proj_turn, spec.pitch, spec.turns, mr.rp.nx, mr.ri.n_slices_recon, n_blocks))
    if n_final is not None:
        text += " thickened to %d x %g mm" % (n_final, spec.slice_thickness)
    return text + ("; adaptive filter on" if spec.adaptive_filtration > 0 else "")


def workload_sizes(mr, blocks):
    nht = [(ri.n_proj_pull // ri.n_ffs - 2 * mr.cg.add_projections) // (mr.cg.n_proj_turn // 2) for ri in blocks]
    plane = mr.rp.nx * mr.rp.ny
    vu_blocks = [plane * mr.ri.n_slices_block * (mr.cg.n_proj_turn // 2) * k for k in nht]
    frame = mr.cg.n_rows_raw * mr.cg.n_channels
    n_readings = mr.rp.n_readings
    h2d = 0
    g0 = g1 = None
    for ri in blocks:
        s = int(ri.idx_pull_start)
        s = s - 2 ** 64 if s >= 2 ** 63 else s
        a, e = max(s, 0), min(s + ri.n_proj_pull, n_readings)
        h2d += max(e - a, 0) * frame * 4
        g0 = s if g0 is None else min(g0, s)
        g1 = s + ri.n_proj_pull if g1 is None else max(g1, s + ri.n_proj_pull)
    union_h2d = max(min(g1, n_readings) - max(g0, 0), 0) * frame * 4
    n_ffs = blocks[0].n_ffs
    return dict(nht=nht, vu_per_block=vu_blocks, vu_total=sum(vu_blocks), h2d_bytes=h2d,
                union_h2d_bytes=union_h2d,
                union_raw_samples=(g1 - g0) * frame,
                union_rebin_samples=((g1 - g0) // n_ffs - 2 * mr.cg.add_projections) * mr.cg.n_rows *
                mr.cg.n_channels_oversampled,
                raw_samples=[ri.n_proj_pull * frame for ri in blocks],
                rebin_samples=[(ri.n_proj_pull // ri.n_ffs - 2 * mr.cg.add_projections) * mr.cg.n_rows *
                               mr.cg.n_channels_oversampled for ri in blocks])


# --------------------------------------------------------------------------
# clocks
# --------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.path = tempfile.mktemp(prefix="ctbb_clocks_", suffix=".csv")
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(gpu_index)], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        os.remove(self.path)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "samples": len(rows), "reasons": reasons}


# --------------------------------------------------------------------------
# The reference CPU path's arithmetic (the oracle port) on host threads
# --------------------------------------------------------------------------

def _ranges(n, parts):
    """[a, b) ranges splitting n items into `parts` nearly equal pieces."""
    parts = max(1, min(parts, n))
    edges = [n * i // parts for i in range(parts + 1)]
    return [(edges[i], edges[i + 1]) for i in range(parts) if edges[i + 1] > edges[i]]


def block_meta(mr, ri):
    """A copy of the plan whose recon_info is the given block's."""
    from ctbangbang_gb300 import structs
    m = structs.ReconMetadata()
    C.memmove(C.byref(m), C.byref(mr), C.sizeof(m))
    m.ri = ri
    m.ctd.raw = m.ctd.rebin = m.ctd.image = None
    return m


def n_views_of(mb):
    return mb.ri.n_proj_pull // mb.ri.n_ffs - 2 * mb.cg.add_projections


def oracle_rows(orc, mb, raw, taps, threads, views=None, double=False):
    """Ramp-filtered rebinned rows of one block from its raw window
    [P][R_raw][N] (float32): the adaptive filter of the whole window on one
    thread (the reference's own is one call per window), then the rebin of
    views [v0, v1) and their ramp filter split over `threads`.  float: the
    reference CPU path's arithmetic; double: the FP64 oracle.  Returns the rows
    [n_views][n_rows][n_os] (only [v0, v1) written) and the stage times (s)."""
    nv = n_views_of(mb)
    v0, v1 = views if views else (0, nv)
    R, N = mb.cg.n_rows, mb.cg.n_channels_oversampled
    D = C.POINTER(C.c_double)
    Fp = C.POINTER(C.c_float)
    taps_p = taps.ctypes.data_as(Fp)
    t = {}
    t0 = time.perf_counter()
    if double:
        filt = np.empty(raw.size, np.float64)
        orc.oracle64_adaptive_filter(C.byref(mb), raw.ctypes.data_as(Fp), filt.ctypes.data_as(D))
        rows = np.zeros(nv * R * N, np.float64)
    else:
        filt = np.ascontiguousarray(raw, np.float32).copy()
        mb.ctd.raw = filt.ctypes.data_as(Fp)
        orc.oracle_adaptive_filter(C.byref(mb))
        mb.ctd.raw = None
        rows = np.zeros(nv * R * N, np.float32)
    t["adaptive_filter"] = time.perf_counter() - t0
    view = R * N

    def rebin_part(r):
        if double:
            orc.oracle64_rebin_views(C.byref(mb), filt.ctypes.data_as(D), v0 + r[0], v0 + r[1],
                                     rows.ctypes.data_as(D))
        else:
            orc.oracle_rebin_views(C.byref(mb), filt.ctypes.data_as(Fp), v0 + r[0], v0 + r[1],
                                   rows.ctypes.data_as(Fp))

    def filter_part(r):
        off = (v0 * R + r[0]) * N
        if double:
            orc.oracle64_filter_rows(rows[off:].ctypes.data_as(D), r[1] - r[0], N, taps_p)
        else:
            orc.oracle_filter_rows(rows[off:].ctypes.data_as(Fp), r[1] - r[0], N, taps_p)

    with cf.ThreadPoolExecutor(threads) as ex:
        t0 = time.perf_counter()
        list(ex.map(rebin_part, _ranges(v1 - v0, 4 * threads)))
        t["rebin"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        list(ex.map(filter_part, _ranges((v1 - v0) * R, 4 * threads)))
        t["ramp_filter"] = time.perf_counter() - t0
    del filt
    assert view * nv == rows.size
    return rows, t


def oracle_patch(orc, mb, rows, patch, double=False):
    """Backprojection (all angles) of the pixels x in [x0, x1), y in [y0, y1)
    of one block from its filtered rows -> [n_slices_block][y1-y0][x1-x0]."""
    x0, x1, y0, y1 = patch
    nx, ny, nz = mb.rp.nx, mb.rp.ny, mb.ri.n_slices_block
    out = np.zeros(nz * ny * nx, np.float64 if double else np.float32)
    if double:
        D = C.POINTER(C.c_double)
        orc.oracle64_backproject_patch(C.byref(mb), rows.ctypes.data_as(D), x0, x1, y0, y1, out.ctypes.data_as(D))
    else:
        Fp = C.POINTER(C.c_float)
        orc.oracle_backproject_patch(C.byref(mb), rows.ctypes.data_as(Fp), x0, x1, y0, y1, out.ctypes.data_as(Fp))
    return out.reshape(nz, ny, nx)[:, y0:y1, x0:x1].copy()


def oracle_taps(orc, mb):
    taps = np.zeros(2 * mb.cg.n_channels_oversampled, np.float32)
    if orc.oracle_load_filter(C.byref(mb), taps.ctypes.data_as(C.POINTER(C.c_float))) != 0:
        raise RuntimeError("oracle: no reconstruction kernel file under %s" % mb.install_dir.decode())
    return taps


# A step of the CPU sample, on block 0 of the workload: the adaptive filter of
# 1/CPU_AF_PARTS of its pull window (one thread: the reference filters a
# window in one call), the rebin and ramp filter of 1/CPU_VIEW_PARTS of its
# views and the backprojection of 1/CPU_ANGLE_PARTS of its half-turn angles
# (every voxel of the block, all half turns), the last two over all host
# threads.  The block's time is composed as CPU_AF_PARTS t_af +
# CPU_VIEW_PARTS t_rebin+filter + CPU_ANGLE_PARTS t_bp, the scan's as the sum
# over its blocks (equal windows).  Each part is a different slice of the
# block from step to step.
CPU_AF_PARTS = 4
CPU_VIEW_PARTS = 32
CPU_ANGLE_PARTS = 64


def cpu_sample_step(orc, mb, raw, taps, threads, step):
    """One step of the CPU sample (see above); returns its stage times (s)."""
    from ctbangbang_gb300 import structs
    Fp = C.POINTER(C.c_float)
    t_step = time.perf_counter()
    t = {}
    # adaptive filter of a sub-window (whole focal-spot cycles)
    P, n_ffs = int(mb.ri.n_proj_pull), int(mb.ri.n_ffs)
    frame = mb.cg.n_rows_raw * mb.cg.n_channels
    sub = (P // CPU_AF_PARTS) // n_ffs * n_ffs
    f0 = ((step * sub) % max(P - sub, 1)) // n_ffs * n_ffs
    ms = structs.ReconMetadata()
    C.memmove(C.byref(ms), C.byref(mb), C.sizeof(ms))
    ms.ri.n_proj_pull = sub
    win = raw[f0 * frame:(f0 + sub) * frame].copy()
    ms.ctd.raw = win.ctypes.data_as(Fp)
    t0 = time.perf_counter()
    orc.oracle_adaptive_filter(C.byref(ms))
    t["adaptive_filter"] = time.perf_counter() - t0
    del win
    # rebin + ramp filter of a view range (from the unfiltered window: the
    # cost does not depend on the values)
    nv = n_views_of(mb)
    R, N = mb.cg.n_rows, mb.cg.n_channels_oversampled
    part = nv // CPU_VIEW_PARTS
    v0 = (step * part) % max(nv - part, 1)
    rows = np.zeros(nv * R * N, np.float32)
    raw_p = raw.ctypes.data_as(Fp)
    taps_p = taps.ctypes.data_as(Fp)

    def rebin_part(r):
        orc.oracle_rebin_views(C.byref(mb), raw_p, v0 + r[0], v0 + r[1], rows.ctypes.data_as(Fp))

    def filter_part(r):
        orc.oracle_filter_rows(rows[(v0 * R + r[0]) * N:].ctypes.data_as(Fp), r[1] - r[0], N, taps_p)

    n_half = mb.cg.n_proj_turn // 2
    n_ang = max(n_half // CPU_ANGLE_PARTS, 1)
    a0 = (step * n_ang) % max(n_half - n_ang, 1)
    plane_block = mb.rp.nx * mb.rp.ny * mb.ri.n_slices_block

    def bp(r):
        out = np.zeros(plane_block, np.float32)
        orc.oracle_backproject_range(C.byref(mb), rows.ctypes.data_as(Fp), a0 + r[0], a0 + r[1],
                                     out.ctypes.data_as(Fp))

    # the rebin's per-call set-up (the reference splits the window by focal
    # spot once per block, rebin_filter_cpu.cu:418-645): timed alone with a
    # call that rebins no view, and counted once per block
    t0 = time.perf_counter()
    orc.oracle_rebin_views(C.byref(mb), raw_p, v0, v0, rows.ctypes.data_as(Fp))
    t["rebin_setup"] = time.perf_counter() - t0
    with cf.ThreadPoolExecutor(threads) as ex:
        t0 = time.perf_counter()
        list(ex.map(rebin_part, _ranges(part, threads)))
        t["rebin"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        list(ex.map(filter_part, _ranges(part * R, 4 * threads)))
        t["ramp_filter"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        list(ex.map(bp, _ranges(n_ang, threads)))
        t["backproject"] = time.perf_counter() - t0
    t["step"] = time.perf_counter() - t_step
    rebin_views = max(t["rebin"] - t["rebin_setup"], 0.0)
    t["block_s"] = (CPU_AF_PARTS * t["adaptive_filter"] + t["rebin_setup"] +
                    CPU_VIEW_PARTS * (rebin_views + t["ramp_filter"]) + CPU_ANGLE_PARTS * t["backproject"])
    return t


def cpu_sample_text(threads, mb, n_blocks):
    nht = n_views_of(mb) // (mb.cg.n_proj_turn // 2)
    return ("%d threads; a step: the adaptive filter of 1/%d of block 0's pull window (%d frames; one thread), "
            "the rebin and ramp filter of 1/%d of its %d views and the backprojection of 1/%d of its %d half-turn "
            "angles (%d x %d x %d voxels x %d half turns), the last two over all threads; scan time composed as "
            "%d x (%d t_af + t_rebin_setup + %d (t_rebin - t_rebin_setup + t_filter) + %d t_backproject), "
            "t_rebin_setup the rebin's per-call split of the window by focal spot, timed alone; finalize "
            "omitted (< 0.1%% of the CPU time)"
            % (threads, CPU_AF_PARTS, mb.ri.n_proj_pull, CPU_VIEW_PARTS, n_views_of(mb), CPU_ANGLE_PARTS,
               mb.cg.n_proj_turn // 2, mb.rp.nx, mb.rp.ny, mb.ri.n_slices_block, nht, n_blocks, CPU_AF_PARTS,
               CPU_VIEW_PARTS, CPU_ANGLE_PARTS))


def window_from_device(d_scan, ri, n_readings, frame):
    """A block's pull window from the resident scan (frames outside the scan are zeros)."""
    s = int(ri.idx_pull_start)
    s = s - 2 ** 64 if s >= 2 ** 63 else s
    P = int(ri.n_proj_pull)
    out = np.zeros(P * frame, np.float32)
    a, e = max(s, 0), min(s + P, n_readings)
    if e > a:
        out[(a - s) * frame:(e - s) * frame] = d_scan[a * frame:e * frame].cpu().numpy()
    return out


def cpu_baseline(mr, blocks, sizes, raw0, steps=1, threads=None):
    """The CPU sample (cpu_sample_step) on block 0's window raw0."""
    from oracle import oracle as O
    orc = O.oracle()
    T = threads or os.cpu_count() or 1
    mb = block_meta(mr, blocks[0])
    taps = oracle_taps(orc, mb)
    res = [cpu_sample_step(orc, mb, raw0, taps, T, k) for k in range(steps)]
    block_s = statistics.median(r["block_s"] for r in res)
    scan_s = len(blocks) * block_s
    return dict(value=sizes["vu_total"] / scan_s, unit="voxel-updates/s", cores=T, kind="port",
                sample=cpu_sample_text(T, mb, len(blocks)), scan_seconds=scan_s,
                step_seconds=statistics.median(r["step"] for r in res))


# --------------------------------------------------------------------------
# HU errors of the benched output on sampled patches
# --------------------------------------------------------------------------

def hu_reference(mr, blocks, d_scan, n_readings, threads=None):
    """The oracle's values at sampled patches of the middle block, for
    hu_compare: the oracle filters, rebins and ramp-filters that block's own
    pull window (float: the reference CPU path's arithmetic; double: the FP64
    oracle) and backprojects two 32 x 32 patches (image centre and
    off-centre); the final slices whose finalize weights all fall on that
    block are formed from them in double."""
    from oracle import oracle as O
    orc = O.oracle()
    T = threads or os.cpu_count() or 1
    b = len(blocks) // 2
    mb = block_meta(mr, blocks[b])
    frame = mr.cg.n_rows_raw * mr.cg.n_channels
    nx, ny, nb = mr.rp.nx, mr.rp.ny, mr.ri.n_slices_block
    raw = window_from_device(d_scan, blocks[b], n_readings, frame)
    taps = oracle_taps(orc, mb)
    t0 = time.perf_counter()
    rows32, _ = oracle_rows(orc, mb, raw, taps, T)
    rows64, _ = oracle_rows(orc, mb, raw, taps, T, double=True)
    h, w = 32, 32
    patches = [(nx // 2 - w // 2, nx // 2 + w // 2, ny // 2 - h // 2, ny // 2 + h // 2),
               (nx // 4 - w // 2, nx // 4 + w // 2, (5 * ny) // 8 - h // 2, (5 * ny) // 8 + h // 2)]
    jobs = [(p, dbl) for p in patches for dbl in (False, True)]
    with cf.ThreadPoolExecutor(len(jobs)) as ex:
        imgs = list(ex.map(lambda j: oracle_patch(orc, mb, rows64 if j[1] else rows32, j[0], j[1]), jobs))
    del rows32, rows64
    n_final = orc.oracle_n_slices_final(C.byref(mr))
    n_raw = nb * mr.ri.n_blocks
    wts = np.zeros(n_raw, np.float64)
    src = np.zeros(n_raw, np.int32)
    slices, e32, e64 = [], [], []
    for k in range(n_final):
        orc.oracle64_finalize_weights(C.byref(mr), k, wts.ctypes.data_as(C.POINTER(C.c_double)),
                                      src.ctypes.data_as(C.POINTER(C.c_int)))
        used = np.nonzero(wts)[0]
        if not len(used) or not all(b * nb <= src[s] < (b + 1) * nb for s in used):
            continue
        slices.append(k)
        for pi in range(len(patches)):
            e32.append(sum(wts[s] * imgs[2 * pi][src[s] - b * nb].astype(np.float64) for s in used))
            e64.append(sum(wts[s] * imgs[2 * pi + 1][src[s] - b * nb] for s in used))
    return {"block": b, "patches": patches, "slices": slices, "e32": e32, "e64": e64, "n_final": n_final,
            "shape": (ny, nx), "oracle_s": time.perf_counter() - t0}


def hu_compare(ref, d_final):
    """HU errors of a GPU final stack against hu_reference's values."""
    from ctbangbang_gb300 import scans
    ny, nx = ref["shape"]
    gpu = d_final.reshape(ref["n_final"], ny, nx)
    d64, d32, rr = [], [], []
    i = 0
    for k in ref["slices"]:
        for (x0, x1, y0, y1) in ref["patches"]:
            g = gpu[k, y0:y1, x0:x1].double().cpu().numpy()
            d64.append((g - ref["e64"][i]).ravel())
            d32.append((g - ref["e32"][i]).ravel())
            rr.append((ref["e32"][i] - ref["e64"][i]).ravel())
            i += 1
    hu = 1000.0 / scans.MU_WATER

    def stats(parts):
        v = np.concatenate(parts) * hu
        return {"max": float(np.abs(v).max()), "rms": float(np.sqrt(np.mean(v ** 2)))}

    return {"hu_vs_fp64": stats(d64), "hu_vs_reference": stats(d32), "reference_vs_fp64": stats(rr),
            "block": ref["block"], "final_slices": len(ref["slices"]), "patches": ref["patches"],
            "pixels": int(sum(x.size for x in d64)), "oracle_s": ref["oracle_s"],
            "how": "block %d's own pull window through the oracle (float: the reference CPU path's arithmetic; "
                   "double: FP64), two 32 x 32 patches backprojected, compared with the GPU stack at the %d final "
                   "slices whose finalize weights all fall on that block" % (ref["block"], len(ref["slices"]))}


# --------------------------------------------------------------------------
# reference arm
# --------------------------------------------------------------------------

def run_reference(args):
    """The reference CPU path (the oracle port: a bit-exact restatement of
    rebin_filter_cpu / backproject_cpu and of the adaptive filter's kernels)
    on the machine's host cores, on our arm's workload.  It plans with the
    oracle's restatement of the reference planner and projects its input with
    the test library's CPU projector: the reconstruction library is never
    loaded.  Each step is the bounded CPU sample of cpu_sample_step; the
    full-scan time is composed from the step's stage times."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from ctbangbang_gb300 import scans
    from oracle import oracle as O
    from oracle import plan as OP
    orc = O.oracle()
    spec = scans.CONFIGS[args.config]
    T = os.cpu_count() or 1
    t_wall = time.perf_counter()
    with tempfile.TemporaryDirectory(prefix="ctbb_bench_ref_") as d:
        mr = OP.plan_spec(spec, d)
        blocks = OP.block_plans(mr)
        sizes = workload_sizes(mr, blocks)
        n_final = orc.oracle_n_slices_final(C.byref(mr))
        mb = block_meta(mr, blocks[0])
        frame = mr.cg.n_rows_raw * mr.cg.n_channels
        s0, P = int(blocks[0].idx_pull_start), int(blocks[0].n_proj_pull)
        objs = ctbb_synth.phantom_objects(spec)
        raw = np.zeros((P, frame), np.float32)

        def gen(r):
            a, e = max(s0 + r[0], 0), min(s0 + r[1], spec.n_readings)
            if e > a:
                raw[a - s0:e - s0] = ctbb_synth.project_host(mr, objs, a, e - a, spec.i0, spec.seed).reshape(e - a, -1)

        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(T) as ex:
            list(ex.map(gen, _ranges(P, 8 * T)))
        gen_s = time.perf_counter() - t0
        raw = raw.reshape(-1)
        taps = oracle_taps(orc, mb)
        for k in range(args.warmup):
            cpu_sample_step(orc, mb, raw, taps, T, k)
        res = []
        t_timed = time.perf_counter()
        for k in range(args.steps):
            res.append(cpu_sample_step(orc, mb, raw, taps, T, args.warmup + k))
        timed_s = time.perf_counter() - t_timed
        workload = workload_text(args.config, spec, mr, len(blocks), n_final)
        OP.free_plan(mr)
    step_ms = timed_s * 1e3 / args.steps
    block_s = statistics.median(r["block_s"] for r in res)
    scan_s = len(blocks) * block_s
    v = sizes["vu_total"] / scan_s
    line = {
        "impl": "reference", "metric": "voxel-updates/s", "value": v, "unit": "voxel-updates/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic seeded helical phantom (water cylinder + ellipsoids, Poisson noise), projected on the CPU",
        "config": {"workload": workload, "voxel_updates_per_scan": sizes["vu_total"],
                   "composed_scan_seconds": scan_s, "scans_per_s": 1.0 / scan_s,
                   "step_stage_seconds": {k: statistics.median(r[k] for r in res)
                                          for k in ("adaptive_filter", "rebin_setup", "rebin", "ramp_filter",
                                                    "backproject")},
                   "input_generation_s": gen_s, "wall_s": time.perf_counter() - t_wall,
                   "note": "value = the scan's voxel updates over its composed CPU time; ms_per_step = the "
                           "measured time of one sample step (real work, not extrapolated)"},
        "cpu_baseline": {"value": v, "unit": "voxel-updates/s", "cores": T, "kind": "port",
                         "sample": cpu_sample_text(T, mb, len(blocks))},
        "e2e": {"value": v, "unit": "voxel-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# our arm
# --------------------------------------------------------------------------

def read_traffic():
    p = os.path.join(HERE, "profiles", "ncu_traffic.json")
    if os.path.exists(p):
        try:
            return json.load(open(p))
        except Exception:
            return {}
    return {}


def measured_peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            return json.load(open(p)), "measured"
        except Exception:
            pass
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def time_h2d_d2h(torch, h_scan, n_bytes_h2d, n_bytes_d2h, reps=3):
    """Pinned host->device and device->host copy times (ms) of the given
    sizes alone, on a stream of their own (the e2e breakdown)."""
    st = torch.cuda.Stream()
    dst = torch.empty(n_bytes_h2d // 4, dtype=torch.float32, device="cuda")
    back = torch.empty(max(n_bytes_d2h // 4, 1), dtype=torch.float32, pin_memory=True)
    src_d = torch.empty_like(back, device="cuda")
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    h2d, d2h = [], []
    with torch.cuda.stream(st):
        for _ in range(reps):
            e[0].record(st)
            dst.copy_(h_scan[:dst.numel()], non_blocking=True)
            e[1].record(st)
            back.copy_(src_d, non_blocking=True)
            e[2].record(st)
            st.synchronize()
            h2d.append(e[0].elapsed_time(e[1]))
            d2h.append(e[1].elapsed_time(e[2]))
    del dst, src_d, back
    return min(h2d), min(d2h)


def measure_config(args, torch, lib, config, rank, world, dist, headline):
    """One workload: the device-resident step (value), the host-buffer step
    (e2e) with its breakdown, and -- for the headline -- the other path, the
    per-stage profile, the clocks and the HU errors of the output."""
    from ctbangbang_gb300 import lib as L
    from ctbangbang_gb300 import scans
    local = int(os.environ.get("LOCAL_RANK", "0"))
    spec = scans.CONFIGS[config]
    tmp = tempfile.TemporaryDirectory(prefix="ctbb_bench_")
    mr = make_plan(spec, tmp.name)
    blocks = block_plans(mr)
    sizes = workload_sizes(mr, blocks)
    n = spec.n_readings
    frame = mr.cg.n_rows_raw * mr.cg.n_channels
    plane = mr.rp.nx * mr.rp.ny
    n_final = lib.ctbb_n_slices_final(C.byref(mr))
    out = {"workload": workload_text(config, spec, mr, len(blocks), n_final), "sizes": sizes, "spec": spec,
           "mr": mr, "blocks": blocks, "tmp": tmp, "n_final": n_final}

    # synthetic scan on the device (each replica its own seed)
    d_scan = ctbb_synth.project_scan_device(torch, mr, spec, seed=replica_seed(spec.seed, rank))
    d_final = torch.empty(n_final * plane, dtype=torch.float32, device="cuda")
    entry = {"scan": ("ctbb_reconstruct_scan_device", "ctbb_reconstruct_scan_host"),
             "blocks": ("ctbb_reconstruct_device", "ctbb_reconstruct_host")}
    other_path = "blocks" if args.path == "scan" else "scan"
    dev_entry, host_entry = entry[args.path]
    alt_dev, alt_host = entry[other_path]
    h2d_key = {"scan": "union_h2d_bytes", "blocks": "h2d_bytes"}
    out.update(dev_entry=dev_entry, host_entry=host_entry, h2d_bytes=sizes[h2d_key[args.path]])

    def step():
        L.call(dev_entry, C.byref(mr), C.c_void_p(d_scan.data_ptr()), C.c_void_p(d_final.data_ptr()),
               C.c_float(0.0))

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(local) if (rank == 0 and headline) else None
    lib.ctbb_profile_read(None, None, 0, 1)
    lib.ctbb_profile_enable(1 if headline else 0)
    launches0 = lib.ctbb_kernel_launch_count()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    ev[0].record()
    for k in range(args.steps):
        step()
        ev[k + 1].record()
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    out["launches"] = lib.ctbb_kernel_launch_count() - launches0
    lib.ctbb_profile_enable(0)
    stage_ms = (C.c_double * 5)()
    stage_n = (C.c_uint64 * 5)()
    lib.ctbb_profile_read(stage_ms, stage_n, 5, 1)
    out["stage_ms"], out["stage_n"] = list(stage_ms), list(stage_n)
    out["clocks"] = clocks.stop() if clocks else None
    per_step = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    ms = max_over_ranks(ev[0].elapsed_time(ev[-1]) / args.steps, dist)
    out.update(ms=ms, per_step=per_step, value=world * sizes["vu_total"] / (ms * 1e-3))

    # e2e through the host-buffer entry point (pinned host scan and stack)
    out["e2e"] = None
    ws_e2e = None
    if not args.no_e2e:
        h_scan = torch.empty(n * frame, dtype=torch.float32, pin_memory=True)
        h_scan.copy_(d_scan)
        h_final = torch.empty(n_final * plane, dtype=torch.float32, pin_memory=True)
        hp = h_scan.numpy().ctypes.data_as(C.POINTER(C.c_float))
        fp = h_final.numpy().ctypes.data_as(C.POINTER(C.c_float))

        def e2e_step():
            L.call(host_entry, C.byref(mr), hp, fp, C.c_float(0.0))

        for _ in range(2):
            e2e_step()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        lib.ctbb_profile_read(None, None, 0, 1)
        lib.ctbb_profile_enable(1)
        t0 = time.perf_counter()
        c0 = time.thread_time()
        e_marks = [t0]
        for _ in range(args.steps):
            e2e_step()  # returns with the stack in host memory
            e_marks.append(time.perf_counter())
        torch.cuda.synchronize()
        e_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / args.steps, dist)
        e_steps = sorted((e_marks[k + 1] - e_marks[k]) * 1e3 for k in range(args.steps))
        cpu_ms = (time.thread_time() - c0) * 1e3 / args.steps
        lib.ctbb_profile_enable(0)
        e_stage_ms = (C.c_double * 5)()
        lib.ctbb_profile_read(e_stage_ms, None, 5, 1)
        e_stages = {name: e_stage_ms[i] / args.steps for i, name in enumerate(STAGES)}
        same = bool(torch.equal(h_final.cuda(), d_final))
        h2d_ms, d2h_ms = time_h2d_d2h(torch, h_scan, out["h2d_bytes"], n_final * plane * 4)
        out["e2e"] = {
            "value": world * sizes["vu_total"] / (e_ms * 1e-3), "unit": "voxel-updates/s",
            "h2d_bytes_per_step": out["h2d_bytes"], "d2h_bytes_per_step": n_final * plane * 4,
            "ms_per_step": e_ms, "matches_device_path": same, "entry_point": host_entry,
            "breakdown_ms": {
                "device_step": ms, "e2e_minus_device": e_ms - ms,
                "h2d_copy_alone": h2d_ms, "d2h_copy_alone": d2h_ms,
                "h2d_gbs": out["h2d_bytes"] / (h2d_ms * 1e-3) / 1e9,
                "calling_thread_cpu": cpu_ms,
                "step_ms_min_median_max": [e_steps[0], e_steps[len(e_steps) // 2], e_steps[-1]],
                "stages_ms_per_step": e_stages,
                "backprojection_stream_idle": e_ms - e_stages.get("backproject", 0.0) - e_stages.get("finalize", 0.0),
                "note": "the host path streams the copy in chunks under the compute, and runs the preparation "
                        "(adaptive filter, rebin, ramp filter, edge patches) on a stream of its own beside the "
                        "backprojections: stages_ms_per_step are each stage's event times in the e2e steps "
                        "(the preparation's overlap the backprojections'), backprojection_stream_idle the part "
                        "of the step in which the backprojection stream had no work (waiting for the first "
                        "block's frames and rows, then any preparation not hidden); calling_thread_cpu includes "
                        "the wait for the stream (a spinning synchronise)"}}
        if headline and not args.no_whole_scan:
            def ws_host_step():
                L.call(alt_host, C.byref(mr), hp, fp, C.c_float(0.0))

            for _ in range(2):
                ws_host_step()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                ws_host_step()
            torch.cuda.synchronize()
            ws_e_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / args.steps, dist)
            ws_e2e = {"value": world * sizes["vu_total"] / (ws_e_ms * 1e-3), "unit": "voxel-updates/s",
                      "h2d_bytes_per_step": sizes[h2d_key[other_path]], "d2h_bytes_per_step": n_final * plane * 4,
                      "ms_per_step": ws_e_ms, "entry_point": alt_host}
        if headline and args.file:
            raw_path = os.path.join(mr.rp.raw_data_dir.decode(), mr.rp.raw_data_file.decode())
            h_scan.numpy().tofile(raw_path)

            def file_step():
                L.call("ctbb_reconstruct_scan_file", C.byref(mr), fp, C.c_float(0.0))

            for _ in range(2):
                file_step()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                file_step()
            torch.cuda.synchronize()
            f_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / args.steps, dist)
            out["e2e_file"] = {"value": world * sizes["vu_total"] / (f_ms * 1e-3), "unit": "voxel-updates/s",
                               "read_bytes_per_step": sizes["union_h2d_bytes"], "ms_per_step": f_ms,
                               "entry_point": "ctbb_reconstruct_scan_file"}
            os.remove(raw_path)
        del h_scan, h_final

    # the other path (block loop or whole scan) on the same resident scan
    out["other_path"] = None
    if headline and not args.no_whole_scan:
        d_final2 = torch.empty_like(d_final)

        def ws_step():
            L.call(alt_dev, C.byref(mr), C.c_void_p(d_scan.data_ptr()), C.c_void_p(d_final2.data_ptr()),
                   C.c_float(0.0))

        for _ in range(max(args.warmup, 3)):
            ws_step()
        torch.cuda.synchronize()
        w0 = torch.cuda.Event(enable_timing=True)
        w1 = torch.cuda.Event(enable_timing=True)
        w0.record()
        for _ in range(args.steps):
            ws_step()
        w1.record()
        torch.cuda.synchronize()
        ws_ms = w0.elapsed_time(w1) / args.steps
        diff = (d_final2 - d_final).double().abs()
        hu = 1000.0 / scans.MU_WATER
        out["other_path"] = {"path": other_path, "value": world * sizes["vu_total"] / (ws_ms * 1e-3),
                             "unit": "voxel-updates/s", "ms_per_step": ws_ms,
                             "max_hu_between_paths": float(diff.max()) * hu,
                             "rms_hu_between_paths": float(diff.pow(2).mean().sqrt()) * hu,
                             "entry_point": alt_dev, "e2e": ws_e2e}
        del d_final2
    out["d_scan"], out["d_final"] = d_scan, d_final
    return out


def measure_fp16(args, torch, lib, m, ref):
    """The reduced-storage mode on the headline scan: the ramp filter as the
    FP16 hi/lo Toeplitz contraction on the tensor cores writing FP16 footprint
    rows with per-view scales, the backprojector reading them (FP32
    accumulation).  Device-resident steps, stage profile, tensor-pipe
    throughput of the filter, HU errors of the output against the FP64 oracle
    and against the float32 path's output."""
    from ctbangbang_gb300 import lib as L
    from ctbangbang_gb300 import scans
    mr, sizes = m["mr"], m["sizes"]
    d_scan, d_ref = m["d_scan"], m["d_final"]
    d_out = torch.empty_like(d_ref)
    L.call("ctbb_set_storage", L.STORAGE_FP16)
    try:
        def step():
            L.call(m["dev_entry"], C.byref(mr), C.c_void_p(d_scan.data_ptr()), C.c_void_p(d_out.data_ptr()),
                   C.c_float(0.0))

        for _ in range(max(args.warmup, 3)):
            step()
        torch.cuda.synchronize()
        lib.ctbb_profile_read(None, None, 0, 1)
        lib.ctbb_profile_enable(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            step()
        e1.record()
        torch.cuda.synchronize()
        lib.ctbb_profile_enable(0)
        stage_ms = (C.c_double * 5)()
        stage_n = (C.c_uint64 * 5)()
        lib.ctbb_profile_read(stage_ms, stage_n, 5, 1)
    finally:
        L.call("ctbb_set_storage", L.STORAGE_FP32)
    ms = e0.elapsed_time(e1) / args.steps
    diff = (d_out - d_ref).double().abs()
    hu = 1000.0 / scans.MU_WATER
    # the filter's tensor work: 3 FP16 products of 2 n^2 FLOP per row over the
    # union's rows and the edge views' rows
    n = mr.cg.n_channels_oversampled
    filter_rows = (sizes["union_rebin_samples"] // n)
    flop = 3 * 2.0 * n * n * filter_rows
    ramp_ms = stage_ms[2] / args.steps
    peaks, peak_kind = measured_peaks()
    peak_tc = peaks.get("bf16_tflops", 1900.0)
    achieved_tc = flop / (ramp_ms * 1e-3) / 1e12
    out = {"value": sizes["vu_total"] / (ms * 1e-3), "unit": "voxel-updates/s", "ms_per_step": ms,
           "scans_per_s": 1e3 / ms,
           "stages_ms_per_step": {name: stage_ms[i] / args.steps for i, name in enumerate(STAGES)},
           "roofline": {"kernel": "ramp_tc_gemm_kernel (with its row-split pass)", "bound": "tensor",
                        "achieved": achieved_tc, "peak": peak_tc, "unit": "TFLOP/s", "frac": achieved_tc / peak_tc,
                        "peak_source": "BF16 dense burst, MEASURED_PEAKS.json (%s); FP16 runs at the same "
                                       "tensor rate" % peak_kind,
                        "flop_per_row": 3 * 2.0 * n * n, "rows_per_step": filter_rows,
                        "algorithmic_tflops": flop / 3 / (ramp_ms * 1e-3) / 1e12,
                        "tensor_pipe_active_ncu": read_traffic().get("ramp_tc_tensor_pipe_active"),
                        "note": "3 FP16 products (hi.hi, hi.lo, lo.hi) of 2 N_os^2 FLOP per row over the union's "
                                "rows (algorithmic_tflops counts one); the stage time also covers the re-made "
                                "edge views' rows and the row split, so achieved is a lower bound"},
           "max_hu_vs_fp32_path": float(diff.max()) * hu,
           "rms_hu_vs_fp32_path": float(diff.pow(2).mean().sqrt()) * hu,
           "entry_point": m["dev_entry"] + " after ctbb_set_storage(CTBB_STORAGE_FP16)"}
    if ref is not None:
        out["hu"] = hu_compare(ref, d_out)
    del d_out
    return out


def run_ours(args):
    import torch

    from ctbangbang_gb300 import lib as L
    from ctbangbang_gb300 import scans

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lib = L.load()
    lib.ctbb_set_stream(C.c_void_p(torch.cuda.current_stream().cuda_stream))
    m = measure_config(args, torch, lib, args.config, rank, world, dist, headline=True)
    mr, blocks, sizes = m["mr"], m["blocks"], m["sizes"]
    plane = mr.rp.nx * mr.rp.ny
    spec = m["spec"]

    if rank != 0:
        del m
        if dist is not None:
            dist.destroy_process_group()
        return

    # HU errors of the benched output (sampled patches of the middle block)
    hu, ref = None, None
    if not args.no_hu:
        try:
            ref = hu_reference(mr, blocks, m["d_scan"], spec.n_readings)
            hu = hu_compare(ref, m["d_final"])
        except Exception as e:  # reported in the line, the rest of the run stands
            hu = {"error": "%s: %s" % (type(e).__name__, e)}
    fp16 = None
    if not args.no_fp16:
        try:
            fp16 = measure_fp16(args, torch, lib, m, ref)
        except Exception as e:
            fp16 = {"error": "%s: %s" % (type(e).__name__, e)}
    raw0 = None
    if world == 1 and not args.no_cpu_baseline:
        raw0 = window_from_device(m["d_scan"], blocks[0], spec.n_readings, mr.cg.n_rows_raw * mr.cg.n_channels)
    del m["d_scan"], m["d_final"]
    torch.cuda.empty_cache()

    # roofline of the dominant kernel (backprojection, FP32-pipe bound)
    stage_ms, stage_n = m["stage_ms"], m["stage_n"]
    peak_fp32 = ctbb_synth.fp32_peak_tflops(5, torch.cuda.current_stream().cuda_stream)
    bp_ms, bp_n = stage_ms[3], max(stage_n[3], 1)
    vu_per_launch = sizes["vu_total"] / len(blocks)
    bp_launch_ms = bp_ms / bp_n
    achieved = FLOP_PER_VU * vu_per_launch / (bp_launch_ms * 1e-3) / 1e12
    traffic = read_traffic().get("backproject")
    peaks, peak_kind = measured_peaks()
    hbm = peaks.get("hbm_gbs", 6800.0)
    if args.path == "scan":
        raw_b, rb_b = sizes["union_raw_samples"], sizes["union_rebin_samples"]
    else:
        nblk = len(blocks)
        raw_b = sum(sizes["raw_samples"]) / nblk
        rb_b = sum(sizes["rebin_samples"]) / nblk
    n_final = m["n_final"]
    stage_bytes = {"adaptive_filter": 8 * raw_b, "rebin": 4 * raw_b + 4 * rb_b, "ramp_filter": 8 * rb_b,
                   "finalize": 4 * plane * (mr.ri.n_slices_recon + n_final)}
    stages = {}
    for i, name in enumerate(STAGES):
        if stage_n[i] == 0:
            continue
        entry = {"ms_per_step": stage_ms[i] / args.steps, "launches_per_step": stage_n[i] / args.steps,
                 "share": stage_ms[i] / max(sum(stage_ms), 1e-9)}
        if name in stage_bytes:
            # algorithmic bytes of one pass over the union (or one block window)
            passes = 1 if args.path == "scan" else len(blocks)
            gbs = stage_bytes[name] * passes / (stage_ms[i] / args.steps * 1e-3) / 1e9
            entry.update({"achieved_gbs_per_pass": gbs, "frac_of_hbm": gbs / hbm})
        stages[name] = entry

    # the other configuration, reported beside the headline
    beside = None
    if world == 1 and args.beside and args.beside != args.config:
        try:
            mb = measure_config(args, torch, lib, args.beside, rank, world, dist, headline=False)
            beside = {"workload": mb["workload"], "value": mb["value"], "unit": "voxel-updates/s",
                      "ms_per_step": mb["ms"], "scans_per_s": 1e3 / mb["ms"],
                      "voxel_updates_per_scan": mb["sizes"]["vu_total"], "e2e": mb["e2e"],
                      "entry_point": mb["dev_entry"]}
            del mb["d_scan"], mb["d_final"]
            scans.free_plan(mb["mr"])
        except Exception as e:
            beside = {"error": "%s: %s" % (type(e).__name__, e)}
        torch.cuda.empty_cache()

    batch = None
    if world == 1 and not args.no_batch:
        try:
            batch = batch_measure(args, torch)
        except Exception as e:
            batch = {"error": "%s: %s" % (type(e).__name__, e)}
        torch.cuda.empty_cache()
    serve = None
    if world == 1 and not args.no_serve:
        try:
            serve = serve_measure(args, torch)
        except Exception as e:  # reported in the line, the rest of the run stands
            serve = {"error": "%s: %s" % (type(e).__name__, e)}
    cpu = None
    if raw0 is not None:
        cpu = cpu_baseline(mr, blocks, sizes, raw0, steps=1)
    per_step_sorted = sorted(m["per_step"])
    ms = m["ms"]
    line = {
        "metric": "voxel-updates/s", "value": m["value"], "unit": "voxel-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic seeded helical phantom (water cylinder + ellipsoids, Poisson noise), generated on the device",
        "config": {
            "workload": m["workload"],
            "path": ("whole scan: the union of the blocks' pull windows (%d frames) adaptive-filtered, rebinned "
                     "and ramp-filtered once, each block's edge views re-made from its own window, each block "
                     "backprojected (%s / %s)" % (sizes["union_h2d_bytes"] // (4 * mr.cg.n_rows_raw *
                                                                                  mr.cg.n_channels),
                                                  m["dev_entry"], m["host_entry"]))
                    if args.path == "scan" else
                    ("block loop as the reference: each block's pull window filtered, rebinned and backprojected "
                     "(%s / %s)" % (m["dev_entry"], m["host_entry"])),
            "scans_per_s": world / (ms * 1e-3),
            "voxel_updates_per_scan": sizes["vu_total"],
            "latency_ms": {"p50": per_step_sorted[len(per_step_sorted) // 2],
                           "p99": per_step_sorted[min(len(per_step_sorted) - 1,
                                                      int(math.ceil(0.99 * len(per_step_sorted))) - 1)]},
            "l2": "no flush: each step reads %.1f GB of raw frames (> 129 MB L2)" % (m["h2d_bytes"] / 1e9),
            "parallelism": "replicas" if world > 1 else "single GPU",
        },
        "hu": hu,
        "fp16_storage": fp16,
        "roofline": {"kernel": "backproject_column_kernel (with its angle-chunk combine)", "bound": "fp32",
                     "achieved": achieved, "peak": peak_fp32,
                     "unit": "TFLOP/s", "frac": achieved / peak_fp32 if peak_fp32 > 0 else None,
                     "traffic": traffic, "flop_per_vu": FLOP_PER_VU, "vu_per_launch": vu_per_launch,
                     "launch_ms": bp_launch_ms,
                     "launch_ms_note": "CUDA events around each block's backprojection: the column kernel and "
                                       "the combine of its 16 angle chunks",
                     "peak_source": "measured FFMA-loop throughput of this GPU in this run "
                                    "(MEASURED_PEAKS.json has no FP32 figure)"},
        "stages": stages,
        "hbm_peak_gbs": hbm, "hbm_peak_kind": peak_kind,
        "cpu_baseline": cpu,
        "e2e": m["e2e"],
        "other_path": m["other_path"],
        "e2e_file": m.get("e2e_file"),
        "beside": beside,
        "batch": batch,
        "serve": serve,
        "gpu_launches": m["launches"] / args.steps,
        "clocks": m["clocks"],
    }
    print(json.dumps(line), flush=True)
    scans.free_plan(mr)
    if dist is not None:
        dist.destroy_process_group()


SERVE_CONFIG = 4  # the served stream: scan i is seeded 1000 * 4 + i


def serve_spec(rng, i, full):
    """One scan of the batched / served size distribution: FFS none / phi /
    z / both, 16 / 32 / 64 rows (after z-FFS), pitch 0.6-1.5, rotations 2-30,
    field 250-500 mm, 256^2 or 512^2, 20-300 slices of 1 mm, I0 2e4-2e5.
    Without `full`, rotations are capped at 8 and slices at 120 (the default
    bench run stays within minutes).  The slice count shrinks until the
    rotations cover every block's pull window."""
    from ctbangbang_gb300 import scans
    z_ffs, phi_ffs = [(0, 0), (0, 1), (1, 0), (1, 1)][int(rng.integers(4))]
    rows = int(rng.choice([16, 32, 64]))
    pitch = float(rng.uniform(0.6, 1.5))
    turns = int(rng.integers(2, 31 if full else 9))
    fov = float(rng.uniform(250.0, 500.0))
    nx = int(rng.choice([256, 512]))
    n_slices = int(rng.integers(20, 301 if full else 121))
    i0 = float(10.0 ** rng.uniform(math.log10(2e4), math.log10(2e5)))
    spec = scans.ScanSpec(name="serve%d" % i, **scans._definition_as(), n_rows=rows, coll=0.6, pitch=pitch,
                          turns=turns, slice_thickness=1.0, recon_fov=fov, nx=nx, ny=nx, start_pos=0.0,
                          n_slices=n_slices, z_ffs=z_ffs, phi_ffs=phi_ffs, adaptive_filtration=1.0,
                          seed=1000 * SERVE_CONFIG + i, n_ellipsoids=30, i0=i0)
    spec.start_pos = scans.allowed_margin(spec) + 1.0
    while spec.n_slices > 4 and scans.needed_turns(spec) > turns:
        spec.n_slices = int(spec.n_slices * 0.85)
    spec.turns = max(float(turns), scans.needed_turns(spec))
    return spec


BATCH_CONFIG = 4  # the batched workload: scan i is seeded 1000 * 4 + i


def batch_measure(args, torch):
    """Batched uneven scans: `batch_scans` seeded scans of the full batched
    distribution (serve_spec with full ranges: rotations 2-30, pitch 0.6-1.5,
    FFS none/phi/z/both, 16/32/64 rows, field 250-500 mm, 256^2 or 512^2,
    20-300 slices, I0 2e4-2e5).  Plain: each scan alone through
    ctbb_reconstruct_scan_device (float32 rows, default launch shape), one
    after another.  Batched: ctbb_batch_begin / _add_device / _run with the
    autotuner's launch shapes, in float32 and in FP16 storage; scans are added
    until their rows would pass the batch memory budget, then the batch runs.
    Times are CUDA events around the library calls (the synthetic scans are
    projected outside them); every batched stack is compared with its scan
    alone."""
    from ctbangbang_gb300 import lib as L
    from ctbangbang_gb300 import scans
    lib = L.load()
    rng = np.random.default_rng(1000 * BATCH_CONFIG)
    tmp = tempfile.TemporaryDirectory(prefix="ctbb_batch_")
    specs, mrs, finals, vus = [], [], [], []
    for i in range(args.batch_scans):
        spec = serve_spec(rng, i, True)
        spec.seed = 1000 * BATCH_CONFIG + i
        mr = scans.plan_spec(spec, os.path.join(tmp.name, str(i)))
        specs.append(spec)
        mrs.append(mr)
        finals.append(lib.ctbb_n_slices_final(C.byref(mr)) * mr.rp.nx * mr.rp.ny)
        vus.append(workload_sizes(mr, block_plans(mr))["vu_total"])
    ev = lambda: torch.cuda.Event(enable_timing=True)

    def timed(fn):
        a, b = ev(), ev()
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b)

    # plain: each scan alone (one warm-up call for the first, whose buffers
    # then cover the sizes that follow only as they grow)
    alone, t_plain = [], []
    for k in range(len(specs)):
        d = ctbb_synth.project_scan_device(torch, mrs[k], specs[k])
        out = torch.empty(finals[k], dtype=torch.float32, device="cuda")
        call = lambda: L.call("ctbb_reconstruct_scan_device", C.byref(mrs[k]), C.c_void_p(d.data_ptr()),
                              C.c_void_p(out.data_ptr()), C.c_float(0.0))
        call()
        t_plain.append(timed(call))
        alone.append(out.cpu())
        del d, out
    lib.ctbb_release_workspace()
    torch.cuda.empty_cache()
    plain_ms = sum(t_plain)
    hu = 1000.0 / scans.MU_WATER
    results = {}
    for storage, mode in (("fp32", L.STORAGE_FP32), ("fp16", L.STORAGE_FP16)):
        L.call("ctbb_set_storage", mode)
        budget = args.batch_budget_gb * (1 << 30)
        row_bytes = 4 if mode == L.STORAGE_FP32 else 12  # float32 rows, or float32 rows + FP16 quads
        outs = [torch.empty(finals[k], dtype=torch.float32, device="cuda") for k in range(len(specs))]
        total_ms, runs, held = 0.0, 0, 0
        try:
            for rep in range(2):  # the first pass tunes and sizes the slots; the second is timed
                total_ms, runs, held = 0.0, 0, 0
                L.call("ctbb_batch_begin")
                for k in range(len(specs)):
                    need = lib.ctbb_scan_workspace_bytes(C.byref(mrs[k]))
                    if held and held + need * row_bytes // 8 > budget:
                        total_ms += timed(lambda: L.call("ctbb_batch_run"))
                        runs += 1
                        held = 0
                        L.call("ctbb_batch_begin")
                    d = ctbb_synth.project_scan_device(torch, mrs[k], specs[k])
                    total_ms += timed(lambda: L.call("ctbb_batch_add_device", C.byref(mrs[k]),
                                                     C.c_void_p(d.data_ptr()), C.c_void_p(outs[k].data_ptr()),
                                                     C.c_float(0.0)))
                    held += need * row_bytes // 8
                    del d
                total_ms += timed(lambda: L.call("ctbb_batch_run"))
                runs += 1
        finally:
            L.call("ctbb_set_storage", L.STORAGE_FP32)
        diffs = [((outs[k].cpu().double() - alone[k].double()).abs()) for k in range(len(specs))]
        results[storage] = {
            "scans_per_s": len(specs) / (total_ms * 1e-3), "ms_total": total_ms, "batch_runs": runs,
            "vs_plain": plain_ms / total_ms,
            "max_hu_vs_alone_fp32": max(float(d.max()) for d in diffs) * hu,
            "rms_hu_vs_alone_fp32": float(np.sqrt(np.mean([float(d.pow(2).mean()) for d in diffs]))) * hu}
        del outs
        lib.ctbb_release_workspace()
        torch.cuda.empty_cache()
    buf = C.create_string_buffer(1 << 16)
    lib.ctbb_autotune_report(buf, len(buf))
    for mr in mrs:
        scans.free_plan(mr)
    desc = ["%s rows %d, %.1f rot, pitch %.2f, %d^2, %d slices, fov %.0f" % (
        {(0, 0): "no FFS", (0, 1): "phi FFS", (1, 0): "z FFS", (1, 1): "phi+z FFS"}[(s.z_ffs, s.phi_ffs)],
        s.n_rows, s.turns, s.pitch, s.nx, s.n_slices, s.recon_fov) for s in specs]
    return {
        "workload": "%d seeded scans of the batched distribution (rotations 2-30, pitch 0.6-1.5, FFS "
                    "none/phi/z/both, 16/32/64 rows, 250-500 mm, 256^2 or 512^2, 20-300 slices)" % len(specs),
        "scans": desc, "voxel_updates": sum(vus),
        "plain_scans_per_s": len(specs) / (plain_ms * 1e-3), "plain_ms_total": plain_ms,
        "batched": results,
        "autotune": buf.value.decode(errors="replace").splitlines(),
        "entry_points": "ctbb_batch_begin / _add_device / _run (autotuned shapes) vs ctbb_reconstruct_scan_device",
        "memory_budget_gb": args.batch_budget_gb,
    }


def percentile(v, q):
    v = sorted(v)
    return v[min(len(v) - 1, max(0, int(math.ceil(q * len(v))) - 1))]


def serve_measure(args, torch):
    """The served reconstruction stream: `serve_requests` requests (600 by
    default), each one of `serve_scans` distinct seeded scans of the batched
    size distribution (serve_spec, full ranges) or, with probability 5 %, a
    large 40-turn 512^2 x 400-slice scan (the precision workload's geometry).
    A request server (ctbb_server_*, `serve_workers` workers, each request
    through ctbb_context_reconstruct_scan_host from pinned host buffers) with a
    150 GB device budget and out-of-order admission (a request that does not
    fit lets the ones behind it that do pass, for at most 2 s).
    Plain: every request alone through ctbb_reconstruct_scan_host, one after
    another (its per-scan times measured once per distinct scan).
    Served, saturated: requests submitted as fast as results come back, with at
    most `serve_window` in flight (throughput).  Served, Poisson: arrivals at a
    rate between 2 and 20 requests/s (80 % of the saturated throughput,
    clipped to that range) for latency, against the plain path's first come
    first served queue under the same arrivals.  Every served stack is checked
    against its scan's stack alone (the same kernels on the same data: equal
    bit for bit)."""
    from ctbangbang_gb300 import lib as L
    from ctbangbang_gb300 import scans
    from ctbangbang_gb300.serving import Server
    lib = L.load()
    rng = np.random.default_rng(1000 * SERVE_CONFIG + 5)
    tmp = tempfile.TemporaryDirectory(prefix="ctbb_serve_")
    pool = [serve_spec(rng, i, True) for i in range(args.serve_scans)]
    for i, sp in enumerate(pool):
        sp.seed = 1000 * 5 + i
    large = dataclasses.replace(scans.CONFIGS["config3"], name="serve_large", seed=1000 * 5 + 99)
    pool.append(large)
    prms, host, finals, vus = [], [], [], []
    for i, spec in enumerate(pool):
        wd = os.path.join(tmp.name, str(i))
        os.makedirs(wd)
        prm, inst = scans.prepare(spec, wd)
        mr = scans.plan(prm, inst)
        n, frame = spec.n_readings, mr.cg.n_rows_raw * mr.cg.n_channels
        d = ctbb_synth.project_scan_device(torch, mr, spec)
        h = torch.empty(n * frame, dtype=torch.float32, pin_memory=True)
        h.copy_(d)
        del d
        prms.append((prm, inst))
        host.append(h)
        finals.append(lib.ctbb_n_slices_final(C.byref(mr)) * mr.rp.nx * mr.rp.ny)
        vus.append(workload_sizes(mr, block_plans(mr))["vu_total"])
        scans.free_plan(mr)
    torch.cuda.empty_cache()
    fptr = lambda t: t.numpy().ctypes.data_as(C.POINTER(C.c_float))
    # plain: each distinct scan alone (one warm-up, one timed run); its stack is the reference
    alone, t_alone = [], []
    for k in range(len(pool)):
        mr = scans.plan(*prms[k])
        out = torch.empty(finals[k], dtype=torch.float32, pin_memory=True)
        L.call("ctbb_reconstruct_scan_host", C.byref(mr), fptr(host[k]), fptr(out), C.c_float(0.0))
        t0 = time.perf_counter()
        L.call("ctbb_reconstruct_scan_host", C.byref(mr), fptr(host[k]), fptr(out), C.c_float(0.0))
        t_alone.append((time.perf_counter() - t0) * 1e3)
        alone.append(out)
        scans.free_plan(mr)
    lib.ctbb_release_workspace()
    torch.cuda.empty_cache()
    n_req = args.serve_requests
    pick = [len(pool) - 1 if rng.uniform() < 0.05 else int(rng.integers(args.serve_scans)) for _ in range(n_req)]
    plain_ms = sum(t_alone[k] for k in pick)
    free, total = torch.cuda.mem_get_info()
    budget = int(min(150 << 30, 0.85 * free))
    n_buf = max(args.serve_window, args.serve_workers + 2)
    bufs = [torch.empty(max(finals), dtype=torch.float32, pin_memory=True) for _ in range(n_buf)]

    def run_stream(srv, arrivals):
        """Submits the requests (at the arrival times, or as buffers free up),
        waits for each, checks it against its scan alone."""
        import collections
        mrs = {}
        inflight = collections.deque()  # (request, ticket, buffer index)
        free_bufs = list(range(n_buf))
        res = [None] * n_req
        same = True
        t0 = time.perf_counter()

        def collect_one():
            nonlocal same
            r, t, bi = inflight.popleft()
            res[r] = srv.wait(t)
            k = pick[r]
            same = same and bool(torch.equal(bufs[bi][:finals[k]], alone[k]))
            scans.free_plan(mrs.pop(r))
            free_bufs.append(bi)

        for r, k in enumerate(pick):
            if arrivals is not None:
                delay = arrivals[r] - (time.perf_counter() - t0)
                while delay > 0 and inflight and len(free_bufs) < n_buf:
                    # keep collecting finished requests while waiting for the next arrival
                    collect_one()
                    delay = arrivals[r] - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
            while not free_bufs:
                collect_one()
            bi = free_bufs.pop()
            mrs[r] = scans.plan(*prms[k])
            inflight.append((r, srv.submit(mrs[r], fptr(host[k]), fptr(bufs[bi])), bi))
        while inflight:
            collect_one()
        wall = (time.perf_counter() - t0) * 1e3
        return res, wall, same

    with Server(args.serve_workers, budget) as srv:
        L.call("ctbb_server_configure", srv._h, L.STORAGE_FP32, C.c_double(2000.0))
        # warm-up: every distinct scan once per worker (the workers size their buffers)
        saved, n_saved = pick, n_req
        pick = [k for k in range(len(pool)) for _ in range(args.serve_workers)]
        n_req = len(pick)
        run_stream(srv, None)
        pick, n_req = saved, n_saved
        res_sat, wall_sat, same_sat = run_stream(srv, None)
        served_rate = n_req / (wall_sat * 1e-3)
        rate = min(20.0, max(2.0, 0.8 * served_rate))
        gaps = rng.exponential(1.0 / rate, size=n_req)
        arrivals = np.cumsum(gaps) - gaps[0]
        res_poi, wall_poi, same_poi = run_stream(srv, arrivals)
        passed = lib.ctbb_server_passed_count(srv._h)
    lat = [r.latency_ms for r in res_poi]
    done, plain_lat = 0.0, []
    for r, k in enumerate(pick):
        start = max(arrivals[r] * 1e3, done)
        done = start + t_alone[k]
        plain_lat.append(done - arrivals[r] * 1e3)
    vu = sum(vus[k] for k in pick)
    desc = ["%s rows %d, %.1f rot, pitch %.2f, %d^2, %d slices, fov %.0f" % (
        {(0, 0): "no FFS", (0, 1): "phi FFS", (1, 0): "z FFS", (1, 1): "phi+z FFS"}[(sp.z_ffs, sp.phi_ffs)],
        sp.n_rows, sp.turns, sp.pitch, sp.nx, sp.n_slices, sp.recon_fov) for sp in pool]
    return {
        "workload": "%d requests, each one of %d seeded scans of the batched distribution or (5 %%, %d requests) "
                    "a 40-turn 512^2 x 400-slice scan" % (n_req, args.serve_scans, pick.count(len(pool) - 1)),
        "scans": desc, "per_scan_alone_ms": t_alone,
        "workers": args.serve_workers, "budget_gb": budget / 2**30, "age_bound_ms": 2000.0,
        "plain_scans_per_s": n_req / (plain_ms * 1e-3),
        "served_scans_per_s": served_rate,
        "served_vs_plain": served_rate / (n_req / (plain_ms * 1e-3)),
        "served_voxel_updates_per_s": vu / (wall_sat * 1e-3),
        "poisson_rate_per_s": rate,
        "latency_ms": {"p50": percentile(lat, 0.5), "p99": percentile(lat, 0.99)},
        "plain_latency_ms_same_arrivals": {"p50": percentile(plain_lat, 0.5), "p99": percentile(plain_lat, 0.99)},
        "requests_started_ahead_of_older": int(passed),
        "matches_alone": bool(same_sat and same_poi),
        "entry_points": "ctbb_server_create / _configure / _submit / _wait (server) vs ctbb_reconstruct_scan_host "
                        "(plain)",
    }


def run_profile_case(args):
    """Block 0 of the configuration: its pull window generated on the device,
    then adaptive filter, rebin, ramp filter (FP32 FFT) and backprojection
    once each, then the reduced-storage stages on the same rebinned rows: the
    tensor-core ramp filter into FP16 footprint words and the backprojection
    from them.  A few GB on the device; every input is larger than L2."""
    import torch

    from ctbangbang_gb300 import lib as L
    from ctbangbang_gb300 import structs
    lib = L.load()
    from ctbangbang_gb300 import scans
    spec = scans.CONFIGS[args.config]
    tmp = tempfile.TemporaryDirectory(prefix="ctbb_prof_")
    mr = make_plan(spec, tmp.name)
    b0 = block_plans(mr)[0]
    m = structs.ReconMetadata()
    C.memmove(C.byref(m), C.byref(mr), C.sizeof(m))
    m.ri = b0
    n = spec.n_readings
    frame = m.cg.n_rows_raw * m.cg.n_channels
    P = b0.n_proj_pull
    nv = P // b0.n_ffs - 2 * m.cg.add_projections
    nos, R = m.cg.n_channels_oversampled, m.cg.n_rows
    ta = torch.from_numpy(np.ctypeslib.as_array(mr.tube_angles, (n,)).copy()).cuda()
    tp = torch.from_numpy(np.ctypeslib.as_array(mr.table_positions, (n,)).copy()).cuda()
    d_raw = torch.empty(P * frame, dtype=torch.float32, device="cuda")
    ctbb_synth.project_device(m, ctbb_synth.phantom_objects(spec), ta.data_ptr(), tp.data_ptr(), int(b0.idx_pull_start),
                              P, spec.i0, spec.seed, d_raw.data_ptr(), torch.cuda.current_stream().cuda_stream)
    d_filt = torch.empty_like(d_raw)
    d_rb = torch.empty(nv * R * nos, dtype=torch.float32, device="cuda")
    d_blk = torch.empty(m.rp.nx * m.rp.ny * m.ri.n_slices_block, dtype=torch.float32, device="cuda")
    taps = (C.c_float * (2 * nos))()
    L.call("ctbb_load_filter", C.byref(m), taps)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(12)]
    ev[0].record()
    L.call("ctbb_adaptive_filter_device", C.byref(m), C.c_void_p(d_raw.data_ptr()), C.c_void_p(d_filt.data_ptr()))
    ev[1].record()
    ev[2].record()
    L.call("ctbb_rebin_device", C.byref(m), C.c_void_p(d_filt.data_ptr()), C.c_void_p(d_rb.data_ptr()))
    ev[3].record()
    del d_raw, d_filt
    d_unfilt = d_rb.clone()
    ev[4].record()
    L.call("ctbb_ramp_filter_device", C.c_void_p(d_rb.data_ptr()), nv * R, nos, taps)
    ev[5].record()
    ev[6].record()
    L.call("ctbb_backproject_device", C.byref(m), C.c_void_p(d_rb.data_ptr()), C.c_void_p(d_blk.data_ptr()))
    ev[7].record()
    del d_rb
    quads = torch.empty(nv * R * nos * 4, dtype=torch.float16, device="cuda")
    qscale = torch.empty(nv * R, dtype=torch.float32, device="cuda")
    ev[8].record()
    L.call("ctbb_ramp_filter_fp16_device", C.c_void_p(d_unfilt.data_ptr()), nv * R, nos, taps, R,
           C.c_void_p(quads.data_ptr()), C.c_void_p(qscale.data_ptr()))
    ev[9].record()
    d_blk16 = torch.empty_like(d_blk)
    ev[10].record()
    L.call("ctbb_backproject_fp16_device", C.byref(m), C.c_void_p(quads.data_ptr()), C.c_void_p(qscale.data_ptr()),
           C.c_void_p(d_blk16.data_ptr()))
    ev[11].record()
    torch.cuda.synchronize()
    ms = [ev[2 * i].elapsed_time(ev[2 * i + 1]) for i in range(6)]
    from ctbangbang_gb300.scans import MU_WATER
    diff = (d_blk16 - d_blk).double().abs() * (1000.0 / MU_WATER)
    print(json.dumps({"profile_case": args.config, "block": 0, "n_proj_pull": P, "n_views": nv,
                      "stage_ms": dict(zip(STAGES[:4] + ["ramp_filter_fp16_tensor", "backproject_fp16"], ms)),
                      "fp16_vs_fp32_block_hu": {"max": float(diff.max()), "rms": float(diff.pow(2).mean().sqrt())},
                      "finite": bool(torch.isfinite(d_blk).all().item() and torch.isfinite(d_blk16).all().item())}),
          flush=True)
    scans.free_plan(mr)


def main():
    args = parse_args()
    if args.profile_case:
        run_profile_case(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
