"""Generates the golden fixtures of tests/golden/ from the reference's own CPU
code (oracle/_ref, compiled from the reference sources by oracle/ref/Makefile).

Run in the container that has the reference tree:
    python tests/golden/make_golden.py

Fixtures:
  plan_<config>.json   the reference planner's outputs (setup.cu): ct_geom,
                       recon_info of every block, sha256 of the per-frame
                       tube-angle and table-position tables.
  block_<case>.npz     the reference's outputs on a synthetic scan whose frames
                       tests/golden/synth.py regenerates bit for bit (sha256
                       stored): per block the samples the adaptive filter
                       changed (index, value), every VIEW_STEP-th view of the
                       rebinned rows without filter (via a unit-impulse
                       kernel: exact, except that samples which are exactly 0
                       come out as ~1e-16 FFT roundoff) and with the ramp
                       filter, then the image stack and the final stack.
  ramp_kat.json        taps of the reference's f_736_sharp / f_672_sharp
                       kernel files around the centre (known answers of the
                       ramp formula in resources/ramp.m).
"""
import ctypes as C
import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from ctbangbang_gb300 import scans, structs  # noqa: E402
from oracle import oracle as O  # noqa: E402

sys.path.insert(0, HERE)
import synth  # noqa: E402

REF_TREE = O.REFERENCE_TREE
VIEW_STEP = 8


def golden_cases():
    """name -> ScanSpec of the block fixtures."""
    kw = dict(n_channels=32, n_rows_raw=4, nx=16, ny=16, n_proj_turn=48)
    cases = {
        "nffs_af0": scans.tiny(0, 0, adaptive_filtration=0.0, seed=11, **kw),
        "pffs_af1": scans.tiny(0, 1, adaptive_filtration=1.0, seed=12, **kw),
        "zffs_af1_rev": scans.tiny(1, 0, adaptive_filtration=1.0, seed=13, reverse_row_interleave=1, **kw),
        "affs_af1": scans.tiny(1, 1, adaptive_filtration=1.0, seed=14, **kw),
        "nffs_2blocks_in": scans.tiny(0, 0, adaptive_filtration=0.5, seed=15, n_slices=12,
                                      slice_thickness=2.5, table_dir="in", **kw),
    }
    for name, spec in cases.items():
        spec.name = name
        spec.i0 = 2e4
    return cases


def synth_frames(spec):
    """The golden input of a case (regenerated bit for bit by the tests)."""
    cc = spec.central_channel
    if spec.phi_ffs:
        cc = np.floor(np.float32(cc)) + np.float32(0.375)
    return synth.frames(spec.n_readings, spec.n_rows_raw, spec.n_channels, spec.n_proj_turn * spec.n_ffs,
                        cc, spec.r_f * spec.fan_angle_increment, spec.seed)


def planner_cases():
    c = dict(scans.CONFIGS)
    c1in = scans.ScanSpec(**{**scans.CONFIGS["config1"].__dict__})
    c1in.name, c1in.table_dir = "config1_in", "in"
    c["config1_in"] = c1in
    c2n = scans.ScanSpec(**{**scans.CONFIGS["config2"].__dict__})
    c2n.name, c2n.start_pos, c2n.n_slices, c2n.slice_thickness = "config2_rev", 95.0, 0, 3.0
    c["config2_rev"] = c2n
    return c


def _geom(mr):
    return {f: getattr(mr.cg, f) for f, _ in structs.CtGeom._fields_}


def _ri(mr):
    ri = {f: getattr(mr.ri, f) for f, _ in structs.ReconInfo._fields_ if f != "cb"}
    ri.update({"cb." + f: getattr(mr.ri.cb, f) for f, _ in structs.BlockInfo._fields_})
    return ri


def _sha(ptr, n, itemsize):
    return hashlib.sha256(C.string_at(ptr, n * itemsize)).hexdigest()


def ref_plan(ref, prm, install, spec_end_override=None):
    mr = structs.ReconMetadata()
    ref.ref_configure_recon_params(prm.encode(), C.byref(mr.rp))
    if spec_end_override is not None:
        mr.rp.end_pos = spec_end_override
    mr.install_dir = install.encode()
    ref.ref_configure_ct_geom(C.byref(mr))
    ref.ref_configure_reconstruction(C.byref(mr))
    return mr


def make_plan_fixture(ref, name, spec, out_dir):
    with tempfile.TemporaryDirectory() as d:
        prm, inst = scans.prepare(spec, d)
        open(os.path.join(d, "scan.raw"), "wb").close()
        mr = ref_plan(ref, prm, inst)
        n = spec.n_readings
        fx = {
            "spec": {k: v for k, v in spec.__dict__.items() if not isinstance(v, tuple)},
            "rp_end_pos": mr.rp.end_pos,
            "geom": _geom(mr),
            "plan": _ri(mr),
            "tube_angles_sha256": _sha(mr.tube_angles, n, 4),
            "table_positions_sha256": _sha(mr.table_positions, n, 8),
            "tube_angles_head": [mr.tube_angles[i] for i in range(8)],
            "table_positions_head": [mr.table_positions[i] for i in range(8)],
            "blocks": [],
        }
        for _ in range(mr.ri.n_blocks):
            ref.ref_update_block_info(C.byref(mr))
            fx["blocks"].append(_ri(mr))
        ref.ref_free(C.byref(mr))
    with open(os.path.join(out_dir, "plan_%s.json" % name), "w") as f:
        json.dump(fx, f, indent=1, sort_keys=True)


def make_block_fixture(ref, name, spec, out_dir):
    with tempfile.TemporaryDirectory() as d:
        prm, inst = scans.prepare(spec, d)
        # unit-impulse kernel (ReconKernel 99 -> f_<N>_b99.txt): filter_cpu is then the identity
        n_os = 2 * spec.n_channels
        delta = np.zeros(2 * n_os, np.float32)
        delta[n_os] = 1.0
        delta.tofile(os.path.join(inst, "resources", "filters", "f_%d_b99.txt" % spec.n_channels))
        frames = synth_frames(spec)
        scans.write_raw(os.path.join(d, "scan.raw"), frames)
        mr = ref_plan(ref, prm, inst)
        out = {}
        n_blocks = mr.ri.n_blocks
        plane = mr.rp.nx * mr.rp.ny
        for b in range(n_blocks):
            ref.ref_update_block_info(C.byref(mr))
            ref.ref_extract_projections(C.byref(mr))
            P = mr.ri.n_proj_pull
            n_raw = P * mr.cg.n_rows_raw * mr.cg.n_channels
            nv = P // mr.ri.n_ffs - 2 * mr.cg.add_projections
            n_rb = nv * mr.cg.n_rows * mr.cg.n_channels_oversampled
            raw = np.ctypeslib.as_array(mr.ctd.raw, (n_raw,))
            before = raw.copy()
            out["raw_sha256_b%d" % b] = np.frombuffer(synth.sha256(before).encode(), dtype=np.uint8)
            ref.ref_adaptive_filter_kk(C.byref(mr))
            changed = np.nonzero(raw != before)[0].astype(np.int32)
            out["adaptive_idx_b%d" % b] = changed
            out["adaptive_val_b%d" % b] = raw[changed].copy()
            kept = raw.copy()
            view_sz = mr.cg.n_rows * mr.cg.n_channels_oversampled
            mr.rp.recon_kernel = 99
            ref.ref_rebin_filter_cpu(C.byref(mr))
            rb = np.ctypeslib.as_array(mr.ctd.rebin, (n_rb,)).reshape(nv, view_sz)
            out["rebin_b%d" % b] = rb[::VIEW_STEP].copy()
            raw[:] = kept
            mr.rp.recon_kernel = spec.recon_kernel
            ref.ref_rebin_filter_cpu(C.byref(mr))
            rb = np.ctypeslib.as_array(mr.ctd.rebin, (n_rb,)).reshape(nv, view_sz)
            out["filtered_b%d" % b] = rb[::VIEW_STEP].copy()
            ref.ref_backproject_cpu(C.byref(mr))
        n_img = plane * mr.ri.n_slices_recon
        out["image"] = np.ctypeslib.as_array(mr.ctd.image, (n_img,)).copy()
        ref.ref_finalize_image_stack_cpu(C.byref(mr))
        n_final = int(np.floor(abs(mr.rp.end_pos - mr.rp.start_pos) / mr.rp.slice_thickness) + 1)
        out["final"] = np.ctypeslib.as_array(mr.ctd.final_image_stack, (plane * n_final,)).copy()
        meta = {"spec": {k: v for k, v in spec.__dict__.items() if not isinstance(v, tuple)},
                "n_blocks": int(n_blocks), "n_final": n_final, "view_step": VIEW_STEP,
                "frames_sha256": synth.sha256(frames)}
        out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
        ref.ref_free(C.byref(mr))
    np.savez_compressed(os.path.join(out_dir, "block_%s.npz" % name), **out)


def make_ramp_kat(out_dir):
    kat = {}
    for n in (672, 736):
        taps = np.fromfile(os.path.join(REF_TREE, "resources", "filters", "f_%d_sharp.txt" % n), dtype="<f4")
        c = len(taps) // 2
        kat["f_%d_sharp" % n] = {"n_os": int(c), "centre_taps": [float(v) for v in taps[c - 8:c + 9]],
                                 "sum": float(taps.astype(np.float64).sum())}
    with open(os.path.join(out_dir, "ramp_kat.json"), "w") as f:
        json.dump(kat, f, indent=1)


def main():
    ref = O.reference()
    if ref is None:
        raise SystemExit("the reference tree is needed to generate the golden fixtures")
    for name, spec in planner_cases().items():
        make_plan_fixture(ref, name, spec, HERE)
        print("plan", name)
    for name, spec in golden_cases().items():
        make_block_fixture(ref, name, spec, HERE)
        print("block", name, os.path.getsize(os.path.join(HERE, "block_%s.npz" % name)))
    make_ramp_kat(HERE)


if __name__ == "__main__":
    main()
