"""CPU tests pinning the oracle restatement: against the golden fixtures the
reference's own CPU code produced, and (where the reference build is present)
against that build directly on fresh inputs."""
import ctypes as C
import glob
import json
import os
import platform

import numpy as np
import pytest

from ctbangbang_gb300 import lib as L
from ctbangbang_gb300 import scans
from tests import helpers as H
from tests.conftest import REPO

GOLDEN = os.path.join(REPO, "tests", "golden")


# The golden fixtures were made on x86_64.  The rebin tables (fan angles and
# their inverse search) come from the host libm's asinf/sinf/cosf, which on
# aarch64 may differ from x86_64 glibc by an ulp; on another architecture the
# unfiltered rebin is therefore compared to 2e-6 relative instead of exactly.
# (On any one machine the GPU rebin is bit-exact with the oracle.)
SAME_LIBM_AS_GOLDEN = platform.machine() in ("x86_64", "AMD64")


def assert_rebin_matches_golden(got, golden):
    """Unfiltered rebin vs the golden made through a unit-impulse kernel: that
    pass is exact except on samples that were exactly 0 (frames past the end
    of the data), where the reference's double FFT leaves ~1e-16 of roundoff."""
    zero = np.abs(golden) < 1e-9
    if SAME_LIBM_AS_GOLDEN:
        np.testing.assert_array_equal(got[~zero], golden[~zero])
    else:
        np.testing.assert_allclose(got[~zero], golden[~zero], rtol=2e-6, atol=1e-7)
    assert np.all(np.abs(got[zero]) < 1e-9)


def golden_block_files():
    return sorted(glob.glob(os.path.join(GOLDEN, "block_*.npz")))


def load_case(path):
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden
    import synth
    z = np.load(path)
    meta = json.loads(bytes(z["meta"]).decode())
    keep = {k: v for k, v in meta["spec"].items() if k in scans.ScanSpec.__dataclass_fields__}
    spec = scans.ScanSpec(**keep)
    frames = make_golden.synth_frames(spec)
    assert synth.sha256(frames) == meta["frames_sha256"], "synthetic input not reproduced bit for bit"
    return z, meta, spec, frames


class GoldenScan(H.Scan):
    """H.Scan whose frames are the golden synthetic input."""

    def __init__(self, spec, frames, workdir):
        self.spec = spec
        self._tmp = None
        self.workdir = workdir
        self.prm, self.install = scans.prepare(spec, workdir)
        self.mr = scans.plan(self.prm, self.install)
        self.frames = frames


@pytest.mark.parametrize("path", golden_block_files(), ids=lambda p: os.path.basename(p)[6:-4])
def test_oracle_matches_reference_golden(lib, oracle_lib, tmp_path, path):
    z, meta, spec, frames = load_case(path)
    scan = GoldenScan(spec, frames, str(tmp_path))
    step = meta["view_step"]
    mr = scan.mr
    for b in range(meta["n_blocks"]):
        raw = scan.next_block()
        d = H.dims(mr)
        import synth
        assert synth.sha256(raw) == bytes(z["raw_sha256_b%d" % b]).decode()
        st = H.oracle_block(oracle_lib, scan, raw, adaptive=True)
        changed = np.nonzero(st["adaptive"] != raw)[0]
        np.testing.assert_array_equal(changed, z["adaptive_idx_b%d" % b])
        np.testing.assert_array_equal(st["adaptive"][changed], z["adaptive_val_b%d" % b])
        vs = mr.cg.n_rows * mr.cg.n_channels_oversampled
        assert_rebin_matches_golden(st["rebin"].reshape(-1, vs)[::step], z["rebin_b%d" % b])
        got_f = st["filtered"].reshape(-1, vs)[::step]
        if SAME_LIBM_AS_GOLDEN:
            np.testing.assert_array_equal(got_f, z["filtered_b%d" % b])
        else:
            # the ramp filter (a high-pass: outputs far below its inputs) carries
            # the rebin's ulp-level input differences; 3.4e-6 of the row
            # maximum seen on aarch64
            np.testing.assert_allclose(got_f, z["filtered_b%d" % b], rtol=0, atol=1e-5 * np.abs(got_f).max())
    if SAME_LIBM_AS_GOLDEN:
        np.testing.assert_array_equal(H.view(mr.ctd.image, d["n_image"]), z["image"])
    else:
        mx, rms = H.hu_errors(H.view(mr.ctd.image, d["n_image"]), z["image"])
        assert mx <= 1.0 and rms <= 0.1
    oracle_lib.oracle_finalize(C.byref(mr))
    n_final = L.load().ctbb_n_slices_final(C.byref(mr))
    assert n_final == meta["n_final"]
    fin = H.view(mr.ctd.final_image_stack, n_final * d["plane"])
    if SAME_LIBM_AS_GOLDEN:
        np.testing.assert_array_equal(fin, z["final"])
    else:
        mx, rms = H.hu_errors(fin, z["final"])
        assert mx <= 1.0 and rms <= 0.1
    scan.close()


@pytest.mark.parametrize("z_ffs,phi_ffs", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_oracle_bit_exact_vs_reference_build(lib, oracle_lib, ref_lib, tmp_path, z_ffs, phi_ffs):
    """Fresh phantom scans through the reference's own CPU functions and the
    oracle: every stage identical."""
    spec = scans.tiny(z_ffs, phi_ffs, adaptive_filtration=3.0, seed=100 + 2 * z_ffs + phi_ffs)
    scan = H.Scan(spec, str(tmp_path))
    from ctbangbang_gb300 import structs
    mref = structs.ReconMetadata()
    ref_lib.ref_configure_recon_params(scan.prm.encode(), C.byref(mref.rp))
    mref.install_dir = scan.install.encode()
    ref_lib.ref_configure_ct_geom(C.byref(mref))
    ref_lib.ref_configure_reconstruction(C.byref(mref))
    mr = scan.mr
    for _ in range(mr.ri.n_blocks):
        raw = scan.next_block()
        ref_lib.ref_update_block_info(C.byref(mref))
        ref_lib.ref_extract_projections(C.byref(mref))
        d = H.dims(mr)
        np.testing.assert_array_equal(H.view(mref.ctd.raw, d["n_raw"]), raw)
        ref_lib.ref_adaptive_filter_kk(C.byref(mref))
        oracle_lib.oracle_adaptive_filter(C.byref(mr))
        np.testing.assert_array_equal(H.view(mr.ctd.raw, d["n_raw"]), H.view(mref.ctd.raw, d["n_raw"]))
        ref_lib.ref_rebin_filter_cpu(C.byref(mref))
        assert oracle_lib.oracle_rebin_filter(C.byref(mr)) == 0
        np.testing.assert_array_equal(H.view(mr.ctd.rebin, d["n_rebin"]), H.view(mref.ctd.rebin, d["n_rebin"]))
        ref_lib.ref_backproject_cpu(C.byref(mref))
        oracle_lib.oracle_backproject(C.byref(mr))
        np.testing.assert_array_equal(H.view(mr.ctd.image, d["n_image"]), H.view(mref.ctd.image, d["n_image"]))
    ref_lib.ref_finalize_image_stack_cpu(C.byref(mref))
    oracle_lib.oracle_finalize(C.byref(mr))
    nf = L.load().ctbb_n_slices_final(C.byref(mr)) * d["plane"]
    np.testing.assert_array_equal(H.view(mr.ctd.final_image_stack, nf), H.view(mref.ctd.final_image_stack, nf))
    ref_lib.ref_free(C.byref(mref))
    scan.close()


def test_interp_edge_rules_match_reference(oracle_lib, ref_lib):
    """interp2 border (value 0 beyond [0, dim-2]) and interp3 clamping/aliasing."""
    rng = np.random.default_rng(3)
    a = rng.standard_normal(6 * 5 * 4).astype(np.float32)
    p = a.ctypes.data_as(C.POINTER(C.c_float))
    pts = [-1.0, -0.0, 0.0, 0.25, 3.0, 3.5, 4.0, 4.0001, 5.0, 6.0]
    for i1 in pts:
        for i2 in pts:
            assert oracle_lib.oracle_interp2(p, 6, 5, i1, i2) == ref_lib.ref_interp2(p, 6, 5, i1, i2)
            for i3 in (-2.0, 0.0, 1.5, 3.0, 3.25, 9.0):
                x = oracle_lib.oracle_interp3(p, 6, 5, 4, i1, i2, i3)
                y = ref_lib.ref_interp3(p, 6, 5, 4, i1, i2, i3)
                assert x == y or (np.isnan(x) and np.isnan(y))


@pytest.mark.parametrize("z_ffs,phi_ffs", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_fp32_reference_path_vs_fp64_oracle(lib, oracle_lib, tmp_path, z_ffs, phi_ffs):
    """The reference's FP32 arithmetic (the oracle's float template) against
    its FP64 template on one block: the precision the reference path itself
    has, against which the GPU's 1 HU / 0.1 HU bars are set."""
    spec = scans.tiny(z_ffs, phi_ffs, adaptive_filtration=3.0, seed=200 + 2 * z_ffs + phi_ffs)
    scan = H.Scan(spec, str(tmp_path))
    raw = scan.next_block()
    f32 = H.oracle_block(oracle_lib, scan, raw)["block"].astype(np.float64)
    taps = H.taps_of(scan.mr)
    f64 = np.zeros(f32.size, np.float64)
    oracle_lib.oracle64_block(C.byref(scan.mr), raw.ctypes.data_as(C.POINTER(C.c_float)), 1,
                              taps.ctypes.data_as(C.POINTER(C.c_float)), f64.ctypes.data_as(C.POINTER(C.c_double)))
    mx, rms = H.hu_errors(f32, f64)
    assert np.abs(f64).max() > 0.01
    assert mx <= 0.1 and rms <= 0.01, (mx, rms)
    scan.close()


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "plan_*.json"))),
                         ids=lambda p: os.path.basename(p))
def test_oracle_planner_bit_exact_vs_reference_golden(oracle_lib, tmp_path, path):
    """The oracle's planner restatement (used by the benchmark's reference arm,
    which must not load the reconstruction library) reproduces the reference
    planner's integers and float tables exactly, from the .prm and .scanner
    files it parses itself."""
    import hashlib

    from ctbangbang_gb300 import structs
    from oracle import plan as OP
    fx = json.load(open(path))
    keep = {k: v for k, v in fx["spec"].items() if k in scans.ScanSpec.__dataclass_fields__}
    spec = scans.ScanSpec(**keep)
    mr = OP.plan_spec(spec, str(tmp_path))
    n = spec.n_readings
    for k, v in fx["geom"].items():
        assert np.float32(getattr(mr.cg, k)) == np.float32(v), k
    assert np.float32(mr.rp.end_pos) == np.float32(fx["rp_end_pos"])

    def ri_of(ri):
        d = {f: getattr(ri, f) for f, _ in structs.ReconInfo._fields_ if f != "cb"}
        d.update({"cb." + f: getattr(ri.cb, f) for f, _ in structs.BlockInfo._fields_})
        return d

    got = ri_of(mr.ri)
    for k, v in fx["plan"].items():
        assert (np.float32(got[k]) == np.float32(v)) if isinstance(v, float) else got[k] == v, k
    assert hashlib.sha256(C.string_at(mr.tube_angles, 4 * n)).hexdigest() == fx["tube_angles_sha256"]
    assert hashlib.sha256(C.string_at(mr.table_positions, 8 * n)).hexdigest() == fx["table_positions_sha256"]
    blocks = OP.block_plans(mr)
    assert len(blocks) == len(fx["blocks"]) == mr.ri.n_blocks
    for ri, blk in zip(blocks, fx["blocks"]):
        got = ri_of(ri)
        for k, v in blk.items():
            assert (np.float32(got[k]) == np.float32(v)) if isinstance(v, float) else got[k] == v, (k, got[k], v)
    OP.free_plan(mr)


def test_oracle_ramp_taps_match_reference_sharp_kernel(oracle_lib):
    """resources/ramp.m restated in the oracle equals the reference's shipped
    f_<N>_sharp taps (the ramp formula with c = a = 1, ds = r_f sin(fai/2))."""
    kat = json.load(open(os.path.join(GOLDEN, "ramp_kat.json")))
    geo = {"f_736_sharp": (595.0, 0.067864 * 3.1415926535897 / 180.0),   # Definition AS
           "f_672_sharp": (570.0, 0.07758621 * 3.1415926535897 / 180.0)}  # Sensation 64
    for name, fx in kat.items():
        r_f, fai = geo[name]
        n_os = fx["n_os"]
        taps = np.zeros(2 * n_os, np.float32)
        ds = np.float32(r_f * np.sin(np.float32(fai) / 2.0))
        oracle_lib.oracle_ramp_taps(n_os, C.c_float(float(ds)), 1.0, 1.0, taps.ctypes.data_as(C.POINTER(C.c_float)))
        np.testing.assert_allclose(taps[n_os - 8:n_os + 9], fx["centre_taps"], rtol=0, atol=2e-7)
        assert abs(taps.astype(np.float64).sum() - fx["sum"]) < 1e-5
