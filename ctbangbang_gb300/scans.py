"""Scan descriptions, .prm / .scanner writers, planning and seeded phantoms.

The reference ships no raw data, so every workload here is a seeded synthetic
helical scan (water cylinder plus random ellipsoids) whose frames the test and
benchmark generator (the synth package) projects; this module only describes
the scans and plans them through the library.

Named workloads (sizes of the benchmark configurations):
  config1  672 ch x 16 rows (1.2 mm), 1152 views/turn, pitch 1.0, 3 turns,
           256^2 @ 0.68 mm, 20 slices of 1.2 mm, ramp kernel, no FFS.
  config2  736 ch x 32 rows (0.6 mm), phi+z FFS (rebinned 1472 x 64), pitch 0.8,
           10 turns, 512^2 @ 0.98 mm, 0.6 mm slices thickened to 3 mm,
           adaptive raw-data filter on, 3 blocks of 32 slices.
  config3  as config2 with 64 raw rows (128 after z-FFS), 40 turns, 512^2 x 400.
Small "tiny_*" scans (64 channels) exercise every FFS mode at sizes the CPU
oracle finishes in well under a second.
"""
import ctypes as C
import dataclasses
import math
import os

import numpy as np

from . import lib as _lib
from .structs import ReconMetadata, ReconParams

MU_WATER = 0.019


@dataclasses.dataclass
class ScanSpec:
    name: str
    # scanner (.scanner keys)
    r_f: float
    src_to_det: float
    anode_angle: float
    fan_angle_increment: float
    central_channel: float
    n_proj_turn: int
    n_channels: int
    # .prm keys
    n_rows: int
    coll: float
    pitch: float              # table feed per turn / (raw rows * coll)
    turns: float
    slice_thickness: float
    recon_fov: float
    nx: int
    ny: int
    start_pos: float
    n_slices: int
    z_ffs: int = 0
    phi_ffs: int = 0
    recon_kernel: int = -100
    acq_fov: float = 500.0
    adaptive_filtration: float = 0.0
    reverse_row_interleave: int = 0
    table_dir: str = "out"
    x_origin: float = 0.0
    y_origin: float = 0.0
    tube_start_angle: float = 0.0
    # phantom
    seed: int = 1
    n_ellipsoids: int = 10
    i0: float = 1e5
    cylinder_radius: float = 150.0
    semi_axis_range: tuple = (5.0, 60.0)
    mu_range: tuple = (0.015, 0.04)

    @property
    def n_rows_raw(self):
        return self.n_rows // (2 ** self.z_ffs)

    @property
    def n_ffs(self):
        return 2 ** (self.z_ffs + self.phi_ffs)

    @property
    def feed(self):
        return self.pitch * self.n_rows_raw * self.coll

    @property
    def n_readings(self):
        return int(round(self.turns * self.n_proj_turn * self.n_ffs))

    @property
    def row_pitch_iso(self):
        """Spacing of the (rebinned) detector rows at the isocentre."""
        return self.coll / (2 ** self.z_ffs)

    @property
    def theta_cone(self):
        half = 0.5 * (self.n_rows - 1) * self.row_pitch_iso
        return 2.0 * math.atan(half / self.r_f)

    @property
    def end_pos(self):
        return self.start_pos + (self.n_slices - 1) * self.slice_thickness


def _definition_as(**kw):
    base = dict(r_f=595.0, src_to_det=1085.6, anode_angle=0.1222,
                fan_angle_increment=0.0011844, central_channel=366.25,
                n_proj_turn=1152, n_channels=736)
    base.update(kw)
    return base


CONFIGS = {
    "config1": ScanSpec(
        name="config1", r_f=595.0, src_to_det=1085.6, anode_angle=0.1222,
        fan_angle_increment=1.4 / 1085.6, central_channel=336.25, n_proj_turn=1152,
        n_channels=672, n_rows=16, coll=1.2, pitch=1.0, turns=3, slice_thickness=1.2,
        recon_fov=256 * 0.68, nx=256, ny=256, start_pos=17.5, n_slices=20,
        seed=1000, n_ellipsoids=10, i0=1e5),
    "config2": ScanSpec(
        name="config2", **_definition_as(), n_rows=64, coll=0.6, pitch=0.8, turns=10,
        slice_thickness=3.0, recon_fov=512 * 0.98, nx=512, ny=512, start_pos=50.0,
        n_slices=16, z_ffs=1, phi_ffs=1, adaptive_filtration=1.0,
        seed=2000, n_ellipsoids=30, i0=5e4),
    "config3": ScanSpec(
        name="config3", **_definition_as(), n_rows=128, coll=0.6, pitch=0.8, turns=40,
        slice_thickness=0.6, recon_fov=512 * 0.98, nx=512, ny=512, start_pos=60.0,
        n_slices=400, z_ffs=1, phi_ffs=1, adaptive_filtration=1.0,
        seed=3000, n_ellipsoids=30, i0=5e4),
}


def tiny(z_ffs=0, phi_ffs=0, *, n_channels=64, n_rows_raw=4, nx=32, ny=32, n_slices=8,
         seed=7, adaptive_filtration=0.0, turns=None, reverse_row_interleave=0,
         table_dir="out", start_pos=None, slice_thickness=None, n_proj_turn=96, i0=1e5,
         fan_angle_increment=None, recon_kernel=-100, pitch=1.0):
    """A small scan of any FFS mode (default 64 channels, 96 views/turn, 32^2 pixels)."""
    fai = fan_angle_increment if fan_angle_increment is not None else 0.48 / n_channels
    n_rows = n_rows_raw * 2 ** z_ffs
    coll = 1.0
    st = slice_thickness if slice_thickness is not None else coll
    spec = ScanSpec(
        name="tiny_z%d_p%d" % (z_ffs, phi_ffs), r_f=300.0, src_to_det=550.0, anode_angle=0.1222,
        fan_angle_increment=fai, central_channel=(n_channels / 2) - 0.75, recon_kernel=recon_kernel,
        n_proj_turn=n_proj_turn, n_channels=n_channels, n_rows=n_rows, coll=coll, pitch=pitch,
        turns=1.0, slice_thickness=st, recon_fov=100.0, nx=nx, ny=ny, start_pos=start_pos,
        n_slices=n_slices, z_ffs=z_ffs, phi_ffs=phi_ffs, adaptive_filtration=adaptive_filtration,
        reverse_row_interleave=reverse_row_interleave, table_dir=table_dir, seed=seed,
        n_ellipsoids=4, i0=i0, cylinder_radius=60.0, semi_axis_range=(5.0, 20.0))
    if start_pos is None:
        spec.start_pos = allowed_margin(spec) + 2.0
    if turns is None:
        spec.turns = needed_turns(spec)
    else:
        spec.turns = turns
    return spec


def allowed_margin(spec):
    """Distance from the first frame to the first allowed slice position
    (projection_padding of src/setup.cu:514)."""
    n_proj_ffs = spec.n_proj_turn * spec.n_ffs
    add = int((spec.fan_angle_increment * spec.n_channels / 2) / (2 * math.pi / spec.n_proj_turn) + 10)
    return spec.feed * (n_proj_ffs // 2 + add * spec.n_ffs + 256) / n_proj_ffs


def needed_turns(spec, margin_turns=0.25):
    """Smallest whole number of quarter turns whose frames cover every pull window."""
    n_proj_ffs = spec.n_proj_turn * spec.n_ffs
    add = int((spec.fan_angle_increment * spec.n_channels / 2) / (2 * math.pi / spec.n_proj_turn) + 10)
    add_ffs = add * spec.n_ffs
    recon_span = spec.end_pos - spec.start_pos + 2 * spec.slice_thickness
    n_block = 32
    n_req = int(math.floor(recon_span / spec.coll)) + 1
    n_recon = (n_req - 1) + (n_block - (n_req - 1) % n_block)
    z_last = spec.start_pos - spec.slice_thickness + (n_recon - 1) * spec.coll
    frames = z_last / spec.feed * n_proj_ffs + n_proj_ffs / 2 + add_ffs + 256 + 128 + n_proj_ffs
    turns = frames / n_proj_ffs + margin_turns
    return max(math.ceil(turns * 4) / 4.0, 1001.0 / n_proj_ffs + 0.25)


# --------------------------------------------------------------------------
# files
# --------------------------------------------------------------------------

def write_scanner(spec, path):
    with open(path, "w") as f:
        f.write("%% synthetic scanner %s %%\n" % spec.name)
        f.write("RSrcToIso:\t%.9g\n" % spec.r_f)
        f.write("RSrcToDet:\t%.9g\n" % spec.src_to_det)
        f.write("AnodeAngle:\t%.9g\n" % spec.anode_angle)
        f.write("FanAngleInc:\t%.9g\n" % spec.fan_angle_increment)
        f.write("ThetaCone:\t%.9g\n" % spec.theta_cone)
        f.write("CentralChannel:\t%.9g\n" % spec.central_channel)
        f.write("NProjTurn:\t%d\n" % spec.n_proj_turn)
        f.write("NChannels:\t%d\n" % spec.n_channels)
        f.write("ReverseRowInterleave:\t%d\n" % spec.reverse_row_interleave)
        f.write("ReverseChanInterleave:\t0\n")


def write_prm(spec, path, raw_dir, raw_file, scanner_path, out_dir=None):
    lines = [
        ("RawDataDir:", raw_dir), ("RawDataFile:", raw_file),
        ("OutputDir:", out_dir or raw_dir), ("OutputFile:", spec.name + ".img"),
        ("Nrows:", "%d" % spec.n_rows), ("CollSlicewidth:", "%.9g" % spec.coll),
        ("StartPos:", "%.9g" % spec.start_pos), ("EndPos:", "%.9g" % spec.end_pos),
        ("PitchValue:", "%.9g" % spec.feed), ("SliceThickness:", "%.9g" % spec.slice_thickness),
        ("AcqFOV:", "%.9g" % spec.acq_fov), ("ReconFOV:", "%.9g" % spec.recon_fov),
        ("ReconKernel:", "%d" % spec.recon_kernel), ("Readings:", "%d" % spec.n_readings),
        ("Xorigin:", "%.9g" % spec.x_origin), ("Yorigin:", "%.9g" % spec.y_origin),
        ("Zffs:", "%d" % spec.z_ffs), ("Phiffs:", "%d" % spec.phi_ffs),
        ("Scanner:", scanner_path), ("FileType:", "0"), ("FileSubType:", "0"),
        ("RawOffset:", "0"), ("Nx:", "%d" % spec.nx), ("Ny:", "%d" % spec.ny),
        ("TubeStartAngle:", "%.9g" % spec.tube_start_angle),
        ("AdaptiveFiltration:", "%.9g" % spec.adaptive_filtration),
        ("TableDir:", spec.table_dir),
    ]
    with open(path, "w") as f:
        f.write("%% %s %%\n" % spec.name)
        for k, v in lines:
            f.write("%s\t%s\n" % (k, v))


def write_ramp_filter(spec, install_dir):
    """Writes f_<N>_ramp.txt (float32 taps) under install_dir/resources/filters."""
    n_os = 2 * spec.n_channels
    ds = np.float32(spec.r_f * math.sin(np.float32(spec.fan_angle_increment) / 2.0))
    taps = (C.c_float * (2 * n_os))()
    _lib.call("ctbb_ramp_filter_taps", n_os, C.c_float(float(ds)), 1.0, 1.0, taps)
    d = os.path.join(install_dir, "resources", "filters")
    os.makedirs(d, exist_ok=True)
    path = os.path.join(d, "f_%d_ramp.txt" % spec.n_channels)
    np.frombuffer(taps, dtype=np.float32).tofile(path)
    return path


def prepare(spec, workdir, raw_file="scan.raw"):
    """Writes the .scanner, .prm and ramp filter of spec into workdir.
    Returns (prm_path, install_dir)."""
    os.makedirs(workdir, exist_ok=True)
    scanner = os.path.join(workdir, spec.name + ".scanner")
    write_scanner(spec, scanner)
    prm = os.path.join(workdir, spec.name + ".prm")
    write_prm(spec, prm, workdir, raw_file, scanner)
    write_ramp_filter(spec, workdir)
    return prm, workdir


# --------------------------------------------------------------------------
# planning through the library (the reference's setup.cu sequence)
# --------------------------------------------------------------------------

def plan(prm_path, install_dir):
    """configure_recon_params -> configure_ct_geom -> configure_reconstruction.
    Returns a ReconMetadata whose host arrays the library allocated."""
    mr = ReconMetadata()
    rp = ReconParams()
    _lib.call("ctbb_configure_recon_params", prm_path.encode(), C.byref(rp))
    mr.rp = rp
    mr.install_dir = install_dir.encode()
    _lib.call("ctbb_configure_ct_geom", C.byref(mr))
    _lib.call("ctbb_configure_reconstruction", C.byref(mr))
    return mr


def plan_spec(spec, workdir):
    prm, inst = prepare(spec, workdir)
    return plan(prm, inst)


def free_plan(mr):
    """Frees the host arrays of a plan (ctbb_finish_and_cleanup without the file)."""
    mr.ctd.final_image_stack = None
    _lib.call("ctbb_finish_and_cleanup", C.byref(mr))


def write_raw(path, frames):
    np.ascontiguousarray(frames, dtype="<f4").tofile(path)
