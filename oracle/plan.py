"""Planning a scan with the oracle alone (TEST INFRASTRUCTURE).

The benchmark's reference arm and the oracle tests plan scans without the
reconstruction library: the .scanner / .prm files are written by
ctbangbang_gb300.scans (plain Python), the ramp kernel file by the oracle's
restatement of resources/ramp.m, and the plan by the oracle's restatement of
the reference planner (ctbb_oracle_plan.cpp: configure_recon_params,
configure_ct_geom, configure_reconstruction, update_block_info of
src/setup.cu).  Nothing here loads libctbb_gb300.so.
"""
import ctypes as C
import math
import os

import numpy as np

from ctbangbang_gb300 import scans
from ctbangbang_gb300.structs import ReconInfo, ReconMetadata, ReconParams

from . import oracle as _oracle


class OraclePlanError(RuntimeError):
    pass


def _check(name, status):
    if status != 0:
        raise OraclePlanError("%s failed with status %d" % (name, status))


def write_ramp_filter(spec, install_dir):
    """f_<N>_ramp.txt (float32 taps, resources/ramp.m with c = a = 1) under
    install_dir/resources/filters."""
    orc = _oracle.oracle()
    n_os = 2 * spec.n_channels
    ds = np.float32(spec.r_f * math.sin(np.float32(spec.fan_angle_increment) / 2.0))
    taps = (C.c_float * (2 * n_os))()
    _check("oracle_ramp_taps", orc.oracle_ramp_taps(n_os, C.c_float(float(ds)), 1.0, 1.0, taps))
    d = os.path.join(install_dir, "resources", "filters")
    os.makedirs(d, exist_ok=True)
    path = os.path.join(d, "f_%d_ramp.txt" % spec.n_channels)
    np.frombuffer(taps, dtype=np.float32).tofile(path)
    return path


def prepare(spec, workdir, raw_file="scan.raw"):
    """.scanner, .prm and ramp kernel of spec in workdir -> (prm, install_dir)."""
    os.makedirs(workdir, exist_ok=True)
    scanner = os.path.join(workdir, spec.name + ".scanner")
    scans.write_scanner(spec, scanner)
    prm = os.path.join(workdir, spec.name + ".prm")
    scans.write_prm(spec, prm, workdir, raw_file, scanner)
    write_ramp_filter(spec, workdir)
    return prm, workdir


def plan(prm_path, install_dir):
    """configure_recon_params -> configure_ct_geom -> configure_reconstruction
    of the oracle.  The per-frame tables are the oracle's (free_plan frees
    them); ctd.raw / rebin / image stay null."""
    orc = _oracle.oracle()
    mr = ReconMetadata()
    rp = ReconParams()
    _check("oracle_configure_recon_params", orc.oracle_configure_recon_params(prm_path.encode(), C.byref(rp)))
    mr.rp = rp
    mr.install_dir = install_dir.encode()
    _check("oracle_configure_ct_geom", orc.oracle_configure_ct_geom(C.byref(mr)))
    _check("oracle_configure_reconstruction", orc.oracle_configure_reconstruction(C.byref(mr)))
    return mr


def plan_spec(spec, workdir):
    return plan(*prepare(spec, workdir))


def block_plans(mr):
    """recon_info of every block, from update_block_info in sequence (mr is
    left unchanged)."""
    orc = _oracle.oracle()
    m = ReconMetadata()
    C.memmove(C.byref(m), C.byref(mr), C.sizeof(m))
    m.ri.cb.block_idx = 0
    out = []
    for _ in range(mr.ri.n_blocks):
        _check("oracle_update_block_info", orc.oracle_update_block_info(C.byref(m)))
        ri = ReconInfo()
        C.memmove(C.byref(ri), C.byref(m.ri), C.sizeof(ri))
        out.append(ri)
    return out


def free_plan(mr):
    _oracle.oracle().oracle_free_plan(C.byref(mr))
