"""Synthetic helical scans for the tests and the benchmark (TEST INFRASTRUCTURE).

The reference ships no raw data, so every workload is a seeded phantom -- a
water cylinder (r = 150 mm, mu = 0.019/mm) plus random ellipsoids (semi-axes
5-60 mm, mu 0.015-0.04/mm, random orientation) -- forward-projected with
analytic line integrals and Poisson noise by libctbb_synth.so (ctbb_synth/csrc).
That library also holds the FP32 FMA peak probe the benchmark's roofline
uses.  Neither is part of the reconstruction library libctbb_gb300.so.

  build()                  nvcc -> ctbb_synth/_build/libctbb_synth.so (sm_103a)
  phantom_objects(spec)    the seeded objects of a ScanSpec
  project_host(...)        frames on the CPU (no CUDA call)
  project_device(...)      frames into a device buffer
  fp32_peak_tflops(n, s)   measured FFMA throughput of the current device
"""
import ctypes as C
import math
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
LIB = os.path.join(HERE, "_build", "libctbb_synth.so")
SOURCES = ["phantom.cu", "peak_probe.cu"]
MU_WATER = 0.019


class PhantomObject(C.Structure):
    """struct ctbb_phantom_object: kind 0 = infinite z-cylinder, 1 = ellipsoid."""
    _fields_ = [
        ("kind", C.c_int),
        ("mu", C.c_float),
        ("center", C.c_float * 3),
        ("semi_axes", C.c_float * 3),
        ("rotation", C.c_float * 9),
    ]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libctbb_synth.so")


def build():
    """Compiles libctbb_synth.so when a source is newer than it."""
    srcs = [os.path.join(HERE, "csrc", s) for s in SOURCES]
    deps = srcs + [os.path.join(HERE, "csrc", "synth.h"), os.path.join(REPO, "include", "ctbb_gb300.h")]
    if os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = [_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-lineinfo",
           "-Xcompiler", "-fPIC", "-shared", "-o", LIB + ".tmp", *srcs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(LIB)
        from ctbangbang_gb300.structs import ReconMetadata
        mr = C.POINTER(ReconMetadata)
        obj = C.POINTER(PhantomObject)
        lib.synth_last_error.restype = C.c_char_p
        lib.synth_last_error.argtypes = []
        lib.synth_project_host.restype = C.c_int
        lib.synth_project_host.argtypes = [mr, obj, C.c_int, C.c_size_t, C.c_size_t, C.c_float, C.c_uint64,
                                           C.POINTER(C.c_float)]
        lib.synth_project_device.restype = C.c_int
        lib.synth_project_device.argtypes = [mr, obj, C.c_int, C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t,
                                             C.c_float, C.c_uint64, C.c_void_p, C.c_void_p]
        lib.synth_fp32_peak_tflops.restype = C.c_double
        lib.synth_fp32_peak_tflops.argtypes = [C.c_int, C.c_void_p]
        _lib = lib
    return _lib


def _check(name, status):
    if status != 0:
        raise RuntimeError("%s failed (%d): %s" % (name, status, load().synth_last_error().decode(errors="replace")))


def _rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
    ])


def phantom_objects(spec, z_range=None):
    """Water cylinder + spec.n_ellipsoids seeded random ellipsoids (mu values
    absolute inside each ellipsoid, stored as differences to water)."""
    rng = np.random.default_rng(spec.seed)
    if z_range is None:
        z_range = (spec.start_pos - 5 * spec.slice_thickness, spec.end_pos + 5 * spec.slice_thickness)
    objs = (PhantomObject * (1 + spec.n_ellipsoids))()
    cyl = objs[0]
    cyl.kind = 0
    cyl.mu = MU_WATER
    cyl.semi_axes[0] = spec.cylinder_radius
    r_max = spec.cylinder_radius
    lo, hi = spec.semi_axis_range
    for i in range(spec.n_ellipsoids):
        o = objs[1 + i]
        o.kind = 1
        axes = rng.uniform(lo, hi, size=3)
        rad = rng.uniform(0, max(r_max - axes.max(), 0.0) * 0.9)
        ang = rng.uniform(0, 2 * math.pi)
        zc = rng.uniform(*z_range)
        o.center[:] = [rad * math.cos(ang), rad * math.sin(ang), zc]
        o.semi_axes[:] = list(axes)
        o.rotation[:] = list(_rotation(rng).ravel())
        o.mu = rng.uniform(*spec.mu_range) - MU_WATER
    return objs


def project_host(mr, objs, frame0, n_frames, i0, seed):
    """Host forward projection of frames [frame0, frame0+n_frames) ->
    float32 [n_frames][n_rows_raw][n_channels]."""
    out = np.empty((n_frames, mr.cg.n_rows_raw, mr.cg.n_channels), dtype=np.float32)
    _check("synth_project_host", load().synth_project_host(
        C.byref(mr), objs, len(objs), frame0, n_frames, C.c_float(i0), seed,
        out.ctypes.data_as(C.POINTER(C.c_float))))
    return out


def project_device(mr, objs, d_tube_angles, d_table_positions, frame0, n_frames, i0, seed, d_out, stream=None):
    """Device forward projection into d_out (device pointers as ints)."""
    _check("synth_project_device", load().synth_project_device(
        C.byref(mr), objs, len(objs), C.c_void_p(d_tube_angles), C.c_void_p(d_table_positions), frame0,
        n_frames, C.c_float(i0), seed, C.c_void_p(d_out), C.c_void_p(stream)))


def project_scan_device(torch, mr, spec, seed=None):
    """The whole scan of a plan as a device tensor [n_readings * frame]."""
    n = spec.n_readings
    frame = mr.cg.n_rows_raw * mr.cg.n_channels
    ta = torch.from_numpy(np.ctypeslib.as_array(mr.tube_angles, (n,)).copy()).cuda()
    tp = torch.from_numpy(np.ctypeslib.as_array(mr.table_positions, (n,)).copy()).cuda()
    d = torch.empty(n * frame, dtype=torch.float32, device="cuda")
    project_device(mr, phantom_objects(spec), ta.data_ptr(), tp.data_ptr(), 0, n, spec.i0,
                   spec.seed if seed is None else seed, d.data_ptr(),
                   torch.cuda.current_stream().cuda_stream)
    return d


def fp32_peak_tflops(repeats=5, stream=None):
    return load().synth_fp32_peak_tflops(repeats, C.c_void_p(stream))
