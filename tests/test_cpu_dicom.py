"""CPU tests of the DICOM CT image series writer (ctbb_write_dicom_series).
Each file is parsed back by a strict reader of the PS3.10 / PS3.5 encoding
(preamble, "DICM", file meta group length, explicit VR little endian, even
value lengths, ascending tags) and its geometry and pixels are checked
against the plan and the stack."""
import ctypes as C
import os
import re
import struct

import numpy as np
import pytest

from ctbangbang_gb300 import lib as L
from ctbangbang_gb300 import scans

LONG_VRS = {b"OB", b"OW", b"OF", b"SQ", b"UT", b"UN"}
UID = re.compile(r"^(0|[1-9][0-9]*)(\.(0|[1-9][0-9]*))*$")


def read_part10(path):
    """{(group, element): (vr, raw value)} of a Part-10 file, checked strictly."""
    d = open(path, "rb").read()
    assert d[:128] == b"\0" * 128 and d[128:132] == b"DICM"
    i, out, last = 132, {}, (0, 0)
    meta_end = None
    while i < len(d):
        g, e = struct.unpack("<HH", d[i:i + 4])
        vr = d[i + 4:i + 6]
        if vr in LONG_VRS:
            assert d[i + 6:i + 8] == b"\0\0"
            n, h = struct.unpack("<I", d[i + 8:i + 12])[0], 12
        else:
            n, h = struct.unpack("<H", d[i + 6:i + 8])[0], 8
        assert n % 2 == 0, ((g, e), n)
        assert (g, e) > last, ((g, e), last)  # ascending, no repeats
        last = (g, e)
        out[(g, e)] = (vr.decode(), d[i + h:i + h + n])
        i += h + n
        if (g, e) == (0x0002, 0x0000):
            meta_end = i + struct.unpack("<I", out[(g, e)][1])[0]
        if g == 0x0002:
            assert i <= meta_end
        elif meta_end is not None:
            assert i > meta_end
    assert i == len(d)
    return out


def text(v):
    return v[1].rstrip(b"\0 ").decode()


def us(v):
    assert v[0] == "US"
    return struct.unpack("<H", v[1])[0]


@pytest.fixture
def planned(lib, tmp_path):
    spec = scans.tiny(0, 1, nx=24, ny=20, n_slices=5, seed=91)
    spec.x_origin, spec.y_origin = 3.5, -2.0
    mr = scans.plan_spec(spec, str(tmp_path / "plan"))
    yield spec, mr
    scans.free_plan(mr)


def test_series_round_trip(lib, tmp_path, planned):
    spec, mr = planned
    n = lib.ctbb_n_slices_final(C.byref(mr))
    assert n == 5
    nx, ny = mr.rp.nx, mr.rp.ny
    rng = np.random.default_rng(5)
    mu_w = np.float32(scans.MU_WATER)
    stack = (mu_w * (1.0 + rng.uniform(-1.2, 2.0, (n, ny, nx)))).astype(np.float32)
    stack[0, 0, 0] = mu_w * 40.0   # 39000 HU: clamped to 32767
    stack[0, 0, 1] = -mu_w * 40.0  # clamped to -32768
    out = tmp_path / "dcm"
    out.mkdir()
    mr.rp.output_file = b"recon.img"
    L.call("ctbb_write_dicom_series", C.byref(mr),
           stack.ctypes.data_as(C.POINTER(C.c_float)), n, C.c_float(float(mu_w)), str(out).encode())
    files = sorted(os.listdir(out))
    assert files == ["recon_%04d.dcm" % (k + 1) for k in range(n)]
    hu = 1000.0 * (stack.astype(np.float64) - float(mu_w)) / float(mu_w)
    want = np.clip(np.rint(hu), -32768, 32767).astype(np.int16)
    pix_x, pix_y = mr.rp.recon_fov / nx, mr.rp.recon_fov / ny
    direction = 1 if mr.rp.end_pos >= mr.rp.start_pos else -1
    studies, series, sops = set(), set(), set()
    for k, name in enumerate(files):
        t = read_part10(str(out / name))
        assert text(t[(0x0002, 0x0002)]) == text(t[(0x0008, 0x0016)]) == "1.2.840.10008.5.1.4.1.1.2"
        assert text(t[(0x0002, 0x0010)]) == "1.2.840.10008.1.2.1"
        assert text(t[(0x0002, 0x0003)]) == text(t[(0x0008, 0x0018)])
        for tag in ((0x0002, 0x0003), (0x0020, 0x000D), (0x0020, 0x000E), (0x0020, 0x0052)):
            uid = text(t[tag])
            assert t[tag][0] == "UI" and len(uid) <= 64 and UID.match(uid), uid
        studies.add(text(t[(0x0020, 0x000D)]))
        series.add(text(t[(0x0020, 0x000E)]))
        sops.add(text(t[(0x0008, 0x0018)]))
        assert text(t[(0x0008, 0x0060)]) == "CT"
        assert text(t[(0x0010, 0x0010)]) == "" and text(t[(0x0010, 0x0020)]) == ""
        assert int(text(t[(0x0020, 0x0013)])) == k + 1
        assert us(t[(0x0028, 0x0010)]) == ny and us(t[(0x0028, 0x0011)]) == nx
        assert [us(t[(0x0028, e)]) for e in (0x0002, 0x0100, 0x0101, 0x0102, 0x0103)] == [1, 16, 16, 15, 1]
        assert text(t[(0x0028, 0x0004)]) == "MONOCHROME2"
        for tag in ((0x0018, 0x0050), (0x0020, 0x0032), (0x0028, 0x0030), (0x0020, 0x1041)):
            assert t[tag][0] == "DS" and all(len(v) <= 16 for v in text(t[tag]).split("\\"))
        sp = [float(v) for v in text(t[(0x0028, 0x0030)]).split("\\")]
        np.testing.assert_allclose(sp, [pix_y, pix_x], rtol=1e-8)
        pos = [float(v) for v in text(t[(0x0020, 0x0032)]).split("\\")]
        z = np.float32(mr.rp.start_pos) + np.float32(direction * k) * np.float32(mr.rp.slice_thickness)
        np.testing.assert_allclose(pos, [pix_x * (0 - (nx - 1) / 2) + mr.rp.x_origin,
                                         pix_y * (0 - (ny - 1) / 2) + mr.rp.y_origin, z], rtol=1e-8, atol=1e-6)
        assert float(text(t[(0x0020, 0x1041)])) == pytest.approx(float(z), abs=1e-6)
        assert float(text(t[(0x0018, 0x0050)])) == pytest.approx(float(mr.rp.slice_thickness))
        assert [text(t[(0x0028, e)]) for e in (0x1052, 0x1053, 0x1054)] == ["0", "1", "HU"]
        vr, raw = t[(0x7FE0, 0x0010)]
        assert vr == "OW"
        np.testing.assert_array_equal(np.frombuffer(raw, "<i2").reshape(ny, nx), want[k])
    assert len(studies) == 1 and len(series) == 1 and len(sops) == n


def test_hu_stack_written_as_is_and_errors(lib, tmp_path, planned):
    spec, mr = planned
    nx, ny = mr.rp.nx, mr.rp.ny
    stack = np.full((1, ny, nx), -1000.4, np.float32)
    stack[0, 3, 4] = 41.6
    out = tmp_path / "hu"
    out.mkdir()
    mr.rp.output_file = b""
    L.call("ctbb_write_dicom_series", C.byref(mr), stack.ctypes.data_as(C.POINTER(C.c_float)), 1,
           C.c_float(0.0), str(out).encode())
    t = read_part10(str(out / "slice_0001.dcm"))  # OutputFile empty: "slice"
    px = np.frombuffer(t[(0x7FE0, 0x0010)][1], "<i2").reshape(ny, nx)
    assert px[3, 4] == 42 and px[0, 0] == -1000
    ptr = stack.ctypes.data_as(C.POINTER(C.c_float))
    st = lib.ctbb_write_dicom_series(C.byref(mr), ptr, 1, C.c_float(0.0), str(tmp_path / "absent").encode())
    assert L.STATUS[st] == "CTBB_ERR_IO"
    st = lib.ctbb_write_dicom_series(C.byref(mr), ptr, 0, C.c_float(0.0), str(out).encode())
    assert L.STATUS[st] == "CTBB_ERR_ARGUMENT"
