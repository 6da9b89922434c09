"""Platform-exact synthetic raw frames for the golden fixtures.

Frames are sinogram-like float32 data built only from IEEE-exact operations
(+, -, *, /, sqrt on float32 and integer hashing), so numpy regenerates them
bit for bit on any machine and the fixtures need not store the input.  Each
frame holds a water-like disc (radius 60 mm) plus three off-centre discs whose
projected centres move with the view angle along a triangle wave, a mild row
dependence, and uniform noise from a counter-based integer hash.
"""
import hashlib

import numpy as np


def _mix64(z):
    z = (z + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    return z ^ (z >> np.uint64(31))


def frames(n_frames, n_rows, n_channels, n_proj_ffs, central_channel, channel_mm, seed, noise=0.02):
    f32 = np.float32
    f = np.arange(n_frames, dtype=np.int64)
    t = ((f % n_proj_ffs).astype(f32) / f32(n_proj_ffs))                # [0, 1)
    u = (np.arange(n_channels, dtype=f32) - f32(central_channel)) * f32(channel_mm)
    out = np.zeros((n_frames, n_rows, n_channels), dtype=f32)

    def chord(radius, centre):
        d = u[None, :] - centre[:, None]
        return f32(2) * np.sqrt(np.maximum(f32(radius) * f32(radius) - d * d, f32(0)))

    base = chord(60.0, np.zeros(n_frames, f32)) * f32(0.019)
    discs = np.zeros((n_frames, n_channels), f32)
    for k, (r0, a, mu, ph) in enumerate([(25.0, 12.0, 0.012, 0.0), (35.0, 8.0, -0.006, 0.37),
                                         (10.0, 15.0, 0.008, 0.71)]):
        tt = t + f32(ph)
        tt = tt - np.floor(tt)
        tri = np.abs(f32(4) * tt - f32(2)) - f32(1)                        # triangle wave in [-1, 1]
        discs = discs + chord(a, f32(r0) * tri) * f32(mu)
    rows = np.arange(n_rows, dtype=f32)
    out[:] = (base + discs)[:, None, :] * (f32(1) + f32(0.01) * rows)[None, :, None]
    idx = (f.astype(np.uint64)[:, None, None] * np.uint64(1 << 20) +
           np.arange(n_rows, dtype=np.uint64)[None, :, None] * np.uint64(1 << 12) +
           np.arange(n_channels, dtype=np.uint64)[None, None, :])
    h = _mix64(idx ^ _mix64(np.full(1, seed, dtype=np.uint64)))
    uni = (h >> np.uint64(40)).astype(f32) * f32(1.0 / 16777216.0)
    out = out + f32(noise) * (uni - f32(0.5))
    return out.astype(f32)


def sha256(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
