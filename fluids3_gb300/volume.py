"""Volume output: SaveBricks (fluids4.0/fluid_system.cpp:1597-1752) over the
sampler (fl_sample_volume, the reference's sampleParticles).

The brick file holds int count, then per accepted brick: int3 brick origin
(in voxels), float3 bmin, float3 bmax, int3 brick size, and size.x*y*z
float32 samples ((z * size.y + y) * size.x + x order). A brick is accepted
when the mean of a 2x2x2 pre-sample over its box exceeds the threshold, as
in SaveBricks. Host byte order.
"""
from __future__ import annotations

import struct

import numpy as np

from .system import FluidSystem


def brick_box(volmin, volmax, res, b, brk):
    """Brick b's box, in the reference's float32 order:
    (volmax - volmin) * (b * brk) / res + volmin."""
    volmin = np.asarray(volmin, np.float32)
    volmax = np.asarray(volmax, np.float32)
    res = np.asarray(res, np.float32)
    b = np.asarray(b, np.int64)
    brk = np.asarray(brk, np.int64)
    lo = (volmax - volmin) * (b * brk).astype(np.float32)
    lo = lo / res + volmin
    hi = (volmax - volmin) * ((b + 1) * brk).astype(np.float32)
    hi = hi / res + volmin
    return lo.astype(np.float32), hi.astype(np.float32)


def save_bricks(system: FluidSystem, path, vol_res=(256, 256, 256), brick=32, thresh: float = 0.0,
                scalar: float = 1.0 / 100.0) -> int:
    """Write the bricks of the system's bounding volume whose pre-sample
    mean exceeds `thresh`; returns the number written. Re-bins and sorts
    the points first, as SaveBricks does."""
    p = system.params
    volmin = np.array(p.bound_min[:], np.float32)
    volmax = np.array(p.bound_max[:], np.float32)
    res = np.array(vol_res, np.int64)
    brk = np.array((brick, brick, brick), np.int64)
    div = res // brk
    first = True
    count = 0
    with open(path, "wb") as f:
        f.write(struct.pack("=i", 0))                       # count, patched at the end
        for by in range(div[1]):
            for bz in range(div[2]):
                for bx in range(div[0]):
                    b = np.array((bx, by, bz), np.int64)
                    lo, hi = brick_box(volmin, volmax, res, b, brk)
                    chk = system.SampleParticles((2, 2, 2), lo, hi, scalar, sort_first=first)
                    first = False
                    s = np.float32(0.0)
                    for v in chk.ravel():
                        s = np.float32(s + v)
                    if np.float32(s / 8.0) <= thresh:
                        continue
                    data = system.SampleParticles(tuple(brk), lo, hi, scalar, sort_first=False)
                    f.write(struct.pack("=3i", *(b * brk).tolist()))
                    f.write(lo.tobytes() + hi.tobytes())
                    f.write(struct.pack("=3i", *brk.tolist()))
                    f.write(np.ascontiguousarray(data, np.float32).tobytes())
                    count += 1
        f.seek(0)
        f.write(struct.pack("=i", count))
    return count


def read_bricks(path) -> list:
    """[(origin int3, bmin, bmax, size int3, data (z, y, x))] of a brick file."""
    raw = open(path, "rb").read()
    (n,) = struct.unpack_from("=i", raw, 0)
    at = 4
    out = []
    for _ in range(n):
        origin = struct.unpack_from("=3i", raw, at); at += 12
        lo = np.frombuffer(raw, np.float32, 3, at); at += 12
        hi = np.frombuffer(raw, np.float32, 3, at); at += 12
        size = struct.unpack_from("=3i", raw, at); at += 12
        k = size[0] * size[1] * size[2]
        data = np.frombuffer(raw, np.float32, k, at).reshape(size[2], size[1], size[0]); at += 4 * k
        out.append((origin, lo, hi, size, data))
    assert at == len(raw), "trailing bytes in brick file"
    return out


__all__ = ["brick_box", "save_bricks", "read_bricks"]
