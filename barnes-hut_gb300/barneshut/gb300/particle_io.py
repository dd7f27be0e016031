"""Particle files in the reference's binary format, and checkpoints.

Format (python-bh/bin/gen_input.py:27-33,52 writes it; base.py:47-72 reads
it): a native int32 particle count N, then N records of five float64
(x, y, mass, vx, vy).  Writing the current state in this format is the
checkpoint: reading it back resumes the run (accelerations are recomputed
every step, so nothing else is needed).

Large files are streamed in chunks through a reusable buffer.
"""
import struct

import numpy as np

REC = np.dtype([("x", "<f8"), ("y", "<f8"), ("m", "<f8"), ("vx", "<f8"), ("vy", "<f8")])
CHUNK = 1 << 20


def read_particles(path):
    """Returns (x, y, m, vx, vy) float64 arrays."""
    with open(path, "rb") as f:
        hdr = f.read(4)
        if len(hdr) != 4:
            raise ValueError(f"{path}: missing particle count")
        (n,) = struct.unpack("<i", hdr)
        if n < 0:
            raise ValueError(f"{path}: negative particle count {n}")
        data = np.fromfile(f, dtype=REC, count=n)
    if len(data) != n:
        raise ValueError(f"{path}: expected {n} records, found {len(data)}")
    return tuple(np.ascontiguousarray(data[k]) for k in ("x", "y", "m", "vx", "vy"))


def write_particles(path, x, y, m, vx, vy):
    n = len(x)
    with open(path, "wb") as f:
        f.write(struct.pack("<i", n))
        buf = np.empty(min(n, CHUNK), dtype=REC)
        for s in range(0, n, CHUNK):
            e = min(n, s + CHUNK)
            b = buf[: e - s]
            b["x"], b["y"], b["m"], b["vx"], b["vy"] = x[s:e], y[s:e], m[s:e], vx[s:e], vy[s:e]
            b.tofile(f)


def records_from_arrays(x, y, m, vx, vy):
    """N x 10 float64 reference record (internals/particle.py:3-15), pid = row."""
    n = len(x)
    P = np.zeros((n, 10))
    P[:, 0], P[:, 1], P[:, 2], P[:, 3], P[:, 4] = x, y, m, vx, vy
    P[:, 9] = np.arange(n, dtype=np.float64)
    return P
