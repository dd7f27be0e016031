"""Host-side grid helpers with the semantics of
python-bh/barneshut/kernels/helpers/grid.py:5-26 (grid sizing and the square box; the
device computes the per-step box)."""
import math

import numpy as np


def next_perfect_square(n):
    """Smallest perfect square >= n (n itself when n is one)."""
    r = math.sqrt(n)
    if r == 0 or math.fmod(n, r) != 0:
        c = math.ceil(r)
        return float(c * c)
    return n


def get_bounding_box(points):
    """Square bounding box ((min_x, min_y), (max_x, max_y)): the shorter
    side's maximum is extended so both edges have the same length."""
    pts = np.asarray(points)
    mn = pts.min(axis=0)[:2]
    mx = pts.max(axis=0)[:2]
    min_x, min_y = float(mn[0]), float(mn[1])
    max_x, max_y = float(mx[0]), float(mx[1])
    xe, ye = max_x - min_x, max_y - min_y
    if xe > ye:
        max_y += xe - ye
    elif ye > xe:
        max_x += ye - xe
    assert (max_x - min_x) - (max_y - min_y) < 0.00001
    return (min_x, min_y), (max_x, max_y)

