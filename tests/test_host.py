"""Host-side logic: config facade, grid helpers, particle files, workloads."""
import os

import numpy as np
import pytest

from barneshut.gb300 import particle_io, workloads
from barneshut.kernels.helpers import get_bounding_box, next_perfect_square


def test_next_perfect_square():
    assert next_perfect_square(256) == 256
    assert next_perfect_square(238.1) == 256
    assert next_perfect_square(0.05) == 1
    assert next_perfect_square(357.14) == 361


def test_bounding_box_is_square():
    pts = np.array([[0.0, 0.0], [2.0, 1.0], [1.0, 0.5]])
    (a, b), (c, d) = get_bounding_box(pts)
    assert (a, b, c, d) == (0.0, 0.0, 2.0, 2.0)


def test_particle_file_roundtrip(tmp_path):
    data = workloads.gen_input(12345, "normal", seed=1)
    f = tmp_path / "p.bin"
    particle_io.write_particles(str(f), *data)
    assert os.path.getsize(f) == 4 + 12345 * 40
    back = particle_io.read_particles(str(f))
    for a, b in zip(data, back):
        np.testing.assert_array_equal(a, b)


def test_particle_file_matches_reference_layout(tmp_path):
    import struct

    f = tmp_path / "p.bin"
    particle_io.write_particles(str(f), np.array([1.5]), np.array([2.5]), np.array([3.0]),
                                np.array([-1.0]), np.array([0.25]))
    raw = open(f, "rb").read()
    assert struct.unpack("i", raw[:4])[0] == 1
    assert struct.unpack("ddddd", raw[4:]) == (1.5, 2.5, 3.0, -1.0, 0.25)


def test_truncated_file_rejected(tmp_path):
    f = tmp_path / "bad.bin"
    with open(f, "wb") as fh:
        fh.write((10).to_bytes(4, "little") + b"\0" * 40)
    with pytest.raises(ValueError):
        particle_io.read_particles(str(f))


def test_workloads_deterministic():
    a = workloads.cluster_mixture(10000, seed=2)
    b = workloads.cluster_mixture(10000, seed=2)
    for u, v in zip(a, b):
        np.testing.assert_array_equal(u, v)
    x, y = a[0], a[1]
    assert x.min() >= 0 and x.max() <= 1 - 2 ** -24 and y.max() <= 1 - 2 ** -24
    systems, grids = workloads.batched_systems(16, seed=4)
    assert len(systems) == 16 and all(1024 <= len(s[0]) <= 262144 for s in systems)
    assert all(g == max(1, round((len(s[0]) / 64) ** 0.5)) for s, g in zip(systems, grids))


def test_config_facade_rejects_cpu_impls(tmp_path):
    from barneshut import BarnesHut

    ini = tmp_path / "c.ini"
    ini.write_text("[general]\nimplementation = sequential\n")
    with pytest.raises(ValueError, match="not provided"):
        BarnesHut(str(ini))


def test_timer_median():
    from timer import Timer

    Timer.reset()
    Timer.verbose = False
    for v in (3.0, 1.0, 2.0):
        Timer._report_time("evaluation", v)
    assert Timer.medians()["evaluation"] == 2.0
    Timer.reset()
    Timer.verbose = True
