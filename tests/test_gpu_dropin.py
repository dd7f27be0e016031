"""The drop-in path end to end, as the reference's own entry points drive it
(run_2d.py: BarnesHut(ini), read_input_file, run; base.py:94-135): the C1 input
written as a particle file, ten rounds through the GB300 implementation, final
positions against the reference's (golden vectors of python-bh's CPU path), the
--check sampler, and a checkpoint after five rounds resumed by a fresh instance
for the other five.

Tolerance as the direct plan test: positions within 2e-7 of the largest
displacement (FP32 forces, ~1e-7 relative)."""
import configparser

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _ini(tmp_path, rounds, skip_timestep=False):
    cp = configparser.ConfigParser()
    cp.read(f"{ROOT}/barnes-hut_gb300/configs/parity_c1.ini")
    cp["general"]["rounds"] = str(rounds)
    cp["general"]["skip_timestep"] = str(skip_timestep)
    path = tmp_path / f"c1_{rounds}_{skip_timestep}.ini"
    with open(path, "w") as f:
        cp.write(f)
    return str(path)


def _final_positions(bh):
    import barneshut.internals.particle as p

    bh.bh.ensure_particles_id_ordered()
    P = bh.bh.get_particles()
    return P[:, p.px], P[:, p.py]


def _check_against_reference(z, x, y):
    disp = max(np.max(np.abs(z["final_x"] - z["x0"])), np.max(np.abs(z["final_y"] - z["y0"])))
    dx = np.max(np.abs(x - z["final_x"]))
    dy = np.max(np.abs(y - z["final_y"]))
    assert max(dx, dy) <= 2e-7 * disp, (dx, dy, disp)


def test_dropin_ten_rounds(tmp_path):
    from barneshut import BarnesHut
    from barneshut.gb300 import particle_io

    z = np.load(f"{GOLDEN}/ref_c1_uniform10k.npz")
    assert int(z["nsteps"]) == 10
    inp = tmp_path / "c1.bin"
    particle_io.write_particles(str(inp), z["x0"], z["y0"], z["m"], z["vx0"], z["vy0"])
    bh = BarnesHut(_ini(tmp_path, 10))
    bh.read_input_file(str(inp))
    bh.run()
    assert bh.bh.grid_dim == int(z["s0_grid_dim"])
    _check_against_reference(z, *_final_positions(bh))


def test_dropin_check_sampler(tmp_path):
    """--check compares a round's accelerations with a seeded FP64 direct-sum sample
    (base.py:16-32,149-205); the tick zeroes the accelerations (gpu/grid.py:159-174), so the
    check is run, as on the reference CPU path whose tick never runs, without the timestep."""
    from barneshut import BarnesHut
    from barneshut.gb300 import particle_io

    z = np.load(f"{GOLDEN}/ref_c1_uniform10k.npz")
    inp = tmp_path / "c1.bin"
    particle_io.write_particles(str(inp), z["x0"], z["y0"], z["m"], z["vx0"], z["vy0"])
    bh = BarnesHut(_ini(tmp_path, 1, skip_timestep=True))
    bh.read_input_file(str(inp))
    bh.run(check_accuracy=True)
    # mean relative error per axis over the sample, against the direct sum with the same cutoff
    acc = bh.bh.last_accuracy
    assert np.all(np.isfinite(acc)) and np.all(acc < 0.05), acc


def test_dropin_checkpoint_resume(tmp_path):
    from barneshut import BarnesHut
    from barneshut.gb300 import particle_io

    z = np.load(f"{GOLDEN}/ref_c1_uniform10k.npz")
    inp, ckpt = tmp_path / "c1.bin", tmp_path / "c1_round5.bin"
    particle_io.write_particles(str(inp), z["x0"], z["y0"], z["m"], z["vx0"], z["vy0"])
    ini = _ini(tmp_path, 5)
    first = BarnesHut(ini)
    first.read_input_file(str(inp))
    first.run()
    first.bh.write_particles_to_file(str(ckpt))
    second = BarnesHut(ini)
    second.read_input_file(str(ckpt))
    second.run()
    _check_against_reference(z, *_final_positions(second))


def test_cli_run_2d(tmp_path):
    """bin/run_2d.py with the reference's arguments (run_2d.py:28-61): one warm-up run, one
    timed run with --check; the Timer report names the reference's phases."""
    import subprocess
    import sys

    from barneshut.gb300 import particle_io

    z = np.load(f"{GOLDEN}/ref_c1_uniform10k.npz")
    inp = tmp_path / "c1.bin"
    particle_io.write_particles(str(inp), z["x0"], z["y0"], z["m"], z["vx0"], z["vy0"])
    cmd = [sys.executable, f"{ROOT}/barnes-hut_gb300/bin/run_2d.py", str(inp), "1", "1",
           _ini(tmp_path, 2, skip_timestep=True), "--check", "--sleep", "0"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "avg relative" in r.stdout and "warmup done" in r.stdout
    for phase in ("grid_creation", "summarization", "evaluation", "end-to-end"):
        assert phase in r.stdout, (phase, r.stdout[-2000:])
