"""The ctypes binding a python-bh maintainer would add to the reference's own package
(barneshut/implementations/gb300_ctypes.py, INTEGRATION's second route), driven by
BaseBarnesHut.run (the mirror of base.py:94-135) through BarnesHut(ini) with
implementation = gb300_ctypes: ten rounds of the C1 input against the reference's final
positions (golden vectors of python-bh's CPU path), same tolerance as the drop-in test
(positions within 2e-7 of the largest displacement)."""
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


def test_ctypes_binding_ten_rounds(tmp_path):
    from barneshut import BarnesHut
    from barneshut.gb300 import particle_io
    import barneshut.internals.particle as p

    z = np.load(f"{GOLDEN}/ref_c1_uniform10k.npz")
    cp = configparser.ConfigParser()
    cp.read(f"{ROOT}/barnes-hut_gb300/configs/parity_c1.ini")
    cp["general"]["implementation"] = "gb300_ctypes"
    cp["general"]["rounds"] = str(int(z["nsteps"]))
    ini = tmp_path / "c1_ctypes.ini"
    with open(ini, "w") as f:
        cp.write(f)
    inp = tmp_path / "c1.bin"
    particle_io.write_particles(str(inp), z["x0"], z["y0"], z["m"], z["vx0"], z["vy0"])
    bh = BarnesHut(str(ini))
    bh.read_input_file(str(inp))
    bh.run()
    assert bh.bh.grid_dim == int(z["s0_grid_dim"])
    bh.bh.ensure_particles_id_ordered()
    P = bh.bh.get_particles()
    np.testing.assert_array_equal(P[:, p.pid], np.arange(len(z["x0"])))
    disp = max(np.max(np.abs(z["final_x"] - z["x0"])), np.max(np.abs(z["final_y"] - z["y0"])))
    err = max(np.max(np.abs(P[:, p.px] - z["final_x"])), np.max(np.abs(P[:, p.py] - z["final_y"])))
    assert err <= 2e-7 * disp, (err, disp)
