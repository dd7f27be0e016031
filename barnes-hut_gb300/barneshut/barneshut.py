"""Config-driven facade (python-bh/barneshut/barneshut.py:4-32).

``[general] implementation`` selects the step implementation:

* ``gb300``     this project's CUDA step (default semantics: the reference
                CPU path's, i.e. r^2 <= 1e-5 pairs contribute nothing);
* ``singlegpu`` the same CUDA step with the reference GPU path's semantics
                (no cutoff; only coincident points are skipped);
* ``gb300_ctypes`` the C ABI bound directly with ctypes
                (``implementations/gb300_ctypes.py``: the module a python-bh
                maintainer would add to the reference's own package).

The reference's ``sequential``, ``multigpu``, ``parla`` and ``pykokkos``
implementations are not provided: this package has one GPU code path and no
CPU fallback.
"""
from barneshut.internals.config import Config


class BarnesHut:

    def __init__(self, ini_file):
        Config.read_file(ini_file)
        impl = Config.get("general", "implementation", fallback="gb300")
        print(f"Using {impl} implementation")
        if impl in ("gb300", "singlegpu"):
            from .implementations.gb300 import GB300BarnesHut
            self.bh = GB300BarnesHut(reference_gpu_semantics=(impl == "singlegpu"))
        elif impl == "gb300_ctypes":
            from .implementations.gb300_ctypes import CtypesGB300BarnesHut
            self.bh = CtypesGB300BarnesHut()
        else:
            raise ValueError(
                f"implementation {impl!r} is not provided by this package; "
                "use 'gb300' (or 'singlegpu' for the reference GPU path's semantics)")

    def read_input_file(self, file):
        self.bh.read_particles_from_file(file)

    def run(self, *args, **kwargs):
        self.bh.run(*args, **kwargs)
