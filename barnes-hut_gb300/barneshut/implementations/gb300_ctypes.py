"""The C ABI bound directly with ctypes: the one module a python-bh maintainer adds next to
``singlegpu.py`` (as ``implementations/gb300.py``, plus a branch in ``barneshut.py:8-25``) to run
the reference's own ``BaseBarnesHut.run`` (``base.py:94-135``) on this project's kernels.

It uses only what the reference's base class provides (``Config``, ``particles`` as the N x 10
record array, ``particles_per_leaf``, ``set_particles_bounding_box``) and the C entry points of
``include/bh_gb300.h``; torch is the caller's device allocator and stream source.  In this
package it runs as ``implementation = gb300_ctypes`` under the mirrored base class.

Semantics: the reference CPU path's (flat far field, pairs with r^2 <= 1e-5 contribute nothing,
no softening), FP32 pairs with compensated far sums.  The library is ``$BH_GB300_LIB``, else the
in-tree build next to this package.
"""
import ctypes
import os

import torch

from barneshut.internals.config import Config

from .base import BaseBarnesHut

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.environ.get("BH_GB300_LIB", os.path.join(_HERE, "..", "..", "lib", "libbh_gb300.so"))
_L = None


class BhParams(ctypes.Structure):
    """bh_params, field for field (include/bh_gb300.h)."""
    _fields_ = [("grav_constant", ctypes.c_double), ("tick_seconds", ctypes.c_double),
                ("softening", ctypes.c_double), ("cutoff_r2", ctypes.c_double),
                ("theta", ctypes.c_double), ("group_dim", ctypes.c_int),
                ("precision", ctypes.c_int), ("flags", ctypes.c_int), ("tune", ctypes.c_int),
                ("correction_theta", ctypes.c_double), ("dense_min", ctypes.c_int),
                ("quad_min", ctypes.c_int)]


def library():
    """The C library, loaded once, with the argument types of the calls used here."""
    global _L
    if _L is None:
        L = ctypes.CDLL(_LIB_PATH)
        vp = ctypes.c_void_p
        L.bh_plan_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.POINTER(ctypes.c_longlong),
                                     ctypes.POINTER(ctypes.c_int), ctypes.POINTER(BhParams)]
        L.bh_workspace_size.argtypes = [vp, ctypes.POINTER(ctypes.c_size_t)]
        L.bh_bind.argtypes = [vp, vp, ctypes.c_size_t, vp]
        L.bh_load_records.argtypes = [vp, vp, vp]
        L.bh_store_records.argtypes = [vp, vp, vp]
        L.bh_plan_destroy.argtypes = [vp]
        L.bh_last_error.argtypes = [vp]
        L.bh_last_error.restype = ctypes.c_char_p
        for f in ("bh_create_tree", "bh_summarize", "bh_evaluate", "bh_timestep"):
            getattr(L, f).argtypes = [vp, vp]
        _L = L
    return _L


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class CtypesGB300BarnesHut(BaseBarnesHut):
    """create_tree / summarize / evaluate / timestep of singlegpu.py:41-99 as single C calls."""

    def __init__(self):
        super().__init__()
        self.plan = None
        self.ws = None

    def _make_plan(self):
        L = library()
        self.set_particles_bounding_box()  # the grid dimension, as the reference sizes it
        prm = BhParams(float(Config.get("bh", "grav_constant")), float(Config.get("bh", "tick_seconds")),
                       0.0, 1e-5, 0.0, 1, 1, 0, 0, 0.0, 0, 0)
        self.plan = ctypes.c_void_p()
        n = (ctypes.c_longlong * 1)(self.n_particles)
        g = (ctypes.c_int * 1)(self.grid_dim)
        self._ok(L.bh_plan_create(ctypes.byref(self.plan), 1, n, g, ctypes.byref(prm)), "bh_plan_create")
        size = ctypes.c_size_t()
        self._ok(L.bh_workspace_size(self.plan, ctypes.byref(size)), "bh_workspace_size")
        self.ws = torch.empty(size.value + 256, dtype=torch.uint8, device="cuda")
        ptr = self.ws.data_ptr() + (-self.ws.data_ptr()) % 256
        self._ok(L.bh_bind(self.plan, ctypes.c_void_p(ptr), size, _stream()), "bh_bind")
        rec = torch.from_numpy(self.particles).cuda()
        self._ok(L.bh_load_records(self.plan, ctypes.c_void_p(rec.data_ptr()), _stream()), "bh_load_records")
        torch.cuda.synchronize()

    def _ok(self, rc, what):
        if rc:
            msg = library().bh_last_error(self.plan) if self.plan else None
            raise RuntimeError(f"{what}: status {rc}: {msg.decode() if msg else ''}")

    def _call(self, name):
        self._ok(getattr(library(), name)(self.plan, _stream()), name)
        torch.cuda.synchronize()

    def create_tree(self):
        if self.plan is None:
            self._make_plan()
        self._call("bh_create_tree")

    def summarize(self):
        self._call("bh_summarize")

    def evaluate(self):
        self._call("bh_evaluate")

    def timestep(self):
        self._call("bh_timestep")

    def ensure_particles_id_ordered(self):
        if self.plan is None:
            return
        out = torch.empty((self.n_particles, 10), dtype=torch.float64, device="cuda")
        self._ok(library().bh_store_records(self.plan, ctypes.c_void_p(out.data_ptr()), _stream()),
                 "bh_store_records")
        torch.cuda.synchronize()
        self.particles = out.cpu().numpy()

    def get_particles(self, sample_indices=None):
        if sample_indices is None:
            return self.particles
        return {i: self.particles[i].copy() for i in sample_indices}

    def cleanup(self):
        pass

    def __del__(self):
        if self.plan is not None and _L is not None:
            _L.bh_plan_destroy(self.plan)
            self.plan = None
