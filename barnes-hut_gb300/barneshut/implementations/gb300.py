"""GB300 implementation of the step interface.

Replaces python-bh/barneshut/implementations/singlegpu.py (create_tree
:41-67, summarize :69-77, evaluate :79-92, timestep :94-99,
ensure_particles_id_ordered :101-103, get_particles :105-112).  Every phase is
one call into libbh_gb300.so on the current torch CUDA stream; each phase
synchronises before returning, as the reference does, so Timer phases are
wall-clock phase times.

Config keys read (reference keys keep their meaning):
  [bh]    grav_constant, tick_seconds
  [grid]  max_particles_per_box (grid sizing, base.py:211-231)
  [gb300] theta (<= 0: the reference's flat far field), softening,
          cutoff_r2 (default 1e-5 = reference CPU kernels; `singlegpu` uses 0),
          grid_dim (override of the derived G), group_dim, precision
          (fp32 | kahan | fp64), use_graph
"""
import numpy as np

import barneshut.internals.particle as p
from barneshut.gb300 import native
from barneshut.internals import Config

from .base import BaseBarnesHut, reference_grid_dim

_PREC = {"fp32": native.BH_PREC_FP32, "kahan": native.BH_PREC_FP32_KAHAN,
         "fp64": native.BH_PREC_FP64}


def _opt(getter, key, fallback):
    try:
        return getter("gb300", key, fallback=fallback)
    except Exception:
        return fallback


class GB300BarnesHut(BaseBarnesHut):

    def __init__(self, reference_gpu_semantics=False):
        super().__init__()
        import torch

        if not torch.cuda.is_available():
            raise RuntimeError("the gb300 implementation needs a CUDA device (no CPU fallback)")
        native.load_library()
        self._torch = torch
        self.G = Config.getfloat("bh", "grav_constant")
        self.tick = Config.getfloat("bh", "tick_seconds")
        default_cut = 0.0 if reference_gpu_semantics else 1e-5
        self.theta = _opt(Config.getfloat, "theta", 0.0)
        self.softening = _opt(Config.getfloat, "softening", 0.0)
        self.cutoff_r2 = _opt(Config.getfloat, "cutoff_r2", default_cut)
        self.grid_override = _opt(Config.getint, "grid_dim", 0)
        self.group_dim = _opt(Config.getint, "group_dim", 0)
        self.precision = _PREC[_opt(Config.get, "precision", "kahan")]
        self.use_graph = _opt(Config.getboolean, "use_graph", False)
        self.plan = None

    # -------------------------------------------------------------- setup
    def _params(self):
        return native.make_params(self.G, self.tick, self.softening, self.cutoff_r2,
                                  self.theta, self.group_dim, self.precision, 0)

    def _ensure_plan(self):
        if self.plan is not None:
            return
        n = self.n_particles
        G = self.grid_override or reference_grid_dim(n, self.particles_per_leaf)
        self.grid_dim = G
        self.plan = native.Plan([n], [G], self._params())
        self.plan.load_records(self.particles)

    def _sync(self):
        self._torch.cuda.synchronize()

    # -------------------------------------------------------------- phases
    def create_tree(self):
        self._ensure_plan()
        self.plan.create_tree()
        self._sync()

    def summarize(self):
        self.plan.summarize()
        self._sync()

    def evaluate(self):
        self.plan.evaluate()
        self._sync()

    def timestep(self):
        self.plan.timestep()
        self._sync()

    def step(self, nsteps=1):
        """nsteps fused rounds (create_tree, summarize, evaluate + tick)."""
        self._ensure_plan()
        if self.use_graph:
            self.plan.step_graph(nsteps)
        else:
            self.plan.step(nsteps)
        self._sync()

    def check_errors(self):
        return self.plan.error_flags(raise_on_error=True)

    # -------------------------------------------------------------- results
    def ensure_particles_id_ordered(self):
        self._ensure_plan()
        self.particles = self.plan.store_records().cpu().numpy()

    def get_particles(self, sample_indices=None):
        if sample_indices is None:
            return self.particles
        return {i: self.particles[i].copy() for i in sample_indices}

    def nsquared_sample(self, sample_indices):
        self._ensure_plan()
        ax, ay = self.plan.direct_sample(np.asarray(sample_indices, dtype=np.int64))
        return ax.cpu().numpy(), ay.cpu().numpy()

    def diagnostics(self, potential=False):
        self._ensure_plan()
        return self.plan.diagnostics(0, potential)
