"""Step interface of the reference (python-bh/barneshut/implementations/base.py:34-258).

``BaseBarnesHut.run`` drives the four phases per round exactly as the
reference does (base.py:94-135): create_tree, summarize, evaluation_rounds x
evaluate, timestep (unless skip_timestep), with the same Timer phase names,
and the same ``--check`` accuracy report (base.py:149-205).  The n^2 sample
of that check is computed by the implementation (on the GPU for gb300).
"""
import logging
import random

import numpy as np

import barneshut.internals.particle as p
from barneshut.gb300 import particle_io
from barneshut.internals import Config
from barneshut.kernels.helpers import next_perfect_square
from barneshut.kernels.helpers.grid import get_bounding_box
from timer import Timer

LEAF_OCCUPANCY = 0.7


def reference_grid_dim(n, particles_per_leaf):
    """base.py:223-231: n / (0.7 ppb) leaves rounded up to a perfect square."""
    if particles_per_leaf == 1:
        nleaves = particles_per_leaf
    else:
        nleaves = n / (LEAF_OCCUPANCY * particles_per_leaf)
    nleaves = next_perfect_square(nleaves)
    return int(nleaves ** 0.5)


class BaseBarnesHut:

    def __init__(self):
        self.particles = None
        self.n_particles = None
        self.checking_accuracy = False
        self.sample_size = int(Config.get("general", "sample_check_size"))
        self.particles_per_leaf = int(Config.get("grid", "max_particles_per_box"))
        self.skip_timestep = Config.get("general", "skip_timestep") == "True"
        self.evaluation_rounds = int(Config.get("general", "evaluation_rounds"))
        self.grid_dim = None
        print(f"Skiping timestep? {self.skip_timestep}")

    def read_particles_from_file(self, filename):
        """Binary file of python-bh/bin/gen_input.py: int32 N, N x (x, y, m, vx, vy)."""
        x, y, m, vx, vy = particle_io.read_particles(filename)
        self.set_particles(x, y, m, vx, vy)

    def set_particles(self, x, y, m, vx, vy):
        self.particles = particle_io.records_from_arrays(x, y, m, vx, vy)
        self.n_particles = len(x)

    def set_particles_bounding_box(self):
        """base.py:211-240: the square box around the particles, the grid dimension from the
        particles per leaf, the box edge."""
        bb_min, bb_max = get_bounding_box(self.particles[:, p.px:p.py + 1])
        self.grid_dim = reference_grid_dim(len(self.particles), self.particles_per_leaf)
        self.step = (bb_max[0] - bb_min[0]) / self.grid_dim
        self.min_xy = np.array(bb_min)
        self.max_xy = np.array(bb_max)

    def write_particles_to_file(self, filename):
        """Checkpoint in the input format (resume = read_particles_from_file)."""
        self.ensure_particles_id_ordered()
        P = self.get_particles()
        particle_io.write_particles(filename, P[:, p.px], P[:, p.py], P[:, p.mass],
                                    P[:, p.vx], P[:, p.vy])

    def create_tree(self):
        raise NotImplementedError()

    def summarize(self):
        raise NotImplementedError()

    def evaluate(self):
        raise NotImplementedError()

    def timestep(self):
        raise NotImplementedError()

    def cleanup(self):
        pass

    def run(self, check_accuracy=False):
        n_iterations = int(Config.get("general", "rounds"))
        self.checking_accuracy = check_accuracy
        if self.checking_accuracy:
            sample_indices = self.generate_sample_indices()
        with Timer.get_handle("end-to-end"):
            for _ in range(n_iterations):
                if self.checking_accuracy:
                    nsquared_sample = self.preround_accuracy_check(sample_indices)
                with Timer.get_handle("grid_creation"):
                    self.create_tree()
                with Timer.get_handle("summarization"):
                    self.summarize()
                for _ in range(self.evaluation_rounds):
                    with Timer.get_handle("evaluation"):
                        self.evaluate()
                if not self.skip_timestep:
                    with Timer.get_handle("timestep"):
                        self.timestep()
                if self.checking_accuracy:
                    self.ensure_particles_id_ordered()
                    self.check_accuracy(sample_indices, nsquared_sample)
        self.cleanup()

    def get_particles(self, sample_indices=None):
        raise NotImplementedError()

    def generate_sample_indices(self):
        random.seed(0)
        samples = random.sample(range(self.n_particles), self.sample_size)
        logging.debug(f"acc_check: sample is {samples}")
        return samples

    def nsquared_sample(self, sample_indices):
        """FP64 direct-sum accelerations (ax, ay arrays) of the sampled pids."""
        raise NotImplementedError()

    def preround_accuracy_check(self, sample_indices):
        particles = self.get_particles()
        ax, ay = self.nsquared_sample(sample_indices)
        samples = {}
        for k, si in enumerate(sample_indices):
            rec = np.array(particles[si], dtype=np.float64, copy=True)
            rec[p.ax], rec[p.ay] = ax[k], ay[k]
            samples[float(rec[p.pid])] = rec
        return samples

    def check_accuracy(self, sample_indices, nsquared_sample):
        impl_sample = self.get_particles(sample_indices)
        cum_err = np.zeros(2)
        for i in sample_indices:
            nsq = nsquared_sample[i][p.ax:p.ay + 1]
            aprox = impl_sample[i][p.ax:p.ay + 1]
            assert nsquared_sample[i][p.pid] == impl_sample[i][p.pid]
            cum_err += np.fabs((nsq - aprox) / nsq)
        cum_err /= float(self.sample_size)
        err = ", ".join(str(x) for x in cum_err)
        print(f"avg relative {self.sample_size} points on each axis:\n\t{err}")
        self.last_accuracy = cum_err
