#!/usr/bin/env python3
"""Input generator with the interface of python-bh/bin/gen_input.py:15-33:
gen_input.py <distribution> <num_particles> <fout> [--seed S] [--device]
distributions: normal, gauss (as the reference), uniform01, cluster (seeded).
--device draws normal / gauss / cluster on the GPU (bh_generate, Philox4x32-10 counters)
instead of numpy on the host; the file format is the same."""
import argparse
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.realpath(__file__))))

from barneshut.gb300 import particle_io, workloads  # noqa: E402

if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("distribution")
    ap.add_argument("num_particles", type=int)
    ap.add_argument("fout")
    ap.add_argument("--seed", type=int, default=None)
    ap.add_argument("--device", action="store_true", help="generate on the GPU")
    a = ap.parse_args()
    n = a.num_particles
    if a.device:
        from barneshut.gb300 import native

        kinds = {"normal": native.BH_GEN_UNIFORM, "gauss": native.BH_GEN_GAUSS, "cluster": native.BH_GEN_CLUSTER}
        if a.distribution not in kinds:
            sys.exit(f"--device supports {sorted(kinds)}")
        out = native.generate(kinds[a.distribution], n, 0 if a.seed is None else a.seed)
        data = tuple(out[k].cpu().numpy() for k in ("x", "y", "m", "vx", "vy"))
    elif a.distribution in ("normal", "gauss"):
        data = workloads.gen_input(n, a.distribution, seed=a.seed)
    elif a.distribution == "uniform01":
        data = workloads.uniform(n, seed=0 if a.seed is None else a.seed)
    elif a.distribution == "cluster":
        data = workloads.cluster_mixture(n, seed=1 if a.seed is None else a.seed)
    else:
        sys.exit(f"unknown distribution {a.distribution}")
    print(f"Using distribution {a.distribution}")
    particle_io.write_particles(a.fout, *data)
