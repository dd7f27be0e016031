#!/usr/bin/env python3
"""CLI with the arguments of python-bh/bin/run_2d.py:28-61:
run_2d.py <input_file> <nwarmups> <nruns> <configfile> [--debug] [--check]"""
import argparse
import logging
import os
import sys
from time import sleep

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.realpath(__file__))))

from barneshut import BarnesHut  # noqa: E402
from timer import Timer  # noqa: E402

if __name__ == "__main__":
    parser = argparse.ArgumentParser()
    parser.add_argument("input_file", help="Path to input file")
    parser.add_argument("nwarmups", help="How many runs to execute as warmup", type=int)
    parser.add_argument("nruns", help="Number of different runs to execute", type=int)
    parser.add_argument("configfile", help="Path to config file")
    parser.add_argument("--debug", help="Turn debug on", action="store_true")
    parser.add_argument("--check", help="Check accuracy after every round", action="store_true")
    parser.add_argument("--sleep", type=float, default=2.0, help="pause between runs (s)")
    args = parser.parse_args()
    if args.debug:
        logging.basicConfig(level=logging.DEBUG)
    else:
        logging.disable(logging.CRITICAL)
    bh = BarnesHut(args.configfile)
    bh.read_input_file(args.input_file)
    for _ in range(args.nwarmups):
        bh.run(check_accuracy=args.check)
    print("warmup done")
    sleep(args.sleep)
    Timer.reset()
    for _ in range(args.nruns):
        bh.run(check_accuracy=args.check)
        sleep(args.sleep)
    Timer.print()
