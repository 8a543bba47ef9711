"""Headless runner: ``python -m tichi_sph_gb300 -c <config.json> -s <scenario.json>``.

Replays the reference's headless loop (``main.py:417-421``): frames at
``gui_fps`` until ``--until`` seconds of simulated time (the reference: 60),
writing per-frame output with ``--write``.  ``--fbm`` enables the
volume-fraction update block that the reference ships disabled.
"""
import argparse
import sys

from . import sph_config
from .simulation import Simulation


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    ap = argparse.ArgumentParser(prog="tichi_sph_gb300")
    ap.add_argument("-c", "--configFile", required=True)
    ap.add_argument("-s", "--scenarioFile", "--secnarioFile", required=True)
    ap.add_argument("--until", type=float, default=60.0)
    ap.add_argument("--write", action="store_true")
    ap.add_argument("--fbm", action="store_true")
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    cfg = sph_config.load(a.configFile, a.scenarioFile)
    sim = Simulation(cfg, fbm=a.fbm, out_dir=a.out)
    sim.init_scenario()
    print("fluid particle count: ", sim.fluid.part_num[None])
    print("bound particle count: ", sim.bound.part_num[None])
    try:
        while sim.globalvar.time_count < a.until:
            sim.run_step(verbose=True)
            if a.write:
                sim.write_files(wait=False)  # files written in the background while stepping on
    finally:
        sim.flush()  # the frames submitted so far reach the disk even if a step raised
    return 0


if __name__ == "__main__":
    sys.exit(main())
