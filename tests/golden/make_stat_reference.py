"""Generates tests/golden/stat_reference.npz: daily new infections of 32
independent runs of the reference's own CPU path (oracle/ref_harness in
native mode: std::mt19937_64 per OpenMP thread with the reference's own
distributions, its FP32 per-location reduction and 1 - expf ratio) on one
seeded population, for the statistical comparison of epidemic curves.
Run where the reference tree is available:
    python tests/golden/make_stat_reference.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import ref_binding as rb  # noqa: E402
from pansim_gb300 import synth  # noqa: E402

# the population and run of the comparison
CONFIG = dict(n_agents=10_000, n_other_locs=2_500, pop_seed=0x5EED0000 + 21, k=1e-3, initial_infected_frac=0.005,
              days=30, seeds=32)


def population(seed=1):
    c = CONFIG
    return synth.make_snapshot(c["n_agents"], c["n_other_locs"], seed=seed, pop_seed=c["pop_seed"], k=c["k"],
                               initial_infected_frac=c["initial_infected_frac"])


def new_infections(snap, t):
    """NI of the statistics row at midnight t (simulation.h:555-562)."""
    ts = snap.agents["st_infected_ts"]
    spd = snap.steps_per_day
    return int(np.sum((ts > t - spd) & (ts <= t) & (snap.agents["st_infected_count"] > 0)))


def main():
    c = CONFIG
    curves = np.zeros((c["seeds"], c["days"]), np.int64)
    for s in range(c["seeds"]):
        snap = population()
        r = rb.RefSim(snap, native=True, native_seed=1000 + s)
        for d in range(c["days"]):
            r.run_day(d)
            r.sync()
            curves[s, d] = new_infections(snap, (d + 1) * snap.steps_per_day)
        r.close()
        print("seed", s, "peak day", int(curves[s].argmax()), "total", int(curves[s].sum()))
    np.savez_compressed(os.path.join(HERE, "stat_reference.npz"), curves=curves,
                        config=np.array(repr(sorted(CONFIG.items()))))


if __name__ == "__main__":
    main()
