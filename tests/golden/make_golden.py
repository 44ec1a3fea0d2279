"""Generates the golden fixtures of tests/golden from the reference's own C++.

Each fixture holds an input snapshot and the state after `days` simulated
days computed by oracle/ref_harness (the reference's hot-path sources with
Philox-stream draws), plus the final CSR.  Run where the reference tree is
available:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import ref_binding as rb  # noqa: E402
from pansim_gb300 import snapshot as snp, synth  # noqa: E402
from pansim_gb300.snapshot import AGENT_MUTABLE, LOC_MUTABLE  # noqa: E402

SCENARIOS = {
    "plain": dict(n=3000, locs=750, seed=21, kw=dict(initial_infected_frac=0.03), days=5, params={}),
    "policies": dict(n=3000, locs=750, seed=22, kw=dict(initial_infected_frac=0.03, quarantine_policy=3, testing=True),
                     days=6, params=dict(t_random=0.02, t_home=0.3, t_work=0.1, t_school=0.1, t_hospital=0.2)),
    "curfew_closures": dict(n=3000, locs=750, seed=23, kw=dict(initial_infected_frac=0.04), days=4,
                            params=dict(enable_curfew=1, curfew_begin=120, curfew_end=36, school_age_restriction=10)),
}


def scenario_snapshot(name):
    sc = SCENARIOS[name]
    s = synth.make_snapshot(sc["n"], sc["locs"], seed=sc["seed"], pop_seed=0x5EED0100 + sc["seed"], **sc["kw"])
    s.params.update(sc["params"])
    if name == "curfew_closures":
        rng = np.random.default_rng(sc["seed"])
        s.locs["open"][rng.random(s.n_locations) < 0.25] = 0
    return s


def main():
    for name, sc in SCENARIOS.items():
        s = scenario_snapshot(name)
        snp.save(s, os.path.join(HERE, name + "_input.npz"))
        r = rb.RefSim(s)
        for d in range(sc["days"]):
            r.run_day(d)
        r.sync()
        off, ag = r.csr()
        out = {"days": np.array(sc["days"]), "csr_agents": ag}
        for k in AGENT_MUTABLE:
            out["agents/" + k] = s.agents[k]
        for k in LOC_MUTABLE:
            out["locs/" + k] = s.locs[k]
        np.savez_compressed(os.path.join(HERE, name + "_reference.npz"), **out)
        print(name, "infected ever", int((s.agents["st_infected_count"] > 0).sum()))


if __name__ == "__main__":
    main()
