"""Shared helpers of the test suite."""
import numpy as np

from pansim_gb300.snapshot import AGENT_MUTABLE, LOC_MUTABLE


def small_snapshot(n=20000, locs=5000, seed=7, **kw):
    from pansim_gb300 import synth
    return synth.make_snapshot(n, locs, seed=seed, pop_seed=0x5EED0000 + 11, **kw)


def diff_state(a, b, fields=None):
    """Names of mutable arrays that differ between two snapshots."""
    out = []
    for k in (fields or AGENT_MUTABLE):
        if not np.array_equal(a.agents[k], b.agents[k]):
            n = int(np.sum(a.agents[k] != b.agents[k]))
            out.append("%s (%d)" % (k, n))
    for k in LOC_MUTABLE:
        if not np.array_equal(a.locs[k], b.locs[k]):
            out.append("loc.%s (%d)" % (k, int(np.sum(a.locs[k] != b.locs[k]))))
    return out


def stats_rows(st):
    return [list(s.v)[: s.n] for s in st]
