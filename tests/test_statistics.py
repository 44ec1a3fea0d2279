"""Epidemic curves against the reference's own CPU path, statistically.

tests/golden/stat_reference.npz holds the daily new infections of 32 runs of
the reference's CPU build (its own RNG, FP32 reduction and 1 - expf ratio;
generated by tests/golden/make_stat_reference.py).  The same population is
run here for 32 Philox seeds, as one batch of 32 replicas: on the CPU oracle
(whose results equal the CUDA path bit for bit) and on the GPU.  Criteria:
for every day the mean daily new infections differ by at most 2 standard
errors of the difference, and a two-sample KS test on the peak day gives
p > 0.05.
"""
import os

import numpy as np
import pytest

from oracle import binding as ob
from pansim_gb300 import snapshot as snp
from tests.golden.make_stat_reference import CONFIG, population

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def reference_curves():
    return np.load(os.path.join(HERE, "stat_reference.npz"))["curves"]


def batch():
    n = CONFIG["seeds"]
    parts = [population() for _ in range(n)]
    seeds = list(range(n))
    return snp.concat(parts, seeds, [CONFIG["k"]] * n)


def compare(ours, ref):
    """(days within 2 SE, worst z, KS p of the peak day)"""
    from scipy import stats
    m1, m2 = ours.mean(0), ref.mean(0)
    se = np.sqrt(ours.var(0, ddof=1) / len(ours) + ref.var(0, ddof=1) / len(ref))
    z = np.abs(m1 - m2) / np.maximum(se, 1e-12)
    p = stats.ks_2samp(ours.argmax(1), ref.argmax(1)).pvalue
    return z, p


def run(sim_factory):
    snap = batch()
    sim = sim_factory(snap)
    days = CONFIG["days"]
    out = np.zeros((CONFIG["seeds"], days), np.int64)
    sim.run_day(0)
    for d in range(1, days + 1):
        st = sim.run_day(d)
        out[:, d - 1] = [st[r].new_infections for r in range(CONFIG["seeds"])]
    return out


def check(ours):
    ref = reference_curves()
    z, p = compare(ours, ref)
    assert (z <= 2.0).all(), ("days beyond 2 SE", np.nonzero(z > 2.0)[0].tolist(), z.max())
    assert p > 0.05, p


def test_oracle_curves_match_reference_statistically():
    check(run(ob.Oracle))


@pytest.mark.gpu
def test_gpu_curves_match_reference_statistically(gpu_lib):
    from pansim_gb300.native import GpuSim
    check(run(GpuSim))
