"""Immunization (include/immunization.h:24-900).

GPU: the library against the oracle over several days, bit for bit, with
draws that decide (group levels and dose budgets below 1) and with booster
rounds, on agents carrying infection and vaccination histories.  The
oracle itself is pinned against the reference's own Immunization in
tests/test_ref_pin.py.
"""
import numpy as np
import pytest

from oracle import binding as ob
from pansim_gb300 import immunization as im
from tests.helpers import diff_state, small_snapshot, stats_rows

DAY0 = 125  # boosters need day >= 90 and doses older than 120 days


def history_snapshot(n=12000, locs=3000, n_variants=2, seed=3):
    """A population with infection and vaccination histories among its
    susceptible agents, pre-conditions, and a few old diagnoses."""
    snap = small_snapshot(n=n, locs=locs, initial_infected_frac=0.01, n_variants=n_variants)
    rng = np.random.default_rng(seed)
    a = snap.agents
    t0 = DAY0 * snap.steps_per_day
    a["precond"][:] = (rng.random(n) < 0.15) * rng.integers(1, 4, n)
    s = a["state"] == 0
    inf = s & (rng.random(n) < 0.2)
    a["st_infected_count"][inf] = 1
    a["st_infected_ts"][inf] = rng.integers(0, t0, inf.sum())
    a["st_variant_mask"][inf] = rng.integers(1, 1 << n_variants, inf.sum())
    vac = s & (rng.random(n) < 0.35)
    a["st_immunization_count"][vac] = rng.integers(1, 4, vac.sum())
    a["st_immunization_ts"][vac] = rng.integers(1, t0, vac.sum())
    diag = rng.random(n) < 0.05
    a["st_diagnosed_ts"][diag] = rng.integers(0, t0, diag.sum())
    return snap


def random_options(levels="0.9,0.5,0.8,0.7,0.6,0.5,0.4,0.3,0.2,0.1", doses=3000, boosters=2000):
    return im.options(immunizations_per_week=[doses, doses * 2, doses],
                      boosters_per_week=[([boosters, boosters * 3], [0.1, 0.2, 0.3, 0.5, 0.6, 0.7, 0.8, 0.9, 1.0, 1.0]),
                                         ([boosters], [1.0] * 10)],
                      immunizationStart=DAY0 - 3, boosterStart="%d,%d" % (DAY0 - 5, DAY0 + 1),
                      vaccinationGroupLevel=levels, immunizationOrder="1,2,3,4,5,6,0,0,7,8",
                      variantSimilarity="0,1,0,1,1,1,1", variantSimilarMultiplier="0.0,0.5,0,0,0,0,0")


def test_options_pack_reference_defaults():
    p = im.options(immunizations_per_week=7000)
    assert p.daily_doses == 1000 and p.start_after_day == 96 and p.n_booster_rounds == 1
    assert list(p.order) == [1, 2, 3, 4, 5, 6, 0, 0, 7, 8]
    assert abs(p.protection_hospitalization[6] - 0.974) < 1e-6
    with pytest.raises(ValueError):
        im.options(immunizationOrder="1,2,3")


@pytest.mark.gpu
def test_immunization_bit_exact(gpu_lib):
    from pansim_gb300.native import GpuSim
    snap = history_snapshot()
    s_cpu, s_gpu = snap, snap.copy()
    o = ob.Oracle(s_cpu)
    g = GpuSim(s_gpu)
    opt = random_options()
    o.immunization_init(opt)
    g.immunization_init(opt)
    g.download()
    assert np.array_equal(s_cpu.agents["imm_round"], s_gpu.agents["imm_round"])
    assert (s_cpu.agents["imm_round"] == 255).any() and (s_cpu.agents["imm_round"] == 1).any()
    vac_days = 0
    for d in range(DAY0, DAY0 + 5):
        st_o = o.run_day(d)
        st_g = g.run_day(d)
        assert stats_rows(st_o) == stats_rows(st_g), d
        vac_days += stats_rows(st_o)[0][len(s_cpu.model["state_wb"]) + 9] > 0
        g.download()
        assert diff_state(s_cpu, s_gpu) == [], d
    assert vac_days > 0
    # boosters and waning did their work
    assert (s_cpu.agents["st_immunization_count"] >= 2).any()
    assert not np.array_equal(s_cpu.agents["symptom_scaling_v"], np.tile(s_cpu.agents["symptom_scaling"], 2))
    o.close()
    g.close()
