"""Closure rules (RuleClosure, closurePolicies.h:48-479).

CPU: the oracle restatement's header split, hysteresis and schedule edits.
GPU: the library's engine against the oracle restatement over several days,
bit for bit (statistics rows, rule state, parameters, schedule table, agent
and location state).
"""
import numpy as np
import pytest

from oracle import binding as ob
from oracle import closures as oc
from pansim_gb300 import closures, synth
from tests.helpers import diff_state, small_snapshot, stats_rows

HOME, WORK, SCHOOL, SHOP = synth.HOME, synth.WORK, synth.SCHOOL, synth.SHOP

SCHEDULED = [
    dict(name="schools", conditionType="afterDays", threshold=1, threshold2=1, openAfter=2, closeAfter=-1,
         parameter=0, locationTypesToClose=[SCHOOL]),
    dict(name="Masks", conditionType="afterDays", threshold=0, threshold2=0, openAfter=3, closeAfter=-1,
         parameter=0.8, locationTypesToClose=[]),
    dict(name="Curfew", conditionType="afterDays", threshold=1, threshold2=1, openAfter=2, closeAfter=-1,
         parameter="2000-0500", locationTypesToClose=[]),
    dict(name="SchoolAgeRestriction", conditionType="afterDays", threshold=2, threshold2=2, openAfter=2,
         closeAfter=-1, parameter=14, locationTypesToClose=[]),
    dict(name="HolidayMode", conditionType="afterDays", threshold=3, threshold2=3, openAfter=1, closeAfter=-1,
         parameter=1.0, locationTypesToClose=[]),
    dict(name="ReduceMovement", conditionType="afterDays", threshold=1, threshold2=1, openAfter=2, closeAfter=-1,
         parameter=0.3, locationTypesToClose=[]),
    dict(name="TestingProb", conditionType="afterDays", threshold=2, threshold2=2, openAfter=5, closeAfter=-1,
         parameter="0.01,0.05,0.01,0.01,0.02", locationTypesToClose=[]),
    dict(name="QuarantinePolicy", conditionType="afterDays", threshold=1, threshold2=1, openAfter=9, closeAfter=-1,
         parameter=2, locationTypesToClose=[]),
]

TRIGGERED = [
    dict(name="work", conditionType="newCasesFraction", threshold=0.002, threshold2=0.001, openAfter=2,
         closeAfter=1, parameter=0, locationTypesToClose=[WORK]),
    dict(name="shops", conditionType="hospitalizedFraction", threshold=0.0005, threshold2=0.0002, openAfter=2,
         closeAfter=2, parameter=0, locationTypesToClose=[SHOP]),
    dict(name="LockdownNonvacc", conditionType="newDeadFraction", threshold=0.0, threshold2=0.0, openAfter=1,
         closeAfter=1, parameter=0, locationTypesToClose=[]),
    dict(name="QuarantineImmune", conditionType="newCasesFraction", threshold=0.001, threshold2=0.0005,
         openAfter=3, closeAfter=2, parameter=0, locationTypesToClose=[]),
]


def header(dead_name="D1"):
    names = [dead_name if n == "D" else n for n in synth.STATE_NAMES]
    return closures.stats_header(names)


def test_split_header_follows_stream_extraction():
    assert oc.split_header("S\tE\tI1\t") == ["S", "E", "I1"]
    # a space before a tab joins the tokens (operator>> skips both)
    assert oc.split_header("ab \tcd\tef") == ["abcd", "ef"]
    assert oc.split_header("a\t\tb") == ["a", "b"]
    h = oc.split_header(header())
    assert h[6] == "I5_h" and h[9] == "D1" and h[10] == "H"


def test_hysteresis_close_and_open():
    c = oc._Cond(dict(threshold=0.5, threshold2=0.2, closeAfter=2, openAfter=3), "hospitalizedFraction")
    seq = [0.6, 0.7, 0.1, 0.1, 0.1, 0.1]
    got = []
    for v in seq:
        c.active = c._hyst(v)
        got.append(c.active)
    # closes once two values in a row were above, opens after three below
    assert got == [False, True, True, True, False, False]


def test_rule_array_and_validation():
    arr = closures.rule_array(SCHEDULED)
    assert len(arr) == len(SCHEDULED) and arr[2].parameter == b"2000-0500"
    with pytest.raises(ValueError):
        closures.rule_array([dict(name="x", conditionType="afterDays", locationTypesToClose=list(range(11)))])


def test_stay_home_roundtrip_on_oracle():
    snap = small_snapshot(n=2000, locs=400)
    o = ob.Oracle(snap)
    eng = oc.OracleClosures(o, [], header())
    before = {k: snap.model[k].copy() for k in ["event_offset", "ev_loc_type", "ev_chance"]}
    eng._stay_home(0.3, set_=True)
    n_set = len(snap.model["ev_loc_type"])
    assert n_set >= len(before["ev_loc_type"])
    home = snap.model["ev_loc_type"] == synth.HOME
    assert home.any()
    eng._stay_home(0.3, set_=False)
    # windows without a home event got one with chance p; undoing it leaves
    # chance 0 (erased where below 1e-10) and restores the other chances
    assert len(snap.model["ev_loc_type"]) <= n_set
    o.close()


def _run_pair(snap, rules, days, hdr, enable=True):
    from pansim_gb300.native import GpuSim
    s_cpu, s_gpu = snap, snap.copy()
    o = ob.Oracle(s_cpu)
    g = GpuSim(s_gpu)
    eng = oc.OracleClosures(o, rules, hdr, enable)
    g.closures_init(rules, hdr, enable)
    seen_closed = set()
    for d in range(days):
        st_o = oc.run_day(o, eng, d)
        st_g = g.run_day(d)
        assert stats_rows(st_o) == stats_rows(st_g), d
        act_o, open_o = eng.status()
        act_g, open_g = g.closures_status()
        assert np.array_equal(act_o, act_g) and np.array_equal(open_o, open_g), d
        seen_closed.update(i for i in range(len(act_o)) if act_o[i])
        p = g.get_params()
        for k in ["enable_curfew", "curfew_begin", "curfew_end", "school_age_restriction", "holiday_mode",
                  "quarantine_policy", "quarantine_immune", "lockdown_nonvacc"]:
            assert getattr(p, k) == int(s_cpu.params.get(k, 0)), (d, k)
        for k in ["t_random", "t_home", "t_work", "t_school", "t_hospital"]:
            assert getattr(p, k) == float(s_cpu.params.get(k, 0.0)), (d, k)
        ev = g.get_events()
        for k in ev:
            assert np.array_equal(ev[k], s_cpu.model[k]), (d, k)
    g.download()
    assert diff_state(s_cpu, s_gpu) == []
    o.close()
    g.close()
    return seen_closed


@pytest.mark.gpu
def test_scheduled_rules_bit_exact(gpu_lib):
    snap = small_snapshot(n=12000, locs=3000, initial_infected_frac=0.02, testing=True)
    seen = _run_pair(snap, SCHEDULED, 6, header())
    assert len(seen) == len(SCHEDULED)


@pytest.mark.gpu
def test_triggered_rules_bit_exact(gpu_lib):
    snap = small_snapshot(n=12000, locs=3000, initial_infected_frac=0.03, quarantine_policy=3, testing=True)
    seen = _run_pair(snap, TRIGGERED, 8, header())
    assert 0 in seen  # the newCasesFraction rule fired


@pytest.mark.gpu
def test_expose_to_mutation_bit_exact(gpu_lib):
    snap = small_snapshot(n=10000, locs=2500, initial_infected_frac=0.01, n_variants=2)
    rules = [dict(name="ExposeToMutation", conditionType="afterDays", threshold=1, threshold2=1, openAfter=2,
                  closeAfter=-1, parameter=2e-3, locationTypesToClose=[])]
    _run_pair(snap, rules, 4, header())
    assert (snap.agents["st_variant_mask"] & 2).any()


@pytest.mark.gpu
def test_disabled_closures_keep_only_switches(gpu_lib):
    snap = small_snapshot(n=8000, locs=2000, initial_infected_frac=0.02)
    _run_pair(snap, SCHEDULED, 3, header(), enable=False)
