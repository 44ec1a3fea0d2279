"""The oracle pinned against the reference's own C++ (CPU).

oracle/ref_harness compiles the reference's hot-path sources (doMovement,
quarantine/plan helpers, DetailedTesting ops, DynamicPPState/MultiBadMatrix,
Util::updatePerLocationAgentLists, TimeDay/AgentTypeList) with an interposed
RandomGenerator drawing from the same Philox streams.  Every agent and
location array must equal the oracle's bit for bit.  Skipped where the
reference tree is absent.
"""
import numpy as np
import pytest

from oracle import binding as ob
from tests.helpers import diff_state, small_snapshot

rb = pytest.importorskip("oracle.ref_binding")
if not rb.ref_build.available():
    pytest.skip("reference tree not available", allow_module_level=True)


def _run_pair(snap, days):
    s_ref = snap.copy()
    o = ob.Oracle(snap)
    r = rb.RefSim(s_ref)
    for d in range(days):
        o.run_day(d)
        r.run_day(d)
        r.sync()
        assert diff_state(snap, s_ref) == [], "day %d" % d
    return o, r, snap, s_ref


def test_schedule_encoding_matches_reference_timeday():
    s = small_snapshot(2000, 500)
    r = rb.RefSim(s.copy())
    st, en, du = r.event_minutes()
    assert np.array_equal(st, s.model["ev_start"])
    assert np.array_equal(en, s.model["ev_end"])
    assert np.array_equal(du, s.model["ev_duration"])


def test_pin_plain_week():
    o, r, a, b = _run_pair(small_snapshot(8000, 2000, seed=5, initial_infected_frac=0.02), 7)
    assert (a.agents["st_infected_count"] > 0).sum() > 100


def test_pin_quarantine_testing():
    s = small_snapshot(8000, 2000, seed=9, initial_infected_frac=0.02, quarantine_policy=3, testing=True)
    s.params.update(t_random=0.02, t_home=0.3, t_work=0.1, t_school=0.1, t_hospital=0.2)
    o, r, a, b = _run_pair(s, 8)
    assert a.agents["quarantined"].sum() > 50
    assert (a.agents["last_test"] != 0xFFFFFFFF).sum() > 100


def test_pin_curfew_closures_school_age():
    s = small_snapshot(6000, 1500, seed=13, initial_infected_frac=0.03)
    s.params.update(enable_curfew=1, curfew_begin=120, curfew_end=36, school_age_restriction=10)
    rng = np.random.default_rng(4)
    s.locs["open"][rng.random(s.n_locations) < 0.25] = 0
    s.locs["closed_until"][rng.random(s.n_locations) < 0.1] = 400
    _run_pair(s, 4)


def test_pin_csr_matches_stable_sort():
    s = small_snapshot(5000, 1200, seed=2)
    s_ref = s.copy()
    o = ob.Oracle(s)
    r = rb.RefSim(s_ref)
    o.midnight(0)
    r.midnight(0)
    for t in range(0, 70):
        o.step(t)
        r.step(t)
    off_o, ag_o = o.csr()
    off_r, ag_r = r.csr()
    assert np.array_equal(ag_o, ag_r)
    # the reference's OpenMP extractOffsets (util.cpp:39-53) leaves the offsets
    # of empty locations below the first occupied one unwritten
    first = int(np.min(s.agents["location"]))
    assert np.array_equal(off_o[first + 1:], off_r[first + 1:])


def _closure_pin(snap, rules, days, header, enable=True):
    """oracle + its closure restatement vs the reference harness + the
    reference's own RuleClosure, fed the same statistics row each midnight."""
    from oracle import closures as oc
    s_ref = snap.copy()
    o = ob.Oracle(snap)
    r = rb.RefSim(s_ref)
    eng = oc.OracleClosures(o, rules, header, enable)
    r.closures_init(rules, header, enable)
    fired = set()
    for d in range(days):
        t0 = d * snap.steps_per_day
        if t0 > 0 and int(snap.params.get("testing_enabled", 0)):
            o.test(t0)
        if t0 > 0:
            o.progress(t0)
        r.midnight_pre(t0)
        row = o.stats(t0)[0]
        eng.midnight(t0, row)
        r.closures_midnight(t0, row)
        a_o, op_o = eng.status()
        a_r, op_r = r.closures_status()
        assert np.array_equal(a_o, a_r) and np.array_equal(op_o, op_r), d
        fired.update(i for i in range(len(a_o)) if a_o[i])
        p = r.params()
        for k in ["enable_curfew", "curfew_begin", "curfew_end", "school_age_restriction", "holiday_mode",
                  "quarantine_policy", "quarantine_immune", "lockdown_nonvacc"]:
            assert getattr(p, k) == int(snap.params.get(k, 0)), (d, k)
        for k in ["t_random", "t_home", "t_work", "t_school", "t_hospital"]:
            assert getattr(p, k) == float(snap.params.get(k, 0.0)), (d, k)
        ev = r.events()
        for k in ev:
            assert np.array_equal(ev[k], snap.model[k]), (d, k)
        o.plan(t0)
        r.plan(t0)
        for s in range(snap.steps_per_day):
            o.step(t0 + s)
            r.step(t0 + s)
        r.sync()
        assert diff_state(snap, s_ref) == [], "day %d" % d
    return fired


def test_pin_closure_rules_scheduled():
    from tests.test_closures import SCHEDULED, header
    snap = small_snapshot(n=6000, locs=1500, initial_infected_frac=0.02, testing=True)
    fired = _closure_pin(snap, SCHEDULED, 6, header())
    assert len(fired) == len(SCHEDULED)


def test_pin_closure_rules_triggered():
    from tests.test_closures import TRIGGERED, header
    # newCasesFraction has no reference counterpart: the reference's init
    # rejects it, and it is checked against the oracle only
    rules = [r for r in TRIGGERED if r["conditionType"] != "newCasesFraction"]
    snap = small_snapshot(n=6000, locs=1500, initial_infected_frac=0.05, quarantine_policy=3, testing=True)
    fired = _closure_pin(snap, rules, 8, header())
    assert fired


def test_reference_rejects_unknown_condition_type():
    from tests.test_closures import TRIGGERED, header
    snap = small_snapshot(n=1000, locs=300)
    r = rb.RefSim(snap)
    with pytest.raises(ValueError):
        r.closures_init([TRIGGERED[0]], header())


def test_pin_closure_rules_disabled_and_expose():
    from tests.test_closures import SCHEDULED, header
    snap = small_snapshot(n=5000, locs=1200, initial_infected_frac=0.01, n_variants=2)
    # fraction * s >= 1 makes every exposure certain, so the reference's
    # single-stream draws inside its for_each cannot change the outcome
    rules = SCHEDULED + [dict(name="ExposeToMutation", conditionType="afterDays", threshold=1, threshold2=1,
                              openAfter=1, closeAfter=-1, parameter=1e6, locationTypesToClose=[])]
    _closure_pin(snap, rules, 3, header(), enable=False)
    assert (snap.agents["st_variant_mask"] & 2).any()


def test_pin_immunization(tmp_path):
    """oracle vs the reference's Immunization (categories, waning, boosters,
    first doses) with group levels of 0 or 1 and budgets that cover every
    eligible agent, so no draw decides anything and the reference's shared
    stream inside its for_each cannot matter."""
    from tests.test_immunization import DAY0, history_snapshot, random_options
    snap = history_snapshot(n=6000, locs=1500)
    s_ref = snap.copy()
    o = ob.Oracle(snap)
    r = rb.RefSim(s_ref)
    opt = random_options(levels="1,0,1,1,0,1,1,0,1,1", doses=7_000_000, boosters=7_000_000)
    o.immunization_init(opt)
    r.immunization_init(opt, tmp_path)
    r.sync()
    assert diff_state(snap, s_ref, fields=["symptom_scaling_v", "st_immunization_ts"]) == []
    doses = 0
    for d in range(DAY0, DAY0 + 4):
        t0 = d * snap.steps_per_day
        o.progress(t0)
        r.midnight_pre(t0)
        n_o = o.immunize(t0)
        n_r = r.immunize(t0)
        assert n_o == n_r, d
        doses += n_o
        o.plan(t0)
        r.plan(t0)
        for s in range(snap.steps_per_day):
            o.step(t0 + s)
            r.step(t0 + s)
        r.sync()
        bad = [k for k in diff_state(snap, s_ref) if not k.startswith("imm_round")]
        assert bad == [], "day %d" % d
    assert doses > 0
    assert (snap.agents["st_immunization_count"] >= 2).any()
    s0 = snap.agents["state"] == 0
    su = snap.agents["susceptible"].reshape(2, -1)
    assert (su[:, s0] < 1.0).any()  # waning protection applied
