"""The runForDay binding (pyPanSim.SimulatorInterface, matlab/mexPanSim.cpp:57-127,
210-219; Simulation::runForDay / processFlags, simulation.h:779-956).

CPU: the flag table against processFlags' own values, and the uninitialized
call.  GPU: a sequence of days with changing flags against the oracle driven
in runForDay's order, bit for bit (statistics rows, agent and location state).
"""
import numpy as np
import pytest

from oracle import binding as ob
from pansim_gb300.interface import FLAG_CLOSE_TYPES, SimulatorInterface, parse_flags
from tests.helpers import diff_state, small_snapshot


def test_flags_follow_process_flags():
    acts, mask = parse_flags(["TP015"], 10, 1.0)
    assert acts == [("params", dict(t_random=0.00005, t_home=0.2, t_work=0.04, t_school=0.04, t_hospital=0.005,
                                     t_nursery=0.05))]
    acts, _ = parse_flags(["TPdef", "TP035"], 10, 1.0)
    assert acts[0][1]["t_home"] == 0.01 and acts[1][1]["t_home"] == 1.0 and acts[1][1]["t_school"] == 0.2
    # curfew 20:00-05:00 in timesteps of the model
    assert parse_flags(["CF2000-0500"], 10, 1.0)[0] == [("params", dict(enable_curfew=1, curfew_begin=120,
                                                                         curfew_end=30))]
    assert parse_flags(["CF2000-0500"], 15, 1.0)[0][0][1]["curfew_begin"] == 80
    assert parse_flags(["CFNONE"], 10, 1.0)[0] == [("params", dict(enable_curfew=0, curfew_begin=0, curfew_end=0))]
    assert parse_flags(["SONONE", "SO12", "SO3"], 10, 1.0)[0] == [
        ("params", dict(school_age_restriction=v)) for v in (99, 12, 3)]
    assert parse_flags(["QU0", "QU3"], 10, 1.0)[0] == [("params", dict(quarantine_policy=0)),
                                                      ("params", dict(quarantine_policy=3))]
    assert parse_flags(["PL0", "PLNONE"], 10, 1.0)[0] == [("types_open", FLAG_CLOSE_TYPES, False),
                                                         ("types_open", FLAG_CLOSE_TYPES, True)]
    assert FLAG_CLOSE_TYPES == (5, 6, 22, 44)
    # masks: applied once per change of value, undone by division
    acts, mask = parse_flags(["MA0.8", "MA0.8"], 10, 1.0)
    assert acts == [("weights", 0.8, False)] and mask == 0.8
    acts, mask = parse_flags(["MA1.0", "MA1.0"], 10, 0.8)
    assert acts == [("weights", 0.8, True)] and mask == 1.0
    assert parse_flags(["MA1.0"], 10, 1.0) == ([], 1.0)
    # unknown flags and values are ignored
    assert parse_flags(["XX", "TP999", "PL1", "CF2100-0600", "SO5", "QU9", "MA0.5", ""], 10, 1.0) == ([], 1.0)


def test_uninitialized_simulation_returns_empty_rows():
    s = SimulatorInterface()
    assert s.runForDay(["TPdef"]) == []
    assert s.runForDayBatch([]) == []


def _shops_as_type6(snap):
    """Relabels the shop type (7) as 6, one of the types the PL flags switch."""
    for arr in (snap.locs["type"], snap.model["ev_loc_type"], snap.agents["poss_type"]):
        arr[arr == 7] = 6
    snap.params["public_type"] = 6
    return snap


def _oracle_run_for_day(o, day, flags, mask):
    """runForDay on the oracle: the flags' actions on its snapshot, then the
    day in runForDay's order."""
    snap = o.snap
    actions, mask = parse_flags(flags, int(snap.params["time_step"]), mask)
    for act in actions:
        if act[0] == "params":
            snap.params.update(act[1])
            o.set_params()
        elif act[0] == "types_open":
            sel = np.isin(snap.locs["type"].astype(np.int64), np.array(act[1], np.int64)) & (snap.locs["essential"] != 1)
            snap.locs["open"][sel] = 1 if act[2] else 0
        else:
            w = snap.locs["infectiousness"]
            sel = snap.locs["type"] != int(snap.params["home_type"])
            w64 = w[sel].astype(np.float64)
            w[sel] = (w64 / act[1] if act[2] else w64 * act[1]).astype(np.float32)
    spd = snap.steps_per_day
    t = day * spd
    o.stats(t)
    o.plan(t)
    for s in range(spd):
        o.step(t + s)
    if int(snap.params.get("testing_enabled", 0)):
        o.test(t + spd)
    o.progress(t + spd)
    rows = o.stats(t + spd)
    return [[int(x) for x in r.v[: r.n]] for r in rows], mask


@pytest.mark.gpu
def test_run_for_day_with_changing_flags_matches_oracle(gpu_lib):
    snap = _shops_as_type6(small_snapshot(n=12000, locs=3000, initial_infected_frac=0.03, testing=True))
    snap.locs["essential"][snap.locs["type"] == 6] = 0
    s_cpu, s_gpu = snap, snap.copy()
    o = ob.Oracle(s_cpu)
    sim = SimulatorInterface()
    sim.initSimulation(s_gpu)
    days = [["TPdef", "QU2"], ["PL0", "MA0.8", "CF2000-0500"], ["SO12", "TP035", "MA0.8"],
            ["PLNONE", "MA1.0", "CFNONE", "QU3"], []]
    mask = 1.0
    for d, flags in enumerate(days):
        rows_o, mask = _oracle_run_for_day(o, d, flags, mask)
        row_g = sim.runForDay(flags)
        assert row_g == rows_o[0], (d, flags)
        assert sim.mask == mask
        if d == 1:
            # PL0 closed the relabelled shops on both sides
            sim.sim.download()
            assert (s_gpu.locs["open"][s_gpu.locs["type"] == 6] == 0).all()
    sim.sim.download()
    assert diff_state(s_cpu, s_gpu) == []
    o.close()
