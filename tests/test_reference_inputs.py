"""The reference's input files as a Snapshot (pansim_gb300.reference_inputs).

CPU: the parsing rules the reference applies (H.MM times, day types, WB
states, the progression index over unsigned age intervals, the classroom
offsets), the reference's own example inputs when the reference tree is
present (counts, the cemetery, three days on the oracle with seeded
infections), and a small city written in the reference's formats by this
test, round-tripped through the binary snapshot.

GPU: that small city against the oracle, bit for bit.
"""
import json
import os

import numpy as np
import pytest

from oracle import binding as ob
from pansim_gb300 import reference_inputs as ri
from pansim_gb300 import snapshot as sn
from tests.helpers import diff_state, stats_rows

# the reference tree, where present (its example inputs); the same variable
# the reference build recipe reads
REF = os.environ.get("PANSIM_REFERENCE", os.path.join(os.sep, "root", "reference"))


def test_time_day_notation():
    # TimeDay(double): hours in an unsigned char, minutes from the fraction / 0.6
    assert ri.time_minutes(8.3) == 8 * 60 + 30
    assert ri.time_minutes(8.30) == 510 and ri.time_minutes(17.45) == 17 * 60 + 45
    assert ri.time_minutes(24.0) == 1440 and ri.time_minutes(0.1) == 10
    assert ri.time_minutes(-1) == 255 * 60


def test_days_and_wb_states():
    assert ri.parse_days("weekdays") == [0, 1, 2, 3, 4] and ri.parse_days("ALL") == list(range(7))
    assert ri.parse_days("Sunday") == [6] and ri.parse_days("WEEKENDS") == [5, 6]
    assert ri.parse_wb("w") == 0 and ri.parse_wb("D") == 4
    with pytest.raises(ri.InputError):
        ri.parse_days("someday")
    with pytest.raises(ri.InputError):
        ri.parse_wb("WN")


def test_progression_index_with_open_age_interval():
    """Ages are unsigned: [80, -1] is the last interval; index = age interval
    x number of pre-conditions + pre-condition (readProgressionMatrices)."""
    cfg = {"transitionMatrices": [{"fileName": "a", "age": [80, -1], "preCond": "0"},
                                  {"fileName": "b", "age": [0, 79], "preCond": "1"},
                                  {"fileName": "c", "age": [0, 79], "preCond": "0"},
                                  {"fileName": "d", "age": [80, -1], "preCond": "1"}]}
    params = {"preCondition": [{"ID": "0"}, {"ID": "1"}]}
    index, files = ri.progression_index(cfg, params)
    assert index == {(0, 79, "0"): 0, (0, 79, "1"): 1, (80, 2**32 - 1, "0"): 2, (80, 2**32 - 1, "1"): 3}
    assert [f["fileName"] for f in files] == ["c", "b", "a", "d"]


def tiny_city(n_homes=60, seed=3):
    """Documents in the reference's formats (include/IO/inputFormats/*.h):
    homes of 1-4 agents, two work places, a school with two classrooms, a
    shop (public space), a hospital (also the doctor)."""
    rng = np.random.default_rng(seed)
    lt = {"publicSpace": 5, "home": 2, "hospital": 12, "doctor": 12, "school": 3, "classroom": 33, "work": 4,
          "nurseryhome": 22, "types": [{"ID": i, "name": "t%d" % i} for i in (2, 3, 4, 5, 12, 22, 33, 44)]}
    places = [{"ID": "h%d" % j, "type": 2, "essential": 0, "coordinates": [0, 0], "infectious": 1.0,
               "area": 1, "state": "ON", "capacity": 10, "ageInter": [0, 100]} for j in range(n_homes)]
    extra = [("w0", 4), ("w1", 4), ("s0", 3), ("c0_s0", 33), ("c1_s0", 33), ("shop", 5), ("hosp", 12)]
    for pid, t in extra:
        places.append({"ID": pid, "type": t, "essential": 1 if t == 12 else 0, "coordinates": [0, 0],
                       "infectious": 0.8 if t != 2 else 1.0, "area": 1, "state": "ON", "capacity": 100,
                       "ageInter": [0, 100]})
    ev = lambda t, ch, st, en, du: {"type": t, "chance": ch, "start": st, "end": en, "duration": du}
    sched = lambda *events: [{"WB": "w", "dayType": "ALL", "schedule": list(events)},
                             {"WB": "n", "dayType": "ALL", "schedule": list(events)},
                             {"WB": "m", "dayType": "ALL", "schedule": [ev(2, 1.0, 0.0, 24.0, -1)]},
                             {"WB": "s", "dayType": "ALL", "schedule": [ev(12, 1.0, 0.0, 24.0, -1)]}]
    at = {"types": [
        {"name": "worker", "ID": 1, "schedulesUnique": sched(ev(4, 1.0, 8.0, 8.10, 8.0), ev(5, 0.5, 17.0, 17.10, 1.3),
                                                             ev(2, 0.5, 17.0, 17.10, 2.0))},
        {"name": "child", "ID": 2, "schedulesUnique": sched(ev(33, 1.0, 8.0, 8.10, 6.0), ev(2, 1.0, 15.0, 15.10, -1))},
        {"name": "retiree", "ID": 3, "schedulesUnique": sched(ev(5, 0.6, 10.0, 10.10, 2.3), ev(2, 0.4, 10.0, 10.10, 3.0))},
    ]}
    people = []
    for j in range(n_homes):
        for _ in range(1 + rng.integers(0, 4)):
            t = int(rng.choice([1, 2, 3], p=[0.5, 0.3, 0.2]))
            age = {1: rng.integers(20, 60), 2: rng.integers(6, 17), 3: rng.integers(65, 90)}[t]
            locs = [{"typeID": 2, "locID": "h%d" % j}, {"typeID": 5, "locID": "shop"}, {"typeID": 12, "locID": "hosp"}]
            if t == 1:
                locs.append({"typeID": 4, "locID": "w%d" % rng.integers(0, 2)})
            if t == 2:
                locs += [{"typeID": 3, "locID": "s0"}, {"typeID": 33, "locID": "c%d_s0" % rng.integers(0, 2)}]
            rng.shuffle(locs)
            people.append({"age": int(age), "sex": "MF"[rng.integers(0, 2)], "preCond": str(rng.integers(0, 2)),
                           "state": "I1" if rng.random() < 0.1 else "S", "typeID": t, "locations": locs,
                           "diagnosed": False})
    people.append({"age": 30, "sex": "M", "preCond": "0", "state": "S", "typeID": 9, "locations": [], "diagnosed": False})
    params = {"sex": [{"name": "M", "symptoms": 1.1}, {"name": "F", "symptoms": 0.9}],
              "age": [{"from": 0, "to": 60, "symptoms": 0.8, "transmission": 1}, {"from": 60, "to": -1, "symptoms": 1.3,
                                                                                   "transmission": 1}],
              "preCondition": [{"ID": "0", "condition": "healthy", "symptoms": 1.0},
                               {"ID": "1", "condition": "other", "symptoms": 1.5}]}
    names = ["S", "E", "I1", "I2", "R", "D1", "D2"]
    cfg = {"stateInformation": {"stateNames": names, "firstInfectedState": "E", "nonCOVIDDeadState": "D2",
                                "susceptibleStates": ["S"], "infectedStates": ["E", "I1", "I2"]},
           "states": [{"stateName": n, "WB": w, "infectious": f, "accuracyPCR": 0.9, "accuracyAntigen": 0.7}
                      for n, w, f in zip(names, "WWWMWDD", [0, 0, 0.8, 0.5, 0, 0, 0])],
           "transitionMatrices": []}
    files = {}
    for a, (lo, hi) in enumerate([(0, 59), (60, -1)]):
        for c in ("0", "1"):
            fn = "t%d_%s.json" % (a, c)
            death = 0.05 if a else 0.01
            st = lambda n, avg, mx, prog: {"stateName": n, "avgLength": avg, "maxlength": mx, "progressions": prog}
            p = lambda n, ch, bad=False: {"name": n, "chance": ch, "isBadProgression": bad}
            files[fn] = {"states": [
                st("S", [-1], [-1], []), st("E", [1, 1], [3, 3], [p("I1", 1, True)]),
                st("I1", [2], [5], [p("I2", 0.7), p("R", 0.3)]),
                st("I2", [3], [6], [p("R", 1 - death), p("D1", death, True)]),
                st("R", [20], [40], [p("S", 1)]), st("D1", [-1], [-1], []), st("D2", [-1], [-1], [])]}
            cfg["transitionMatrices"].append({"fileName": fn, "age": [lo, hi], "preCond": c})
    cfg["_files"] = files
    return dict(agents={"people": people}, locations={"places": places}, agent_types=at, location_types=lt,
                parameters=params, progression_config=cfg)


def test_tiny_city_converts_as_the_reference_initialises():
    docs = tiny_city()
    s = ri.load(**docs, infectiousness_multiplier=(1.0, 1.5), days_seed=7)
    s.validate()
    n_people = len(docs["agents"]["people"]) - 1  # the tourist (type 9) is dropped
    assert s.n_agents == n_people and s.n_locations == len(docs["locations"]["places"]) + 1
    # the cemetery: the last location, of the largest location type
    assert s.params["cemetery_loc"] == s.n_locations - 1 and s.locs["type"][-1] == 44
    # progression = age interval x pre-condition; days drawn only for dwelling states
    a = s.agents
    for i, p in enumerate(docs["agents"]["people"][:n_people]):
        assert a["prog_id"][i] == (0 if p["age"] <= 59 else 1) * 2 + int(p["preCond"])
        assert (a["days"][i] == -1) == (p["state"] == "S")
        sym = np.float32(np.float32(np.float32(1.0) * np.float32(1.1 if p["sex"] == "M" else 0.9)) *
                         np.float32(0.8 if p["age"] < 60 else 1.3))
        assert a["symptom_scaling"][i] == np.float32(sym * np.float32(1.5 if p["preCond"] == "1" else 1.0))
        home = [q["locID"] for q in p["locations"] if q["typeID"] == 2][0]
        assert a["location"][i] == int(home[1:])
        types = a["poss_type"][a["loc_offset"][i]:a["loc_offset"][i + 1]]
        assert list(types) == sorted(types)
    infected = a["state"] == 2
    assert (a["infectious"][infected] == np.float32(0.8)).all() and (a["st_infected_ts"][infected] == 0).all()
    assert (a["st_infected_count"][infected] == 1).all() and (a["st_worst_state"][infected] == 2).all()
    # bad transitions before neutral ones; terminal states loop on themselves
    m = s.model
    S = m["n_states"]
    r = 1 * S + 3  # progression 1, state I2
    assert m["tr_bad_count"][r] == 1 and m["tr_next"][m["tr_bad_begin"][r]] == 5
    assert m["tr_neu_count"][r] == 1 and m["tr_next"][m["tr_neu_begin"][r]] == 4
    r = 2 * S + 6  # D2
    assert m["tr_neu_count"][r] == 1 and m["tr_next"][m["tr_neu_begin"][r]] == 6 and m["tr_chance"][m["tr_neu_begin"][r]] == 1
    # lengths: E gives two variants, the others one, copied to all
    o = (0 * S + 1) * 7
    assert list(m["len_avg"][o:o + 7]) == [1.0] * 7 and list(m["len_max"][o:o + 7]) == [3.0] * 7
    # schedules: worker, weekday W: work 08:00-08:10 for 8 h
    off = m["event_offset"]
    b = off[0 * 28 + 7 * 0 + 0]
    assert m["ev_loc_type"][b] == 4 and m["ev_start"][b] == 480 and m["ev_end"][b] == 490 and m["ev_duration"][b] == 480
    # schools and classrooms (classroom "c<k>_<school ID>")
    assert list(s.locs["schools"]) == [62] and sorted(s.locs["classrooms"]) == [63, 64]
    assert list(s.locs["classroom_offsets"]) == [0, 2]


def test_tiny_city_snapshot_round_trip_and_oracle(tmp_path):
    s = ri.load(**tiny_city(), days_seed=7)
    sn.save(s, str(tmp_path / "city.npz"))
    s2 = sn.load(str(tmp_path / "city.npz"))
    for k in s.agents:
        assert np.array_equal(s.agents[k], s2.agents[k]), k
    o = ob.Oracle(s2)
    for d in range(3):
        o.run_day(d)
    assert (s2.agents["state"] != s.agents["state"]).any()


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "inputRealExample")), reason="reference tree absent")
def test_reference_example_inputs(tmp_path):
    """The reference's own example (22,364 agents of which 5,999 tourists,
    8,165 locations) with its default configuration files."""
    import tarfile
    for f in ("agents.tar", "locations.tar"):
        with tarfile.open(os.path.join(REF, "inputRealExample", f)) as t:
            t.extractall(tmp_path, filter="data")
    cfg = os.path.join(REF, "inputConfigFiles")
    agents = json.load(open(tmp_path / "agents.json"))
    # seed infections: every 50th agent starts in I1
    for i, p in enumerate(agents["people"]):
        if i % 50 == 0:
            p["state"] = "I1"
    s = ri.load(agents, str(tmp_path / "locations.json"), os.path.join(cfg, "agentTypes.json"),
                os.path.join(cfg, "locationTypes.json"), os.path.join(cfg, "parameters.json"),
                os.path.join(cfg, "progressions", "transition_config.json"))
    s.validate()
    assert s.n_agents == 22364 - 5999 and s.n_locations == 8166
    assert s.model["n_prog"] == 35 and s.model["n_states"] == 12 and s.model["n_agent_types"] == 9
    assert s.model["state_names"][s.model["first_infected_state"]] == "E"
    assert s.model["state_names"][s.model["noncovid_dead_state"]] == "D2"
    assert s.locs["type"][-1] == 44
    o = ob.Oracle(s)
    for d in range(3):
        o.run_day(d)
    assert (s.agents["state"] == 1).any()  # newly exposed agents
    assert (s.agents["location"] != s.agents["location"][0]).any()


@pytest.mark.gpu
def test_tiny_city_gpu_matches_oracle(gpu_lib):
    from pansim_gb300.native import GpuSim
    s_cpu = ri.load(**tiny_city(n_homes=200), days_seed=11)
    s_gpu = s_cpu.copy()
    o = ob.Oracle(s_cpu)
    g = GpuSim(s_gpu)
    for d in range(4):
        assert stats_rows(o.run_day(d)) == stats_rows(g.run_day(d)), d
        g.download()
        assert diff_state(s_cpu, s_gpu) == [], d
