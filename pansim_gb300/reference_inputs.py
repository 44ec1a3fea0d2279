"""The reference's input files as a Snapshot.

Reads the JSON documents whose formats include/IO/inputFormats/*.h define
(agents, locations, agent types, location types, parameters, the
progression directory and its transition matrices) and builds what the
reference's constructor builds from them (Simulation::Simulation,
include/simulation.h:708-766):

- the state table and the per-(age interval, pre-condition) transition
  matrices and dwell lengths (DynamicPPState::initTransitionMatrix,
  src/agentData/dynamicPPState.cpp:66-140; MultiBadMatrix,
  src/tools/progressionMatrices/multiBadMatrix.cpp:42-80; LengthOfState,
  src/tools/progressionMatrices/basicLengthAbstract.cpp:32-46), with the
  progression index ageIndex * numberOfPreConditions + preConditionIndex
  (DataProvider::readProgressionMatrices, src/IO/dataProviders/dataProvider.cpp:25-57);
- the locations and the cemetery appended last, schools and their
  classrooms (LocationsList::initLocations, include/locationList.h:90-222);
- the schedule table (AgentList::initAgentTypes, include/agentsList.h:94-119;
  AgentTypeList::addSchedule, src/agentData/agentType.cpp:21-27);
- the agents: type, progression, symptom scaling, location list and home,
  state and initial statistics (AgentList::initAgents,
  include/agentsList.h:137-271; BasicAgentMeta, src/agentData/agentMeta.cpp:27-77).

Where the reference leaves a choice open, this reader fixes it:
- An agent's locations are sorted by type with a stable sort.  The
  reference's std::sort leaves the order of same-type entries unspecified.
- The initial dwell times of the agents' states are geometric draws
  (calculateJustDays).  The reference takes them from its per-thread
  generators seeded by std::random_device; here they come from numpy's PCG64
  seeded with `days_seed`.
- An agent whose age no progression interval covers, and an average dwell
  length without a maximum length, are rejected.  The reference reads past
  its map and loops on an undefined bound, respectively.
"""
import json
import os

import numpy as np

from .snapshot import Snapshot
from .synth import MAX_STRAINS, NONE, calculate_modified_p, default_params

WB = {"W": 0, "N": 1, "M": 2, "S": 3, "D": 4}
DAYS = {"ALL": range(7), "WEEKDAYS": range(5), "WEEKENDS": range(5, 7), "MONDAY": [0], "TUESDAY": [1],
        "WEDNESDAY": [2], "THURSDAY": [3], "FRIDAY": [4], "SATURDAY": [5], "SUNDAY": [6]}
FLT_MAX = float(np.finfo(np.float32).max)

# the reference's defaults for --infectiousnessMultiplier, --diseaseProgressionScaling
# and --diseaseProgressionDeathScaling (include/simulation.h:136-147)
DEFAULT_MULTIPLIER = (1.03, 1.79, 2.45, 2.7, 3.6)
DEFAULT_PROGRESSION_SCALING = (0.9, 1.05, 0.9, 0.8, 0.8)
DEFAULT_DEATH_SCALING = (1.0, 1.03, 1.3, 0.6, 0.6)


class InputError(ValueError):
    pass


def read_json(path):
    with open(path) as f:
        return json.load(f)


def time_minutes(raw):
    """TimeDay(double) (src/tools/timeDay.cpp:58-62) of a schedule time given
    in the files' H.MM notation (AgentTypeList::Event casts it to float
    first), in minutes: hours in an unsigned char, -1 = 255 hours."""
    r = float(np.float32(raw))
    hours = 255 if r == -1.0 else int(r) & 0xFF
    minutes = int(round(((r - int(r)) / 0.6) * 60)) & 0xFF
    return hours * 60 + minutes


def parse_wb(s):
    """states::parseWBState (src/agentData/globalStates.cpp:7-24)."""
    if len(s) != 1 or s.upper() not in WB:
        raise InputError("invalid WB state %r" % s)
    return WB[s.upper()]


def parse_days(s):
    """Timehandler::parseDays (src/tools/timeHandler.cpp:53-88)."""
    d = s.upper()
    if d not in DAYS:
        raise InputError("invalid day type %r" % s)
    return list(DAYS[d])


def _u32(x):
    return int(x) % (1 << 32)


def _age_range(f):
    """ProgressionType's ages are unsigned: an end of -1 has no bound."""
    return _u32(f["age"][0]), _u32(f["age"][1])


def progression_index(config, parameters):
    """{(age_begin, age_end, preCond): index} and the files in the order of
    the reference's map (by age begin, then pre-condition)."""
    files = sorted(config["transitionMatrices"], key=lambda f: (_age_range(f)[0], f["preCond"]))
    inters = []
    for f in files:
        a, b = _age_range(f)
        pos = None
        for j, (ia, ib) in enumerate(inters):
            if b < ia:
                pos = j
                break
            if (ia, ib) == (a, b):
                pos = -1
                break
        if pos is None:
            inters.append((a, b))
        elif pos >= 0:
            inters.insert(pos, (a, b))
    conds = [c["ID"] for c in parameters["preCondition"]]
    index = {}
    for f in files:
        a, b = _age_range(f)
        age_i = next(j for j, (ia, _) in enumerate(inters) if ia == a)
        cond_i = conds.index(f["preCond"]) if f["preCond"] in conds else len(conds)
        index[(a, b, f["preCond"])] = age_i * len(conds) + cond_i
    return index, files


def load(agents, locations, agent_types, location_types, parameters, progression_config, *,
         infectiousness_multiplier=DEFAULT_MULTIPLIER, progression_scaling=DEFAULT_PROGRESSION_SCALING,
         death_scaling=DEFAULT_DEATH_SCALING, disable_tourists=True, quarantine_policy=0, quarantine_length=10,
         time_step=10, days_seed=1, params=None):
    """Snapshot of the reference's inputs.  Each input is a path or an
    already-decoded document; the progression directory's transition files
    are read from the directory of `progression_config` when it is a path,
    or taken from a dict {fileName: document} given as
    progression_config["_files"]."""
    docs = {}
    for name, v in [("agents", agents), ("locations", locations), ("agent_types", agent_types),
                    ("location_types", location_types), ("parameters", parameters),
                    ("progression", progression_config)]:
        docs[name] = read_json(v) if isinstance(v, (str, os.PathLike)) else v
    prog_cfg = docs["progression"]
    if isinstance(progression_config, (str, os.PathLike)):
        base = os.path.dirname(os.path.abspath(progression_config))
        matrices = {f["fileName"]: read_json(os.path.join(base, f["fileName"])) for f in prog_cfg["transitionMatrices"]}
    else:
        matrices = prog_cfg["_files"]
    lt = docs["location_types"]
    V = len(infectiousness_multiplier)
    if not 1 <= V <= MAX_STRAINS:
        raise InputError("1 to %d variants" % MAX_STRAINS)
    model = _model(prog_cfg, matrices, docs["parameters"], docs["agent_types"], lt, infectiousness_multiplier,
                   progression_scaling, death_scaling)
    locs, loc_map, cemetery = _locations(docs["locations"], lt)
    index, _ = progression_index(prog_cfg, docs["parameters"])
    agents_d = _agents(docs["agents"], model, index, docs["parameters"], docs["agent_types"], lt, loc_map,
                       disable_tourists, quarantine_policy, quarantine_length, time_step, days_seed)
    p = default_params()
    p.update({"time_step": time_step, "home_type": lt["home"], "work_type": lt["work"], "school_type": lt["school"],
              "classroom_type": lt["classroom"], "hospital_type": lt["hospital"], "doctor_type": lt["doctor"],
              "public_type": lt["publicSpace"], "nursery_type": lt["nurseryhome"], "cemetery_loc": cemetery,
              "quarantine_policy": quarantine_policy, "quarantine_length": quarantine_length, "n_bands": 1,
              "sigma_band": np.ones(16, np.float32)})
    if params:
        p.update(params)
    return Snapshot(model, agents_d, locs, p)


def _model(cfg, matrices, parameters, agent_types, lt, multiplier, prog_scaling, death_scaling):
    info = cfg["stateInformation"]
    names = list(info["stateNames"])
    S = len(names)
    idx = {n: j for j, n in enumerate(names)}
    wb = np.zeros(S, np.uint8)
    inf = np.zeros(S, np.float32)
    pcr = np.zeros(S, np.float32)
    ant = np.zeros(S, np.float32)
    for st in cfg["states"]:
        j = idx[st["stateName"]]
        wb[j] = parse_wb(st["WB"])
        inf[j] = st["infectious"]
        pcr[j] = st["accuracyPCR"]
        ant[j] = st["accuracyAntigen"]
    infected = np.zeros(S, np.uint8)
    infected[[idx[n] for n in info["infectedStates"]]] = 1
    susc = np.zeros(S, np.uint8)
    susc[[idx[n] for n in info["susceptibleStates"]]] = 1
    dead = [j for j in range(S) if wb[j] == WB["D"]]
    index, files = progression_index(cfg, parameters)
    n_prog = max(index.values()) + 1
    # per progression, per state (the file's own state order, as the
    # reference indexes them): bad transitions, then neutral ones
    bb, bc, nb, nc = ([0] * (n_prog * S) for _ in range(4))
    nxt, ch = [], []
    la = np.zeros(n_prog * S * MAX_STRAINS, np.float32)
    lm = np.zeros_like(la)
    lp = np.zeros(n_prog * S * MAX_STRAINS, np.float64)
    seen = set()
    for f in files:
        pi = index[_age_range(f) + (f["preCond"],)]
        seen.add(pi)
        states = matrices[f["fileName"]]["states"]
        if len(states) != S:
            raise InputError("%s: %d states, the directory names %d" % (f["fileName"], len(states), S))
        own = {s["stateName"]: j for j, s in enumerate(states)}
        for s_i, s in enumerate(states):
            bad = [(own[t["name"]], t["chance"]) for t in s["progressions"] if t["isBadProgression"]]
            neu = [(own[t["name"]], t["chance"]) for t in s["progressions"] if not t["isBadProgression"]]
            if s["progressions"] and not (0.9999 < sum(t["chance"] for t in s["progressions"]) < 1.0001):
                raise InputError("%s: chances of %s do not sum to 1" % (f["fileName"], s["stateName"]))
            if not bad and not neu:
                neu = [(s_i, 1.0)]  # NextStatesInit::cleanUp
            r = pi * S + s_i
            bb[r], bc[r] = len(nxt), len(bad)
            for n_, c_ in bad:
                nxt.append(n_)
                ch.append(c_)
            nb[r], nc[r] = len(nxt), len(neu)
            for n_, c_ in neu:
                nxt.append(n_)
                ch.append(c_)
            avg = [float(np.float32(x)) for x in s["avgLength"]]
            mx = [float(np.float32(x)) for x in s["maxlength"]]
            if not avg or len(avg) != len(mx):
                raise InputError("%s: avgLength and maxlength of %s" % (f["fileName"], s["stateName"]))
            for v in range(MAX_STRAINS):
                a = avg[min(v, len(avg) - 1)]
                m = mx[min(v, len(mx) - 1)]
                if a != -1.0 and m == -1.0:
                    raise InputError("%s: %s has an average length but no maximum" % (f["fileName"], s["stateName"]))
                o = r * MAX_STRAINS + v
                la[o] = a
                lm[o] = FLT_MAX if m == -1.0 else m
                with np.errstate(over="ignore", invalid="ignore"):
                    lp[o] = calculate_modified_p(a, m)
    if len(seen) != n_prog:
        raise InputError("progression indices are not contiguous")
    model = {
        "n_states": S, "n_variants": len(multiplier), "n_prog": n_prog,
        "n_agent_types": len(agent_types["types"]),
        "first_infected_state": idx[info["firstInfectedState"]],
        "noncovid_dead_state": idx[info["nonCOVIDDeadState"]], "dead_state": dead[0] if dead else 0,
        "state_wb": wb, "state_infectious": inf, "state_susceptible": susc, "state_infected": infected,
        "state_acc_pcr": pcr, "state_acc_antigen": ant,
        "variant_multiplier": np.asarray(multiplier, np.float32),
        "prog_scaling": np.asarray(_per_variant(prog_scaling, len(multiplier)), np.float32),
        "death_scaling": np.asarray(_per_variant(death_scaling, len(multiplier)), np.float32),
        "tr_bad_begin": np.array(bb, np.uint32), "tr_bad_count": np.array(bc, np.uint32),
        "tr_neu_begin": np.array(nb, np.uint32), "tr_neu_count": np.array(nc, np.uint32),
        "tr_next": np.array(nxt, np.uint32), "tr_chance": np.array(ch, np.float32),
        "len_avg": la, "len_max": lm, "len_p": lp, "state_names": names,
    }
    model.update(_schedules(agent_types))
    return model


def _per_variant(values, n):
    values = list(values)
    return [values[min(v, len(values) - 1)] for v in range(n)]


def _schedules(agent_types):
    """The event table indexed 28 * type + 7 * WB + day; a schedule is inserted
    at the front of its slot (AgentTypeList::addSchedule)."""
    T = len(agent_types["types"])
    slots = [[] for _ in range(T * 28)]
    for ti, t in enumerate(agent_types["types"]):
        for sch in t["schedulesUnique"]:
            w = parse_wb(sch["WB"])
            ev = [(int(e["type"]), float(np.float32(e["chance"])), time_minutes(e["start"]), time_minutes(e["end"]),
                   time_minutes(e["duration"])) for e in sch["schedule"]]
            for d in parse_days(sch["dayType"]):
                slot = 7 * w + d + ti * 28
                slots[slot] = ev + slots[slot]
    off = np.zeros(T * 28 + 1, np.uint32)
    events = []
    for j, sl in enumerate(slots):
        off[j] = len(events)
        events.extend(sl)
    off[-1] = len(events)
    e = np.array(events, dtype=object).reshape(-1, 5) if events else np.zeros((0, 5))
    return {
        "event_offset": off, "ev_loc_type": np.array(e[:, 0], np.uint32), "ev_chance": np.array(e[:, 1], np.float32),
        "ev_start": np.array(e[:, 2], np.uint16), "ev_end": np.array(e[:, 3], np.uint16),
        "ev_duration": np.array(e[:, 4], np.uint16),
    }


def _locations(doc, lt):
    """Locations in file order, the cemetery appended; ID -> first index."""
    places = doc["places"]
    ids = {}
    L = len(places) + 1
    ltype = np.zeros(L, np.uint8)
    w = np.zeros(L, np.float32)
    open_ = np.ones(L, np.uint8)
    ess = np.zeros(L, np.uint8)
    schools, school_ids, classrooms, classroom_ids = [], [], [], []
    for j, p in enumerate(places):
        ids.setdefault(p["ID"], j)
        if not 0 <= p["type"] < 256:
            raise InputError("location type %r" % p["type"])
        ltype[j] = p["type"]
        w[j] = p["infectious"]
        ess[j] = p["essential"]
        # the reference compares the state as written (its upper-case pass
        # discards the result, include/locationList.h:157-166)
        if p["state"] in ("ON", "OPEN"):
            open_[j] = 1
        elif p["state"] in ("OFF", "CLOSED"):
            open_[j] = 0
        else:
            raise InputError("location state %r" % p["state"])
        if p["type"] == lt["classroom"]:
            classrooms.append(j)
            classroom_ids.append(p["ID"])
        if p["type"] == lt["school"]:
            schools.append(j)
            school_ids.append(p["ID"])
    cem = L - 1
    ltype[cem] = max(t["ID"] for t in lt["types"])
    w[cem], open_[cem], ess[cem] = 0.0, 1, 1
    # classroom -> school pairing by "<class>_<schoolID>", stable by school
    school_of = []
    for cid in classroom_ids:
        pos = cid.find("_")
        if pos < 0 or cid[pos + 1:] not in ids:
            raise InputError("classroom id %r does not name its school" % cid)
        school_of.append(ids[cid[pos + 1:]])
    order = sorted(range(len(classrooms)), key=lambda q: school_of[q])
    classrooms = [classrooms[q] for q in order]
    school_of = [school_of[q] for q in order]
    offsets = []
    for s in schools:
        if s in school_of:
            offsets.append(school_of.index(s))
        else:
            if not offsets:
                offsets.append(0)
            offsets.append(offsets[-1])
    offsets.append(len(school_of))
    locs = {
        "type": ltype, "infectiousness": w, "open": open_, "essential": ess,
        "closed_until": np.zeros(L, np.uint32), "quarantine_until": np.zeros(L, np.uint32),
        "schools": np.array(schools, np.uint32), "classrooms": np.array(classrooms, np.uint32),
        "classroom_offsets": np.array(offsets, np.uint32),
    }
    return locs, ids, cem


def _agents(doc, model, index, parameters, agent_types, lt, loc_map, disable_tourists, qpolicy, qlength, time_step,
            days_seed):
    type_map = {}
    for ti, t in enumerate(agent_types["types"]):
        type_map.setdefault(t["ID"], ti)
    sex_sym = {}
    for sx in parameters["sex"]:
        sex_sym[sx["name"]] = np.float32(sx["symptoms"])
    if sorted(sex_sym) != ["F", "M"]:
        raise InputError("sexes F and M")
    ages = [(a["from"], a["to"] if a["to"] >= 0 else 2 ** 32 - 1, np.float32(a["symptoms"])) for a in parameters["age"]]
    pre = {c["ID"]: np.float32(c["symptoms"]) for c in parameters["preCondition"]}
    names = model["state_names"]
    sidx = {n: j for j, n in enumerate(names)}
    people = [p for p in doc["people"] if not (disable_tourists and p["typeID"] == 9)]
    N = len(people)
    rng = np.random.default_rng(days_seed)
    S = model["n_states"]
    a = {k: np.zeros(N, dt) for k, dt in [("type", np.uint8), ("age", np.uint8), ("band", np.uint8),
                                          ("prog_id", np.uint16), ("symptom_scaling", np.float32),
                                          ("precond", np.uint8), ("sex", np.uint8), ("location", np.uint32),
                                          ("state", np.int8), ("days", np.int16), ("diagnosed", np.uint8)]}
    off = np.zeros(N + 1, np.uint32)
    poss_loc, poss_type = [], []
    home = lt["home"]
    for i, p in enumerate(people):
        key = [k for k in index if k[0] <= p["age"] <= k[1] and k[2] == p["preCond"]]
        if not key:
            raise InputError("agent %d: no progression for age %d, pre-condition %r" % (i, p["age"], p["preCond"]))
        a["prog_id"][i] = index[key[0]]
        if p["state"] not in sidx:
            raise InputError("agent %d: unknown state %r" % (i, p["state"]))
        st = sidx[p["state"]]
        a["state"][i] = st
        o = (int(a["prog_id"][i]) * S + st) * MAX_STRAINS
        if model["len_avg"][o] == -1.0:
            a["days"][i] = -1
        else:
            pp, mx = float(model["len_p"][o]), float(model["len_max"][o])
            d = rng.geometric(pp) - 1
            while mx < d:
                d = rng.geometric(pp) - 1
            a["days"][i] = d
        if len(p["sex"]) != 1 or p["sex"] not in sex_sym:
            raise InputError("agent %d: sex %r" % (i, p["sex"]))
        if p["typeID"] not in type_map:
            raise InputError("agent %d: agent type %r" % (i, p["typeID"]))
        a["type"][i] = type_map[p["typeID"]]
        a["age"][i] = p["age"]
        a["sex"][i] = 1 if p["sex"] == "M" else 0
        a["precond"][i] = int(p["preCond"])
        age_sym = next((s for lo, hi, s in ages if lo <= p["age"] < hi), None)
        if age_sym is None or p["preCond"] not in pre:
            raise InputError("agent %d: age %d or pre-condition %r undefined" % (i, p["age"], p["preCond"]))
        scale = np.float32(1.0) * sex_sym[p["sex"]]
        scale = np.float32(scale * age_sym)
        a["symptom_scaling"][i] = np.float32(scale * pre[p["preCond"]])
        a["diagnosed"][i] = 1 if p.get("diagnosed") else 0
        ls = sorted(p["locations"], key=lambda q: q["typeID"])
        for q in ls:
            if q["locID"] not in loc_map:
                raise InputError("agent %d: location %r" % (i, q["locID"]))
            poss_loc.append(loc_map[q["locID"]])
            poss_type.append(q["typeID"])
        off[i + 1] = len(poss_loc)
        homes = [loc_map[q["locID"]] for q in ls if q["typeID"] == home]
        a["location"][i] = homes[0] if homes else 0
    V = model["n_variants"]
    st = a["state"].astype(np.int64)
    infected0 = model["state_infected"][st] == 1
    diag = a["diagnosed"] == 1
    U32MAX = np.uint32(NONE)
    z32 = np.zeros(N, np.uint32)
    a.update({
        "loc_offset": off, "poss_loc": np.array(poss_loc, np.uint32), "poss_type": np.array(poss_type, np.uint8),
        "steps_until_move": z32.copy(), "variant": np.zeros(N, np.uint8),
        "infectious": (model["state_infectious"][st] * model["variant_multiplier"][0]).astype(np.float32),
        "susceptible": np.tile(model["state_susceptible"][st].astype(np.float32), V),
        "quarantined": (diag & (qpolicy > 0)).astype(np.uint8), "stayed_home": np.ones(N, np.uint8),
        "no_work": np.zeros(N, np.uint8), "last_test": np.full(N, U32MAX, np.uint32),
        "st_infected_ts": np.where(infected0, 0, U32MAX).astype(np.uint32),
        "st_infected_loc": z32.copy(), "st_worst_ts": z32.copy(), "st_worst_end_ts": z32.copy(),
        "st_diagnosed_ts": diag.astype(np.uint32),
        "st_quarantined_ts": z32.copy(),
        "st_quarantined_until": np.where(diag & (qpolicy > 0), qlength * 24 * 60 // time_step, 0).astype(np.uint32),
        "st_days_in_quarantine": np.where(diag & (qpolicy > 0), qlength, 0).astype(np.uint32),
        "st_hospitalized_ts": z32.copy(), "st_hospitalized_until": z32.copy(), "st_immunization_ts": z32.copy(),
        "st_recovered_ts": np.full(N, U32MAX, np.uint32), "st_variant_mask": z32.copy(),
        "st_immunization_count": np.zeros(N, np.uint8), "st_infected_count": infected0.astype(np.uint8),
        "st_worst_state": np.where(infected0, st, 0).astype(np.int8),
    })
    return a

