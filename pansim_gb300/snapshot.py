"""Host-side structure-of-arrays snapshot of a PanSim population.

A Snapshot holds numpy arrays named after the fields of the C ABI structs
(include/pansim_gb300.h) and builds the ctypes views the library and the
oracle read and write in place.  It is the exchange format between the
generator, the GPU context and the oracle.
"""
import copy
import ctypes as C

import numpy as np

from . import cabi

NONE = 0xFFFFFFFF

# dtype of every array field
AGENT_DTYPES = {
    "type": np.uint8, "age": np.uint8, "band": np.uint8, "prog_id": np.uint16,
    "symptom_scaling": np.float32, "loc_offset": np.uint32, "poss_loc": np.uint32,
    "poss_type": np.uint8, "location": np.uint32, "steps_until_move": np.uint32,
    "state": np.int8, "days": np.int16, "variant": np.uint8, "infectious": np.float32,
    "susceptible": np.float32, "diagnosed": np.uint8, "quarantined": np.uint8,
    "stayed_home": np.uint8, "no_work": np.uint8, "last_test": np.uint32,
    "st_infected_ts": np.uint32, "st_infected_loc": np.uint32, "st_worst_ts": np.uint32,
    "st_worst_end_ts": np.uint32, "st_diagnosed_ts": np.uint32, "st_quarantined_ts": np.uint32,
    "st_quarantined_until": np.uint32, "st_days_in_quarantine": np.uint32,
    "st_hospitalized_ts": np.uint32, "st_hospitalized_until": np.uint32,
    "st_immunization_ts": np.uint32, "st_recovered_ts": np.uint32, "st_variant_mask": np.uint32,
    "st_immunization_count": np.uint8, "st_infected_count": np.uint8, "st_worst_state": np.int8,
    "precond": np.uint8, "imm_round": np.uint8, "symptom_scaling_v": np.float32, "sex": np.uint8,
}
AGENT_MUTABLE = [
    "location", "steps_until_move", "state", "days", "variant", "infectious", "susceptible",
    "diagnosed", "quarantined", "stayed_home", "no_work", "last_test",
    "st_infected_ts", "st_infected_loc", "st_worst_ts", "st_worst_end_ts", "st_diagnosed_ts",
    "st_quarantined_ts", "st_quarantined_until", "st_days_in_quarantine", "st_hospitalized_ts",
    "st_hospitalized_until", "st_immunization_ts", "st_recovered_ts", "st_variant_mask",
    "st_immunization_count", "st_infected_count", "st_worst_state", "imm_round", "symptom_scaling_v",
]
LOC_DTYPES = {
    "type": np.uint8, "infectiousness": np.float32, "open": np.uint8, "essential": np.uint8,
    "closed_until": np.uint32, "quarantine_until": np.uint32, "schools": np.uint32,
    "classrooms": np.uint32, "classroom_offsets": np.uint32,
}
LOC_MUTABLE = ["infectiousness", "open", "closed_until", "quarantine_until"]
MODEL_DTYPES = {
    "state_wb": np.uint8, "state_infectious": np.float32, "state_susceptible": np.uint8,
    "state_infected": np.uint8, "state_acc_pcr": np.float32, "state_acc_antigen": np.float32,
    "variant_multiplier": np.float32, "prog_scaling": np.float32, "death_scaling": np.float32,
    "tr_bad_begin": np.uint32, "tr_bad_count": np.uint32, "tr_neu_begin": np.uint32,
    "tr_neu_count": np.uint32, "tr_next": np.uint32, "tr_chance": np.float32,
    "len_avg": np.float32, "len_max": np.float32, "len_p": np.float64,
    "event_offset": np.uint32, "ev_loc_type": np.uint32, "ev_chance": np.float32,
    "ev_start": np.uint16, "ev_end": np.uint16, "ev_duration": np.uint16,
}
MODEL_SCALARS = ["n_states", "n_variants", "n_prog", "n_agent_types", "first_infected_state",
                 "noncovid_dead_state", "dead_state"]


def _ptr(a):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "arrays must be contiguous"
    return a.ctypes.data_as(C.c_void_p)


class Snapshot:
    """model: dict (arrays + scalars); agents, locs: dict of arrays;
    params: dict of scalars; reps: dict with agent_offset, loc_offset, seed, k, cemetery."""

    def __init__(self, model, agents, locs, params, reps=None):
        self.model = model
        self.agents = agents
        self.locs = locs
        self.params = params
        if reps is None:
            n, L = len(agents["location"]), len(locs["type"])
            reps = {
                "agent_offset": np.array([0, n], np.uint32),
                "loc_offset": np.array([0, L], np.uint32),
                "seed": np.array([params["seed"]], np.uint64),
                "k": np.array([params["k"]], np.float64),
                "cemetery": np.array([params["cemetery_loc"]], np.uint32),
            }
        self.reps = reps
        self._normalize()

    def _normalize(self):
        # immunization and other-disease fields absent from older snapshots:
        # their neutral values
        n = len(self.agents["location"])
        V = int(self.model["n_variants"])
        if "sex" not in self.agents:
            self.agents["sex"] = np.zeros(n, np.uint8)
        if "precond" not in self.agents:
            self.agents["precond"] = np.zeros(n, np.uint8)
        if "imm_round" not in self.agents:
            self.agents["imm_round"] = np.zeros(n, np.uint8)
        if "symptom_scaling_v" not in self.agents:
            self.agents["symptom_scaling_v"] = np.tile(np.asarray(self.agents["symptom_scaling"], np.float32), V)
        for k, dt in AGENT_DTYPES.items():
            self.agents[k] = np.ascontiguousarray(self.agents[k], dtype=dt)
        for k, dt in LOC_DTYPES.items():
            self.locs[k] = np.ascontiguousarray(self.locs.get(k, np.zeros(0)), dtype=dt)
        for k, dt in MODEL_DTYPES.items():
            self.model[k] = np.ascontiguousarray(self.model[k], dtype=dt)
        r = self.reps
        r["agent_offset"] = np.ascontiguousarray(r["agent_offset"], np.uint32)
        r["loc_offset"] = np.ascontiguousarray(r["loc_offset"], np.uint32)
        r["seed"] = np.ascontiguousarray(r["seed"], np.uint64)
        r["k"] = np.ascontiguousarray(r["k"], np.float64)
        r["cemetery"] = np.ascontiguousarray(r["cemetery"], np.uint32)

    # sizes
    @property
    def n_agents(self):
        return int(len(self.agents["location"]))

    @property
    def n_locations(self):
        return int(len(self.locs["type"]))

    @property
    def n_replicas(self):
        return int(len(self.reps["seed"]))

    @property
    def steps_per_day(self):
        return 1440 // int(self.params["time_step"])

    def copy(self):
        return Snapshot(copy.deepcopy(self.model), {k: v.copy() for k, v in self.agents.items()},
                        {k: v.copy() for k, v in self.locs.items()}, dict(self.params),
                        {k: v.copy() for k, v in self.reps.items()})

    # ctypes views (keep the returned tuple alive while the C side uses it)
    def structs(self):
        m = cabi.PsimModel()
        for k in MODEL_SCALARS:
            setattr(m, k, int(self.model[k]))
        m.n_trans = len(self.model["tr_next"])
        m.n_events = len(self.model["ev_loc_type"])
        for k in MODEL_DTYPES:
            setattr(m, k, _ptr(self.model[k]))
        a = cabi.PsimAgents()
        a.n = self.n_agents
        a.n_poss = len(self.agents["poss_loc"])
        for k in cabi.AGENT_PTR_FIELDS:
            setattr(a, k, _ptr(self.agents[k]))
        lo = cabi.PsimLocations()
        lo.n = self.n_locations
        lo.n_schools = len(self.locs["schools"])
        lo.n_classrooms = len(self.locs["classrooms"])
        for k in cabi.LOC_PTR_FIELDS:
            arr = self.locs[k]
            setattr(lo, k, _ptr(arr) if arr.size else None)
        p = self.params_struct()
        r = cabi.PsimReplicas()
        r.n = self.n_replicas
        for k in ["agent_offset", "loc_offset", "seed", "k", "cemetery"]:
            setattr(r, k, _ptr(self.reps[k]))
        return m, a, lo, p, r

    def params_struct(self):
        p = cabi.PsimParams()
        for k in cabi.PARAM_U32:
            setattr(p, k, int(self.params.get(k, 0)))
        for k in ["k", "c0", "trunc", "t_random", "t_home", "t_work", "t_school", "t_hospital", "t_nursery"]:
            setattr(p, k, float(self.params.get(k, 0.0)))
        for k in ["d_offset0", "d_offset1", "d_peak_offset", "n_d_offset"]:
            setattr(p, k, int(self.params.get(k, 0)))
        p.seed = int(self.params.get("seed", 0))
        sig = self.params.get("sigma_band", np.ones(cabi.PSIM_MAX_BANDS, np.float32))
        for b in range(cabi.PSIM_MAX_BANDS):
            p.sigma_band[b] = float(sig[b]) if b < len(sig) else 1.0
        return p

    def validate(self):
        """Host-side checks the reference needs for a well-defined run
        (dataProvider.cpp:67-79: every agent has a home, hospital, public
        space and doctor location plus one of every type its schedule names)."""
        a, p, m = self.agents, self.params, self.model
        N, L = self.n_agents, self.n_locations
        off = a["loc_offset"]
        assert len(off) == N + 1 and off[0] == 0 and off[-1] == len(a["poss_loc"])
        assert np.all(np.diff(off.astype(np.int64)) >= 0)
        assert np.all(a["poss_loc"] < L), "per-agent location out of range"
        assert np.all(a["location"] < L), "agent location out of range"
        assert len(a["susceptible"]) == m["n_variants"] * N
        owner = np.repeat(np.arange(N), np.diff(off.astype(np.int64)))
        for need in ["home_type", "hospital_type", "public_type", "doctor_type"]:
            has = np.zeros(N, bool)
            has[owner[a["poss_type"] == p[need]]] = True
            assert has.all(), "agent without a %s location" % need
        return True


def save(snap, path, compress=True):
    """Binary snapshot (numpy .npz): every array and scalar of the model,
    agents, locations, parameters and replicas."""
    out = {}
    for k, v in snap.model.items():
        out["model/" + k] = np.asarray(v)
    for k, v in snap.agents.items():
        out["agents/" + k] = v
    for k, v in snap.locs.items():
        out["locs/" + k] = v
    for k, v in snap.params.items():
        out["params/" + k] = np.asarray(v)
    for k, v in snap.reps.items():
        out["reps/" + k] = v
    (np.savez_compressed if compress else np.savez)(path, **out)


def load(path):
    d = np.load(path, allow_pickle=False)
    parts = {"model": {}, "agents": {}, "locs": {}, "params": {}, "reps": {}}
    for key in d.files:
        group, name = key.split("/", 1)
        v = d[key]
        if group in ("model", "params") and v.ndim == 0:
            v = v.item()
        parts[group][name] = v
    return Snapshot(parts["model"], parts["agents"], parts["locs"], parts["params"], parts["reps"])


def concat(snaps, seeds, ks):
    """Batch replicas into one snapshot (agents and locations concatenated,
    per-agent location indices shifted)."""
    base = snaps[0]
    agents, locs = {}, {}
    a_off, l_off = [0], [0]
    for s in snaps:
        a_off.append(a_off[-1] + s.n_agents)
        l_off.append(l_off[-1] + s.n_locations)
    for k in AGENT_DTYPES:
        parts = []
        for r, s in enumerate(snaps):
            x = s.agents[k]
            if k in ("poss_loc", "location"):
                x = x + np.uint32(l_off[r])
            elif k == "st_infected_loc":
                x = x + np.uint32(l_off[r])
            elif k == "loc_offset":
                x = x[:-1] + np.uint32(sum(len(q.agents["poss_loc"]) for q in snaps[:r]))
            parts.append(x)
        if k == "loc_offset":
            parts.append(np.array([sum(len(q.agents["poss_loc"]) for q in snaps)], np.uint32))
        if k in ("susceptible", "symptom_scaling_v"):
            V = int(base.model["n_variants"])
            parts = [np.concatenate([s.agents[k].reshape(V, -1)[v] for s in snaps]) for v in range(V)]
        agents[k] = np.concatenate(parts).astype(AGENT_DTYPES[k])
    for k in ["type", "infectiousness", "open", "essential", "closed_until", "quarantine_until"]:
        locs[k] = np.concatenate([s.locs[k] for s in snaps])
    sch, cls, coff = [], [], [0]
    for r, s in enumerate(snaps):
        sch.append(s.locs["schools"] + l_off[r])
        cls.append(s.locs["classrooms"] + l_off[r])
        o = s.locs["classroom_offsets"]
        if len(o):
            coff.extend((o[1:] + coff[-1]).tolist())
    locs["schools"] = np.concatenate(sch) if sch else np.zeros(0, np.uint32)
    locs["classrooms"] = np.concatenate(cls) if cls else np.zeros(0, np.uint32)
    locs["classroom_offsets"] = np.array(coff if len(locs["schools"]) else [], np.uint32)
    params = dict(base.params)
    params["cemetery_loc"] = l_off[1] - 1
    reps = {
        "agent_offset": np.array(a_off, np.uint32),
        "loc_offset": np.array(l_off, np.uint32),
        "seed": np.array(seeds, np.uint64),
        "k": np.array(ks, np.float64),
        "cemetery": np.array([l_off[r + 1] - 1 for r in range(len(snaps))], np.uint32),
    }
    return Snapshot(copy.deepcopy(base.model), agents, locs, params, reps)
