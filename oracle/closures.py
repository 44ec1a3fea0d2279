"""Oracle restatement of the closure rule engine — TEST INFRASTRUCTURE ONLY.

RuleClosure (include/policies/closurePolicies.h:48-479) over the oracle's
in-place snapshot: conditions afterDays / hospitalizedFraction /
newDeadFraction (:109-232) plus the newCasesFraction extension (NI column,
hospitalizedFraction's hysteresis), and the rules of :234-471.  Schedule
edits restate AgentTypeList::setStayHome / unsetStayHome
(src/agentData/agentType.cpp:28-119).  Float arithmetic follows the
reference's float/double mixing with numpy scalars.
"""
import numpy as np

from pansim_gb300 import snapshot as snp

from . import binding as ob

SWITCH_RULES = {"Masks", "Curfew", "HolidayMode", "SchoolAgeRestriction", "ExposeToMutation", "ReduceMovement",
                "QuarantinePolicy", "QuarantineImmune", "LockdownNonvacc", "TestingProb"}


def split_header(h):
    """ClosureHelpers::splitHeader (closurePolicies.h:9-28)."""
    out, arg, i = [], "", 0
    while i < len(h):
        ch = h[i]
        i += 1
        if ch in " \t\n\r\v\f":
            continue
        arg += ch
        if i < len(h) and h[i] == "\t":
            if arg:
                out.append(arg)
                arg = ""
            i += 1
    if arg:
        out.append(arg)
    return out


class _Cond:
    def __init__(self, rule, kind, cols=(), prev=0):
        self.kind = kind
        self.th, self.th2 = float(rule.get("threshold", 0)), float(rule.get("threshold2", 0))
        self.ca, self.oa = int(rule.get("closeAfter", 0)), int(rule.get("openAfter", 0))
        self.cols, self.prev = list(cols), prev
        self.active = False
        self.pos = 0
        self.hist = [0.0] if kind == "afterDays" else [0.0] * (max(self.ca, self.oa) + 2)

    def _hyst(self, value):
        H = len(self.hist)
        self.hist[self.pos] = value
        self.pos = (self.pos + 1) % H
        if not self.active and value > self.th:
            i = (self.pos - self.ca) % H
            below = False
            while i != self.pos:
                below |= self.hist[i] < self.th
                i = (i + 1) % H
            return self.active if below else True
        if self.active and value <= self.th2:
            i = (self.pos - self.oa) % H
            above = False
            while i != self.pos:
                above |= self.hist[i] >= self.th2
                i = (i + 1) % H
            return self.active if above else False
        return self.active

    def update(self, row, n_agents):
        v = list(row.v)[: row.n]
        at = lambda c: v[c] if c < len(v) else 0
        if self.kind == "afterDays":
            day = int(self.hist[0])
            self.hist[0] += 1.0
            self.active = day >= self.th and day < self.th + self.oa
        elif self.kind == "hospitalizedFraction":
            acc = 0.0
            for c in self.cols:
                acc += at(c)
            self.active = self._hyst(acc / float(n_agents))
        elif self.kind == "newDeadFraction":
            d = at(self.cols[0])
            value = float((d - self.prev) & 0xFFFFFFFF) / float(n_agents)
            self.prev = d
            self.active = self._hyst(value)
        else:  # newCasesFraction
            self.active = self._hyst(float(row.new_infections) / float(n_agents))


class OracleClosures:
    def __init__(self, oracle, rules, header, enable_closures=True):
        self.o = oracle
        self.snap = oracle.snap
        cols = split_header(header)
        hosp = [i for i, c in enumerate(cols) if "_h" in c]
        dead = [i for i, c in enumerate(cols) if c == "D1"]
        self.conds, self.rules = [], []
        V = int(self.snap.model["n_variants"])
        for r in rules:
            name, ct = r["name"], r.get("conditionType", "")
            if not enable_closures and name not in SWITCH_RULES:
                continue
            if ct == "afterDays":
                if int(r["closeAfter"]) >= 0 or int(r["openAfter"]) <= 0:
                    raise ValueError("afterDays: closeAfter must be -1, openAfter > 0")
                cd = _Cond(r, ct)
            elif ct in ("hospitalizedFraction", "newDeadFraction", "newCasesFraction"):
                if int(r["closeAfter"]) <= 0 or int(r["openAfter"]) <= 0:
                    raise ValueError(ct + ": closeAfter and openAfter must be > 0")
                if ct == "newDeadFraction":
                    if not dead:
                        raise ValueError("no D1 column")
                    cd = _Cond(r, ct, [dead[0]], dead[1] if len(dead) > 1 else 0)
                else:
                    cd = _Cond(r, ct, hosp if ct == "hospitalizedFraction" else [])
            else:
                raise ValueError("Unknown closure type " + ct)
            self.conds.append(cd)
            rr = dict(name=name, cond=cd, prev_open=True, param=str(r.get("parameter", "")), rule=r)
            if name == "Curfew":
                p = rr["param"]
                if len(p) == 9:
                    rr["cb"] = int(p[0:2]) * 60 + int(p[2:4])
                    rr["ce"] = int(p[5:7]) * 60 + int(p[7:9])
                elif p:
                    raise ValueError("curfew parameter string needs to be exactly 9 characters long")
                else:
                    rr["cb"] = rr["ce"] = 0
            if name == "ExposeToMutation":
                rr["variant"] = int(float(r.get("threshold2", 0)))
                if rr["variant"] >= V:
                    raise ValueError("More ExposeToMutation events defined than variants")
            self.rules.append(rr)
        self.current_mask = 1.0

    # --- actions on the oracle's snapshot
    def _params(self, **kw):
        self.snap.params.update(kw)
        self.o.set_params()

    def _masks(self, coef, open_):
        locs = self.snap.locs
        w = locs["infectiousness"]
        sel = locs["type"] != int(self.snap.params["home_type"])
        w64 = w[sel].astype(np.float64)
        w[sel] = (w64 / coef if open_ else w64 * coef).astype(np.float32)

    def _close_types(self, types, open_):
        locs = self.snap.locs
        sel = np.isin(locs["type"].astype(np.int64), np.array(types, np.int64)) & (locs["essential"] != 1)
        locs["open"][sel] = 1 if open_ else 0

    def _events(self):
        m = self.snap.model
        return (list(m["event_offset"]), list(m["ev_loc_type"]), [np.float32(x) for x in m["ev_chance"]],
                list(m["ev_start"]), list(m["ev_end"]), list(m["ev_duration"]))

    def _store_events(self, ev):
        off, ty, ch, st, en, du = ev
        m = self.snap.model
        m["event_offset"] = np.array(off, np.uint32)
        m["ev_loc_type"] = np.array(ty, np.uint32)
        m["ev_chance"] = np.array(ch, np.float32)
        m["ev_start"] = np.array(st, np.uint16)
        m["ev_end"] = np.array(en, np.uint16)
        m["ev_duration"] = np.array(du, np.uint16)
        ms = self.o.structs[0]
        for k in ["event_offset", "ev_loc_type", "ev_chance", "ev_start", "ev_end", "ev_duration"]:
            setattr(ms, k, snp._ptr(m[k]))
        ms.n_events = len(ty)

    def _stay_home(self, p, set_):
        off, ty, ch, st, en, du = self._events()
        home = int(self.snap.params["home_type"])
        one_m = 1.0 - p
        for s in range(len(off) - 1):
            ws = we = off[s]
            while ws < off[s + 1]:
                while we < len(ty) and st[we] == st[ws]:
                    we += 1
                if set_:
                    present = False
                    for i in range(ws, we):
                        if ty[i] == home:
                            present = True
                            ch[i] = np.float32(float(ch[i]) + (1.0 - float(ch[i])) * p)
                            break
                    if present and we - ws == 1:
                        ws = we
                        continue
                    if not present:
                        for arr, val in ((ty, home), (ch, np.float32(p)), (st, st[ws]), (en, en[ws]), (du, du[ws])):
                            arr.insert(ws, val)
                        we += 1
                        for q in range(s + 1, len(off)):
                            off[q] += 1
                    for i in range(ws, we):
                        if ty[i] != home:
                            ch[i] = np.float32(float(ch[i]) * one_m)
                else:
                    for i in range(ws, we):
                        if ty[i] != home:
                            ch[i] = np.float32(float(ch[i]) / one_m)
                    for i in range(ws, we):
                        if ty[i] == home:
                            ch[i] = np.float32((float(ch[i]) - p) / one_m)
                            if abs(float(ch[i])) < 1e-10:
                                for arr in (ty, ch, st, en, du):
                                    del arr[i]
                                for q in range(s + 1, len(off)):
                                    off[q] -= 1
                            break
                ws = we
        self._store_events((off, ty, ch, st, en, du))

    def midnight(self, t, row):
        n_agents = self.snap.n_agents
        for c in self.conds:
            c.update(row, n_agents)
        P = self.snap.params
        dt = int(P["time_step"])
        for r in self.rules:
            close = r["cond"].active
            open_ = not close
            tog = r["prev_open"] != open_
            name = r["name"]
            if name == "Masks":
                if tog:
                    coef = float(r["param"])
                    self.current_mask = 1.0 if open_ else coef
                    self._masks(coef, open_)
                    r["prev_open"] = open_
            elif name == "Curfew":
                if tog:
                    self._params(enable_curfew=int(close), curfew_begin=r["cb"] // dt, curfew_end=r["ce"] // dt)
                    r["prev_open"] = open_
            elif name in ("HolidayMode", "QuarantineImmune", "LockdownNonvacc"):
                if tog:
                    key = {"HolidayMode": "holiday_mode", "QuarantineImmune": "quarantine_immune",
                           "LockdownNonvacc": "lockdown_nonvacc"}[name]
                    self._params(**{key: int(close)})
                    r["prev_open"] = open_
            elif name == "QuarantinePolicy":
                if close:
                    self._params(quarantine_policy=int(r["param"]))
                    r["prev_open"] = close
            elif name == "SchoolAgeRestriction":
                if tog:
                    self._params(school_age_restriction=int(r["param"]) if close else 99)
                    r["prev_open"] = open_
            elif name == "TestingProb":
                if close:
                    keys = ["t_random", "t_home", "t_work", "t_school", "t_hospital", "t_nursery"]
                    vals = [float(x) for x in r["param"].split(",") if x.strip()]
                    self._params(**dict(zip(keys, vals)))
            elif name == "ExposeToMutation":
                if close:
                    ob.lib().psim_oracle_expose(self.o.h, t, r["variant"], float(r["param"]))
            elif name == "ReduceMovement":
                if tog:
                    self._stay_home(float(r["param"]), set_=not open_)
                    r["prev_open"] = open_
            else:
                if tog:
                    self._close_types(r["rule"].get("locationTypesToClose", []), open_)
                    r["prev_open"] = open_

    def status(self):
        return (np.array([r["cond"].active for r in self.rules], bool),
                np.array([r["prev_open"] for r in self.rules], bool))


def run_day(oracle, engine, day):
    """One day of runSimulation (simulation.h:906-922) with the rules after
    the statistics."""
    snap = oracle.snap
    t0 = day * snap.steps_per_day
    if t0 > 0 and int(snap.params.get("testing_enabled", 0)):
        oracle.test(t0)
    if t0 > 0:
        oracle.progress(t0)
    st = oracle.stats(t0)
    if engine is not None:
        engine.midnight(t0, st[0])
    oracle.plan(t0)
    for s in range(snap.steps_per_day):
        oracle.step(t0 + s)
    return st
