"""Seeded synthetic PanSim populations for the benchmark configurations.

No public dataset is involved: the workloads are defined by their sizes and
distributions.  Model mapping onto the reference's semantics
(include/IO/dataProviders/dataProvider.cpp:67-79, movementPolicies.h):

* Location types use the reference's ids (inputConfigFiles/locationTypes.json):
  home 2, school 3, work 4, shop 7 (= publicSpace), hospital 12 (= doctor),
  classroom 33 and nursery home 22 are defined but unused; the cemetery gets
  the next id (34).
* Agent types: 0 child (age < 18) -> school, 1 adult -> work, 2 retiree
  (age >= 65) -> shop, 3 health worker (5% of adults) -> a hospital as work.
  Every agent has a home, two shops and a hospital (required types).
* Schedules: per agent type, weekday and weekend, WB states W and N; 3-6
  move windows per day, start uniform on the 10-min grid in [05:00, 23:00),
  window length 10 min, stay duration 1-8 h; 25% of windows offer two
  alternatives with Dirichlet(1) chances.  M-state agents have no events
  (stay home); S goes to hospital and D to the cemetery in the movement code.
* Disease: 10 states S E I1 I2 I3 I4 I5_h I6_h R D, an exact per-day Markov
  chain (avgLength 1, maxlength 0 -> dwell 0 days), one Dirichlet(1) row per
  infected state over its allowed successors, per age band (9 bands of 10
  years).  Per-state infectiousness U(0,1) for E..I6_h.
* 0.1% of agents start in I1.
"""
import math

import numpy as np

from .snapshot import Snapshot, NONE

HOME, SCHOOL, WORK, SHOP, HOSPITAL, CLASSROOM, NURSERY = 2, 3, 4, 7, 12, 33, 22
CEMETERY_TYPE = 34
STATE_NAMES = ["S", "E", "I1", "I2", "I3", "I4", "I5_h", "I6_h", "R", "D"]
WB = {"W": 0, "N": 1, "M": 2, "S": 3, "D": 4}
STATE_WB = [WB[x] for x in ["W", "W", "W", "N", "M", "M", "S", "S", "W", "D"]]
SUCCESSORS = {1: [1, 2], 2: [2, 3, 4], 3: [3, 4, 8], 4: [4, 5, 8], 5: [5, 6, 8], 6: [6, 7, 8], 7: [7, 8, 9]}
N_BANDS = 9
TYPE_W = {HOME: 1.0, WORK: 0.6, SCHOOL: 0.8, SHOP: 0.3, HOSPITAL: 0.5, CEMETERY_TYPE: 0.0}
MAX_STRAINS = 7


def expected_length(p, mx):
    """LengthOfState::expectedLength, basicLengthAbstract.cpp:4-14 (C double semantics)."""
    if p < 0.0:
        return np.float64(0.0)
    se, sc = np.float64(0.0), np.float64(0.0)
    for i in range(int(round(mx))):
        ch = np.float64((1.0 - p) ** i * p)
        se += (i + 1) * ch
        sc += ch
    with np.errstate(divide="ignore", invalid="ignore"):
        return se * (np.float64(1.0) / sc)


def calculate_modified_p(avg, mx):
    """LengthOfState::calculateModifiedP, basicLengthAbstract.cpp:16-29 with
    SecantMethod (include/tools/smallTools.h:15-31)."""
    if avg == -1.0:
        return 1.0
    n = float(avg)
    p_new = 1.0 / n

    def f(x):
        return expected_length(x, mx) - n

    try:
        xk, xprev = p_new - p_new * 0.1, p_new
        it = 0
        while 0.0001 < abs(f(xk)):
            tmp = xk
            diff = f(xk) - f(xprev)
            if diff != 0.0:
                xk = xk - f(xk) * (xk - xprev) / diff
            else:
                raise RuntimeError("secant stuck")
            xprev = tmp
            it += 1
            if it > 10000:
                raise RuntimeError("secant did not converge")
        p_new = float(xk)
    except RuntimeError:
        p_new = 1.0 / n
    if (p_new * 10.0 < 1.0 / n) or p_new > 1.0:
        p_new = 1.0 / n
    return p_new


def make_model(seed=0x5EED0000, n_variants=1, avg_len=1.0, max_len=0.0, acc_pcr=0.95):
    rng = np.random.default_rng(seed)
    S = len(STATE_NAMES)
    inf = np.zeros(S, np.float32)
    inf[1:8] = rng.random(7).astype(np.float32)
    susc = np.zeros(S, np.uint8)
    susc[0] = 1
    infected = np.zeros(S, np.uint8)
    infected[1:8] = 1
    pcr = np.where(infected == 1, acc_pcr, 0.0).astype(np.float32)
    ant = np.where(infected == 1, 0.8, 0.0).astype(np.float32)
    bb, bc, nb, nc, nxt, ch = [], [], [], [], [], []
    la, lm, lp = [], [], []
    for band in range(N_BANDS):
        for s in range(S):
            bb.append(len(nxt))
            bc.append(0)
            nb.append(len(nxt))
            succ = SUCCESSORS.get(s)
            if succ is None:
                nxt.append(s)
                ch.append(1.0)  # MultiBadMatrix::NextStatesInit::cleanUp
                nc.append(1)
                a, m = -1.0, -1.0
            else:
                w = rng.dirichlet(np.ones(len(succ)))
                for t_, c_ in zip(succ, w):
                    nxt.append(t_)
                    ch.append(float(np.float32(c_)))
                nc.append(len(succ))
                a, m = avg_len, max_len
            p = calculate_modified_p(a, m) if a != -1.0 else 1.0
            for v in range(MAX_STRAINS):
                la.append(a)
                lm.append(m if m != -1.0 else np.finfo(np.float32).max)
                lp.append(p)
    model = {
        "n_states": S, "n_variants": n_variants, "n_prog": N_BANDS, "n_agent_types": 4,
        "first_infected_state": 1, "noncovid_dead_state": 9, "dead_state": 9,
        "state_wb": np.array(STATE_WB, np.uint8), "state_infectious": inf,
        "state_susceptible": susc, "state_infected": infected,
        "state_acc_pcr": pcr, "state_acc_antigen": ant,
        "variant_multiplier": np.ones(n_variants, np.float32),
        "prog_scaling": np.ones(n_variants, np.float32),
        "death_scaling": np.ones(n_variants, np.float32),
        "tr_bad_begin": np.array(bb, np.uint32), "tr_bad_count": np.array(bc, np.uint32),
        "tr_neu_begin": np.array(nb, np.uint32), "tr_neu_count": np.array(nc, np.uint32),
        "tr_next": np.array(nxt, np.uint32), "tr_chance": np.array(ch, np.float32),
        "len_avg": np.array(la, np.float32), "len_max": np.array(lm, np.float32),
        "len_p": np.array(lp, np.float64),
    }
    model.update(make_schedules(rng))
    return model


def make_schedules(rng, n_types=4):
    """AgentTypeList events, offsets indexed 28*type + 7*WB + day for WB in
    W, N, M, S (agentType.cpp:13-19; D never looks up a schedule)."""
    primary = {0: SCHOOL, 1: WORK, 2: SHOP, 3: WORK}
    per_slot = {}
    for ty in range(n_types):
        for kind in ("weekday", "weekend"):
            k = int(rng.integers(3, 7))
            starts = np.sort(rng.choice(np.arange(5 * 6, 23 * 6), size=k, replace=False)) * 10
            evs = []
            for j, st in enumerate(starts):
                dur = int(rng.integers(6, 49)) * 10
                if j == 0 and kind == "weekday":
                    tgt = primary[ty]
                else:
                    tgt = [HOME, SHOP, primary[ty]][int(rng.integers(0, 3))]
                if rng.random() < 0.25:
                    alt = [HOME, SHOP][int(rng.integers(0, 2))]
                    w = rng.dirichlet([1.0, 1.0])
                    evs.append((tgt, float(np.float32(w[0])), st, st + 10, dur))
                    evs.append((alt, float(np.float32(w[1])), st, st + 10, int(rng.integers(6, 49)) * 10))
                else:
                    evs.append((tgt, 1.0, st, st + 10, dur))
            per_slot[(ty, kind)] = evs
    offsets = [0]
    ev = []
    for ty in range(n_types):
        for wb in range(4):
            for day in range(7):
                if wb in (WB["W"], WB["N"]):
                    evs = per_slot[(ty, "weekday" if day < 5 else "weekend")]
                elif ty == n_types - 1 and wb == WB["S"] and day == 6:
                    # padding: when the last event of a slot is active the
                    # reference reads the event after it as the next window
                    # (movementPolicies.h:601-603, 794-811); for the last slot
                    # with events that is this one, a 24:00 window.  S-state
                    # agents never look up a schedule, so it is never active.
                    evs = [(HOME, 1.0, 1440, 1440, 0)]
                else:
                    evs = []
                ev.extend(evs)
                offsets.append(len(ev))
    ev = np.array(ev, dtype=np.float64).reshape(-1, 5)
    return {
        "event_offset": np.array(offsets, np.uint32),
        "ev_loc_type": ev[:, 0].astype(np.uint32), "ev_chance": ev[:, 1].astype(np.float32),
        "ev_start": ev[:, 2].astype(np.uint16), "ev_end": ev[:, 3].astype(np.uint16),
        "ev_duration": ev[:, 4].astype(np.uint16),
    }


def default_params(seed=1, k=3.74e-4, quarantine_policy=0, testing=False):
    return {
        "time_step": 10, "start_day": 2, "start_date": 267,
        "home_type": HOME, "work_type": WORK, "school_type": SCHOOL, "classroom_type": CLASSROOM,
        "hospital_type": HOSPITAL, "doctor_type": HOSPITAL, "public_type": SHOP, "nursery_type": NURSERY,
        "cemetery_loc": 0, "quarantine_policy": quarantine_policy, "quarantine_length": 10,
        "enable_curfew": 0, "curfew_begin": 0, "curfew_end": 0, "school_age_restriction": 99,
        "holiday_mode": 0, "quarantine_immune": 0, "lockdown_nonvacc": 0,
        "testing_enabled": 1 if testing else 0, "testing_delay": 5, "use_pcr": 1,
        "n_bands": N_BANDS, "tracked": NONE, "pad0": 0,
        "k": k, "c0": 3.08, "trunc": 0.5, "d_offset0": -5, "d_offset1": 0, "d_peak_offset": 0, "n_d_offset": 1,
        "t_random": 5e-5, "t_home": 1e-2, "t_work": 5e-4, "t_school": 5e-4, "t_hospital": 5e-3, "t_nursery": 0.05,
        "seed": seed, "sigma_band": np.ones(16, np.float32),
    }


def make_population(model, n_agents, n_other_locs, pop_seed, initial_infected_frac=0.001,
                    frac=(0.30, 0.02, 0.676, 0.004)):
    """Households 1+Poisson(1.5), one home each; n_other_locs split over
    work/school/shop/hospital by `frac`; cemetery last."""
    rng = np.random.default_rng(pop_seed)
    N = int(n_agents)
    age = rng.integers(0, 91, N).astype(np.uint8)
    sizes = 1 + rng.poisson(1.5, size=N)
    cs = np.cumsum(sizes)
    H = int(np.searchsorted(cs, N) + 1)
    home = np.repeat(np.arange(H, dtype=np.uint32), sizes[:H])[:N]
    n_work = max(1, int(n_other_locs * frac[0]))
    n_school = max(1, int(n_other_locs * frac[1]))
    n_hosp = max(1, int(n_other_locs * frac[3]))
    n_shop = max(2, int(n_other_locs) - n_work - n_school - n_hosp)
    base_work = H
    base_school = base_work + n_work
    base_shop = base_school + n_school
    base_hosp = base_shop + n_shop
    L = base_hosp + n_hosp + 1
    cemetery = L - 1
    ltype = np.empty(L, np.uint8)
    ltype[:H] = HOME
    ltype[base_work:base_school] = WORK
    ltype[base_school:base_shop] = SCHOOL
    ltype[base_shop:base_hosp] = SHOP
    ltype[base_hosp:cemetery] = HOSPITAL
    ltype[cemetery] = CEMETERY_TYPE
    w = np.zeros(256, np.float32)
    for t_, v_ in TYPE_W.items():
        w[t_] = v_
    infl = w[ltype]

    atype = np.where(age < 18, 0, np.where(age >= 65, 2, 1)).astype(np.uint8)
    hcw = (atype == 1) & (rng.random(N) < 0.05)
    atype[hcw] = 3
    school = base_school + rng.integers(0, n_school, N)
    work = base_work + rng.integers(0, n_work, N)
    work_h = base_hosp + rng.integers(0, n_hosp, N)
    shop1 = base_shop + rng.integers(0, n_shop, N)
    shop2 = base_shop + (shop1 - base_shop + 1 + rng.integers(0, n_shop - 1, N)) % n_shop
    hosp = base_hosp + rng.integers(0, n_hosp, N)

    cnt = np.where(atype == 2, 4, 5).astype(np.int64)
    off = np.zeros(N + 1, np.int64)
    off[1:] = np.cumsum(cnt)
    M = int(off[-1])
    pl = np.zeros(M, np.uint32)
    pt = np.zeros(M, np.uint8)
    o = off[:-1]
    pl[o] = home
    pt[o] = HOME
    # second entry: school / work / (shop for retirees)
    is_child, is_ret = atype == 0, atype == 2
    sec_loc = np.where(is_child, school, np.where(atype == 3, work_h, work))
    sec_type = np.where(is_child, SCHOOL, WORK)
    nr = ~is_ret
    pl[o[nr] + 1] = sec_loc[nr]
    pt[o[nr] + 1] = sec_type[nr]
    k = np.where(is_ret, 1, 2)
    pl[o + k] = shop1
    pt[o + k] = SHOP
    pl[o + k + 1] = shop2
    pt[o + k + 1] = SHOP
    pl[o + k + 2] = hosp
    pt[o + k + 2] = HOSPITAL

    V = int(model["n_variants"])
    S = int(model["n_states"])
    state = np.zeros(N, np.int8)
    n_inf = max(1, int(round(N * initial_infected_frac)))
    inf_idx = rng.choice(N, size=n_inf, replace=False)
    state[inf_idx] = 2  # I1
    band = np.minimum(age // 10, N_BANDS - 1).astype(np.uint8)
    days = np.where(state == 0, -1, 0).astype(np.int16)
    variant = np.zeros(N, np.uint8)
    infectious = (model["state_infectious"][state] * model["variant_multiplier"][variant]).astype(np.float32)
    su = model["state_susceptible"][state].astype(np.float32)
    susceptible = np.tile(su, V)
    U32MAX = np.uint32(NONE)
    z32 = np.zeros(N, np.uint32)
    infected0 = model["state_infected"][state] == 1
    # pre-conditions (immunization categories) from their own stream, so the
    # draws above do not change: 10% of agents, index 1..3
    rng_pc = np.random.default_rng(pop_seed + 0x9C)
    precond = ((rng_pc.random(N) < 0.1) * rng_pc.integers(1, 4, N)).astype(np.uint8)
    # sex (non-COVID hospitalization tables), its own stream too: half F (0), half M (1)
    sex = np.random.default_rng(pop_seed + 0x9D).integers(0, 2, N).astype(np.uint8)
    agents = {
        "type": atype, "age": age, "band": band, "prog_id": band.astype(np.uint16),
        "symptom_scaling": np.ones(N, np.float32), "precond": precond, "sex": sex,
        "loc_offset": off.astype(np.uint32), "poss_loc": pl, "poss_type": pt,
        "location": home.astype(np.uint32), "steps_until_move": z32.copy(),
        "state": state, "days": days, "variant": variant, "infectious": infectious,
        "susceptible": susceptible, "diagnosed": np.zeros(N, np.uint8),
        "quarantined": np.zeros(N, np.uint8), "stayed_home": np.ones(N, np.uint8),
        "no_work": np.zeros(N, np.uint8), "last_test": np.full(N, U32MAX, np.uint32),
        "st_infected_ts": np.where(infected0, 0, U32MAX).astype(np.uint32),
        "st_infected_loc": z32.copy(), "st_worst_ts": z32.copy(), "st_worst_end_ts": z32.copy(),
        "st_diagnosed_ts": z32.copy(), "st_quarantined_ts": z32.copy(), "st_quarantined_until": z32.copy(),
        "st_days_in_quarantine": z32.copy(), "st_hospitalized_ts": z32.copy(),
        "st_hospitalized_until": z32.copy(), "st_immunization_ts": z32.copy(),
        "st_recovered_ts": np.full(N, U32MAX, np.uint32), "st_variant_mask": z32.copy(),
        "st_immunization_count": np.zeros(N, np.uint8),
        "st_infected_count": infected0.astype(np.uint8),
        "st_worst_state": np.where(infected0, state, 0).astype(np.int8),
    }
    locs = {
        "type": ltype, "infectiousness": infl, "open": np.ones(L, np.uint8),
        "essential": np.isin(ltype, [HOME, HOSPITAL, CEMETERY_TYPE]).astype(np.uint8),
        "closed_until": np.zeros(L, np.uint32), "quarantine_until": np.zeros(L, np.uint32),
        "schools": np.zeros(0, np.uint32), "classrooms": np.zeros(0, np.uint32),
        "classroom_offsets": np.zeros(0, np.uint32),
    }
    return agents, locs, cemetery


def make_snapshot(n_agents, n_other_locs, seed=1, pop_seed=None, model_seed=0x5EED0000, k=3.74e-4,
                  quarantine_policy=0, testing=False, n_variants=1, initial_infected_frac=0.001,
                  avg_len=1.0, max_len=0.0):
    model = make_model(model_seed, n_variants=n_variants, avg_len=avg_len, max_len=max_len)
    if pop_seed is None:
        pop_seed = model_seed + 1
    agents, locs, cem = make_population(model, n_agents, n_other_locs, pop_seed, initial_infected_frac)
    params = default_params(seed=seed, k=k, quarantine_policy=quarantine_policy, testing=testing)
    params["cemetery_loc"] = cem
    return Snapshot(model, agents, locs, params)


# The five workloads (population seed 0x5EED0000 + config number).
CONFIGS = {
    1: dict(n_agents=100_000, n_other_locs=20_000, weeks=1),
    2: dict(n_agents=2_000_000, n_other_locs=500_000, weeks=12),
    3: dict(n_agents=20_000_000, n_other_locs=5_000_000, weeks=4, quarantine_policy=3, testing=True),
}


def config_snapshot(cfg, scale=1.0, seed=1):
    c = CONFIGS[cfg]
    n = max(100, int(c["n_agents"] * scale))
    L = max(20, int(c["n_other_locs"] * scale))
    return make_snapshot(n, L, seed=seed, model_seed=0x5EED0000, pop_seed=0x5EED0000 + cfg,
                         quarantine_policy=c.get("quarantine_policy", 0), testing=c.get("testing", False))


def batch_sizes(n_replicas=64, lo=250_000, hi=2_000_000, seed=0x5EED0004, k_lo=1e-4, k_hi=1e-3):
    """C4: agent counts log-uniform on [lo, hi], k log-uniform on [k_lo, k_hi]."""
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(math.log(lo), math.log(hi), n_replicas)).astype(np.int64)
    k = np.exp(rng.uniform(math.log(k_lo), math.log(k_hi), n_replicas))
    seeds = rng.integers(1, 2**63 - 1, n_replicas, dtype=np.int64).astype(np.uint64)
    return n, k, seeds
