"""Non-COVID hospitalization and death (Simulation::otherDisease,
include/simulation.h:169-423).

CPU: the oracle's rates against the reference's tables (hospitalization by
kind, sex and age group; death at the end of a stay), the stay lengths
against the geometric law with the truncated average, the yearly
occupancy multipliers and the daily-target multiplier with both
dueWithCOVID counts, and the agents that draw nothing.  The reference's
function is a member of its Simulation template and draws from per-thread
generators, so the oracle is pinned to the reference through these
distributions and through the tables it shares with the library.

GPU: the library against the oracle over several days, bit for bit, with
one and with two replicas.
"""
import functools

import numpy as np
import pytest

from oracle import binding as ob
from pansim_gb300 import cabi
from tests.helpers import diff_state, small_snapshot, stats_rows

# simulation.h:229-308, by [kind][outcome][sex 0 = F, 1 = M][age group]
HOSP = {
    (0, 1): [0.00017785, 0.000118567, 0.000614453, 0.003174864, 0.001016573, 0.0011019, 0.000926381],
    (0, 0): [9.52062E-05, 6.34708E-05, 0.000328928, 0.000986754, 0.00044981, 0.000623826, 0.000855563],
    (1, 1): [0.000364207, 0.000242805, 0.001240249, 0.006390329, 0.002081773, 0.002256508, 0.001897075],
    (1, 0): [9.97603E-05, 6.65068E-05, 0.000335, 0.000999373, 0.000471326, 0.000653666, 0.000896488],
    (2, 1): [0.00036181, 0.000241207, 0.001237053, 0.006378891, 0.002068074, 0.002241659, 0.001884591],
    (2, 0): [9.84773E-05, 6.56515E-05, 0.000333289, 0.000995818, 0.000465264, 0.000645259, 0.000884959],
}
DEATH = {
    (0, 1): [0.006333678, 0.004222452, 0.008444904, 0.030227275, 0.036202732, 0.03924143, 0.032990764],
    (0, 0): [0.003390532, 0.002260355, 0.00452071, 0.009394699, 0.016018856, 0.022216016, 0.030468759],
    (1, 1): [0.002751133, 0.001834089, 0.003668178, 0.013129695, 0.015725228, 0.017045135, 0.014330059],
    (1, 0): [0.001472731, 0.000981821, 0.001963642, 0.004080736, 0.006958043, 0.009649877, 0.013234587],
    (2, 1): [0.012211473, 0.008140982, 0.016281963, 0.058278861, 0.069799674, 0.075658351, 0.063606928],
    (2, 0): [0.006537022, 0.004358015, 0.008716029, 0.018113189, 0.030884712, 0.042832973, 0.058744446],
}
AGES = [2, 10, 20, 45, 65, 75, 85]       # one age in each group 0-4 ... 80+
PRECOND = [0, 2, 4]                      # general, cardiovascular, pulmonary
AVG_DAYS = [5, 2, 5]                     # (unsigned) 5.55, 2.78, 5.24
NONCOVID_DEAD = 9


@functools.lru_cache(maxsize=4)
def _base_snapshot(n, locs):
    return small_snapshot(n=n, locs=locs, initial_infected_frac=0.0)


def cell_snapshot(per_cell):
    """Susceptible agents spread evenly over kind x sex x age group (42 cells)."""
    n = per_cell * 42
    snap = _base_snapshot(n, max(n // 4, 100)).copy()
    a = snap.agents
    idx = np.arange(n)
    cell = idx % 42
    a["precond"][:] = np.array(PRECOND, np.uint8)[cell // 14]
    a["sex"][:] = (cell // 7) % 2
    a["age"][:] = np.array(AGES, np.uint8)[cell % 7]
    a["state"][:] = 0
    a["st_hospitalized_ts"][:] = 0
    a["st_hospitalized_until"][:] = 0
    return snap, cell


def sigma_bound(k, n, p, z=5.0):
    return abs(k - n * p) <= z * np.sqrt(max(n * p * (1 - p), 1.0))


def run_oracle(snap, t, od):
    o = ob.Oracle(snap)
    o.other_disease_init(od)
    o.other_disease(t)
    return o


def test_hospitalization_rates_and_stay_lengths():
    per = 6000
    snap, cell = cell_snapshot(per)
    spd = snap.steps_per_day
    day = 3
    t = day * spd
    # a target of 4.8M with nobody in states 6..8: probabilityMul = 100
    od = cabi.other_disease_options(total_hospitalizations=[4_800_000] * 10)
    run_oracle(snap, t, od)
    a = snap.agents
    hosp = a["st_hospitalized_until"] > 0
    assert (a["st_hospitalized_ts"][hosp] == t).all()
    for c in range(42):
        kind, sex, ag = c // 14, (c // 7) % 2, c % 7
        p = HOSP[(kind, sex)][ag] * 100.0
        k = int(hosp[cell == c].sum())
        assert sigma_bound(k, per, p), (kind, sex, ag, k, per * p)
    # lengths: max(1, failures before the first success), p = 1 / avg, in whole days
    lens = (a["st_hospitalized_until"][hosp] - t)
    assert (lens % spd == 0).all() and (lens >= spd).all()
    days = lens // spd
    kinds = (cell[hosp] // 14)
    for kind in range(3):
        p = 1.0 / AVG_DAYS[kind]
        d = days[kinds == kind].astype(np.float64)
        mean = (1 - p) / p + p          # E[max(1, G)]
        var = (1 - p) / p ** 2          # Var[G] bounds Var[max(1, G)]
        assert abs(d.mean() - mean) < 5 * np.sqrt(var / len(d)), (kind, d.mean(), mean)
    # nobody died: the sudden-death draw never applies
    assert (a["state"] == 0).all()


def test_deaths_at_the_end_of_a_stay():
    per = 8000
    snap, cell = cell_snapshot(per)
    spd = snap.steps_per_day
    t = 40 * spd
    a = snap.agents
    a["st_hospitalized_ts"][:] = t - 4 * spd
    a["st_hospitalized_until"][:] = t
    run_oracle(snap, t, cabi.other_disease_options())
    dead = a["state"] == NONCOVID_DEAD
    assert (a["days"][dead] == -1).all()
    assert (a["st_worst_state"][dead] == NONCOVID_DEAD).all() and (a["st_worst_ts"][dead] == t).all()
    assert (a["infectious"][dead] == 0).all()
    for c in range(42):
        kind, sex, ag = c // 14, (c // 7) % 2, c % 7
        k = int(dead[cell == c].sum())
        assert sigma_bound(k, per, DEATH[(kind, sex)][ag]), (kind, sex, ag, k)
    # survivors go on to the hospitalization draw: some are admitted again
    again = (~dead) & (a["st_hospitalized_ts"] == t)
    assert again.any()


@pytest.mark.parametrize("day,mult", [(0, 0.82), (99, 0.82), (150, 0.67), (600, 0.9), (1000, 0.9), (1500, 0.9)])
def test_yearly_occupancy_multipliers(day, mult):
    """General, male, 30-59: p = 0.003174864 times the multiplier of the day
    (days 99, 464, 829, 1194 start the next multiplier; the reference reads
    past its tables after day 1194, where the last one is kept here)."""
    n = 400_000
    snap = _base_snapshot(n, 1000).copy()
    a = snap.agents
    a["precond"][:] = 0
    a["sex"][:] = 1
    a["age"][:] = 45
    a["state"][:] = 0
    a["st_hospitalized_ts"][:] = 0
    a["st_hospitalized_until"][:] = 0
    t = day * snap.steps_per_day
    run_oracle(snap, t, cabi.other_disease_options())
    k = int((a["st_hospitalized_until"] > t).sum())
    assert sigma_bound(k, n, 0.003174864 * mult, z=4.0), (day, k, n * 0.003174864 * mult)


@pytest.mark.parametrize("due_with_covid", [0, 1])
def test_daily_target_counts_agents_in_hospital_with_covid(due_with_covid):
    """probabilityMul = max(0, target - with_covid * 9730000/179500) / 48000:
    enough agents in hospital with COVID bring it to 0, and the yearly
    multiplier applies again."""
    per = 3000
    snap, cell = cell_snapshot(per)
    a = snap.agents
    spd = snap.steps_per_day
    t = 5 * spd
    target = 480_000  # 10x the tables with nobody counted
    hosp_type = int(snap.params["hospital_type"])
    # 9000 counted agents: 480000 - 9000 * 9730000/179500 < 0, so the
    # multiplier is 0 and the yearly one (0.82 on day 5) applies
    covid = np.arange(9000) * 14 + 3
    if due_with_covid == 0:
        a["state"][covid] = 6                       # I5_h
    else:
        hospitals = np.flatnonzero(snap.locs["type"] == hosp_type)
        a["state"][covid] = 2                       # infected, WB W
        a["location"][covid] = hospitals[0]
    od = cabi.other_disease_options(due_with_covid=due_with_covid, total_hospitalizations=[target] * 10)
    free = np.ones(len(cell), bool)
    free[covid] = False
    rate = {c: HOSP[(c // 14, (c // 7) % 2)][c % 7] for c in range(42)}
    n_free = {c: int((cell[free] == c).sum()) for c in range(42)}
    s2 = snap.copy()
    run_oracle(s2, t, od)
    k = int((s2.agents["st_hospitalized_until"][free] > t).sum())
    exp = sum(rate[c] * 0.82 * n_free[c] for c in range(42))
    assert abs(k - exp) < 5 * np.sqrt(exp), (k, exp)
    # nobody counted: the target's multiplier, 10
    s3 = snap.copy()
    s3.agents["state"][covid] = 0
    run_oracle(s3, t, od)
    k3 = int((s3.agents["st_hospitalized_until"][free] > t).sum())
    exp3 = sum(rate[c] * 10.0 * n_free[c] for c in range(42))
    assert abs(k3 - exp3) < 5 * np.sqrt(exp3), (k3, exp3)


def test_dead_severe_and_hospitalized_agents_draw_nothing():
    snap, cell = cell_snapshot(1000)
    a = snap.agents
    spd = snap.steps_per_day
    t = 7 * spd
    n = len(cell)
    kind = np.arange(n) % 3
    a["state"][kind == 0] = NONCOVID_DEAD            # WB D
    a["state"][kind == 1] = 7                        # I6_h, WB S
    a["st_hospitalized_ts"][kind == 2] = t - spd     # in hospital until t + 2 days
    a["st_hospitalized_until"][kind == 2] = t + 2 * spd
    before = snap.copy()
    run_oracle(snap, t, cabi.other_disease_options(total_hospitalizations=[48000 * 100] * 10))
    assert diff_state(before, snap) == []


@pytest.mark.gpu
@pytest.mark.parametrize("replicas,targets,due", [(1, None, 0), (1, [48000 * 40] * 30, 0), (2, [48000 * 40] * 30, 1)])
def test_other_disease_bit_exact(gpu_lib, replicas, targets, due):
    from pansim_gb300 import snapshot as sn
    from pansim_gb300.native import GpuSim
    parts = [small_snapshot(n=9000, locs=2200, seed=7 + q, initial_infected_frac=0.03) for q in range(replicas)]
    snap = parts[0] if replicas == 1 else sn.concat(parts, seeds=[11, 12], ks=[3.74e-4, 5e-4])
    rng = np.random.default_rng(1)
    a = snap.agents
    n = len(a["age"])
    a["precond"][:] = rng.choice([0, 1, 2, 3, 4], n)
    # stays ending on the simulated midnights: deaths at their end
    spd = snap.steps_per_day
    end = rng.random(n) < 0.05
    a["st_hospitalized_ts"][end] = 2 * spd
    a["st_hospitalized_until"][end] = rng.integers(3, 7, end.sum()) * spd
    s_cpu, s_gpu = snap, snap.copy()
    o = ob.Oracle(s_cpu)
    g = GpuSim(s_gpu)
    od = cabi.other_disease_options(due_with_covid=due, total_hospitalizations=targets)
    o.other_disease_init(od)
    g.other_disease_init(od)
    for d in range(3, 8):
        assert stats_rows(o.run_day(d)) == stats_rows(g.run_day(d)), d
        g.download()
        assert diff_state(s_cpu, s_gpu) == [], d
    assert (s_cpu.agents["state"] == NONCOVID_DEAD).any()
    assert (s_cpu.agents["st_hospitalized_ts"] >= 3 * spd).any()
