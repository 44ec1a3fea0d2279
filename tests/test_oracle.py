"""The CPU oracle on its own (CPU): invariants of each phase."""
import numpy as np

from oracle import binding as ob
from tests.helpers import small_snapshot, stats_rows


def test_generator_is_valid_and_seeded():
    a = small_snapshot(5000, 1200)
    b = small_snapshot(5000, 1200)
    a.validate()
    for k in a.agents:
        assert np.array_equal(a.agents[k], b.agents[k]), k
    assert a.n_locations == int(a.params["cemetery_loc"]) + 1


def test_csr_is_stable_grouping():
    s = small_snapshot(4000, 1000)
    o = ob.Oracle(s)
    for t in range(0, 60):
        o.movement(t)
    o.regroup()
    off, ag = o.csr()
    loc = s.agents["location"]
    assert off[0] == 0 and off[-1] == s.n_agents
    assert np.array_equal(np.diff(off), np.bincount(loc, minlength=s.n_locations))
    # thrust::stable_sort_by_key equivalent
    assert np.array_equal(ag, np.argsort(loc, kind="stable"))


def test_oracle_deterministic():
    r = []
    for _ in range(2):
        s = small_snapshot(3000, 800)
        o = ob.Oracle(s)
        rows = [stats_rows(o.run_day(d)) for d in range(3)]
        r.append((rows, s.agents["state"].copy(), s.agents["location"].copy()))
    assert r[0][0] == r[1][0]
    assert np.array_equal(r[0][1], r[1][1]) and np.array_equal(r[0][2], r[1][2])


def test_infection_hazard_within_fp64_tolerance():
    s = small_snapshot(6000, 1500, initial_infected_frac=0.05)
    o = ob.Oracle(s)
    o.run_day(0)
    o.movement(144)
    o.regroup()
    out = o.infect(144)
    h, r64 = out["hazard"].astype(np.float64), out["r64"]
    nz = r64 > 0
    assert nz.sum() > 50
    rel = np.abs(h[nz] - r64[nz]) / r64[nz]
    assert rel.max() < 1e-5, rel.max()
    # fixed-point sums are the exact sums of the FP32 values
    assert np.allclose(out["fix"] * 2.0 ** -40, out["sum64"], rtol=1e-12, atol=1e-12)


def test_progression_follows_tables():
    """One day of DynamicPPState::update on many infected agents: the
    empirical transition frequencies match the row of the table."""
    s = small_snapshot(40000, 5000, initial_infected_frac=0.9)
    st0 = s.agents["state"].copy()
    band = s.agents["prog_id"].copy()
    o = ob.Oracle(s)
    o.progress(144)
    m = s.model
    S = int(m["n_states"])
    st1 = s.agents["state"]
    sel = (st0 == 2) & (band == 3)
    ti = 3 * S + 2
    b, n = int(m["tr_neu_begin"][ti]), int(m["tr_neu_count"][ti])
    nxt, ch = m["tr_next"][b:b + n], m["tr_chance"][b:b + n]
    cnt = np.array([(st1[sel] == x).sum() for x in nxt], float)
    tot = sel.sum()
    assert cnt.sum() == tot
    se = np.sqrt(ch * (1 - ch) / tot)
    assert np.all(np.abs(cnt / tot - ch) < 5 * se + 1e-3), (cnt / tot, ch)


def test_stats_row_layout():
    s = small_snapshot(3000, 800)
    o = ob.Oracle(s)
    st = o.run_day(0)[0]
    S = int(s.model["n_states"])
    row = list(st.v)[: st.n]
    assert sum(row[:S]) == s.n_agents
    assert st.n == S + 7 + 1 + 1 + 1 + 4 + 1 + 2 + 1 + 2
