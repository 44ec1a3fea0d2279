"""GPU parity against the CPU oracle at the benchmark workloads' sizes (gpu).

The small-population tests cover every phase and tuning; these run the
workloads the throughput figures are quoted on, where the paths that only
grow with size are exercised: thousands of scan tiles, work-list segments
holding about a million movers in one step, several grid-stride trips per
thread, and 32-bit offsets of a 20M-agent agent list.

  * 100k agents, 20k non-home locations, 7 days: every daily row, the full
    end state and the canonical agent list;
  * the benchmark's own 2M-agent snapshot (bench.make_snapshot), 2 days:
    rows, full state, canonical agent list;
  * 20M agents, 5M non-home locations, quarantine policy 3, testing, the
    new-cases closure rule and immunization, 2 days (the second midnight
    runs testing, progression and immunization);
  * 8 uneven replicas of the 64-replica ensemble (agents log-uniform on
    250k-2M, own seeds and k), 2 days in one batched context.

Each comparison is bit for bit: agent and location arrays, statistics rows,
location offsets and the agent list in canonical order (ascending agent id
inside a location, thrust::stable_sort_by_key's order, util.cpp:69).
"""
import numpy as np
import pytest

from oracle import binding as ob
from oracle import closures as oc
from pansim_gb300 import closures, immunization, synth
from pansim_gb300 import snapshot as snp
from tests.helpers import diff_state, stats_rows

pytestmark = pytest.mark.gpu


def _compare_state(o, g, s_cpu, s_gpu, where):
    g.download()
    assert diff_state(s_cpu, s_gpu) == [], where
    off_o, ag_o = o.csr()
    off_g, ag_g = g.csr(canonical=True)
    assert np.array_equal(off_o, off_g), where
    assert np.array_equal(ag_o, ag_g), where


def _run_plain(s_cpu, days):
    from pansim_gb300.native import GpuSim
    s_gpu = s_cpu.copy()
    o = ob.Oracle(s_cpu)
    g = GpuSim(s_gpu)
    for d in range(days):
        ro = stats_rows(o.run_day(d))
        rg = stats_rows(g.run_day(d))
        assert ro == rg, d
    _compare_state(o, g, s_cpu, s_gpu, "end of day %d" % (days - 1))
    o.close()
    g.close()


def test_100k_agents_one_week(gpu_lib):
    s = synth.config_snapshot(1)
    assert s.n_agents == 100_000
    _run_plain(s, 7)


def test_bench_2m_snapshot_two_days(gpu_lib):
    import bench
    s = bench.make_snapshot(0)
    assert s.n_agents == 2_000_000 and s.n_locations == 1_299_752
    _run_plain(s, 2)


def _oracle_day(o, eng, day):
    """psim_midnight's order on the oracle: testing, progression,
    immunization, statistics, closure rules, plan; then the day's steps."""
    snap = o.snap
    t0 = day * snap.steps_per_day
    if t0 > 0 and int(snap.params.get("testing_enabled", 0)):
        o.test(t0)
    if t0 > 0:
        o.progress(t0)
    o.immunize(t0)
    st = o.stats(t0)
    eng.midnight(t0, st[0])
    o.plan(t0)
    for s in range(snap.steps_per_day):
        o.step(t0 + s)
    return st


def test_20m_agents_with_policies(gpu_lib):
    from pansim_gb300.native import GpuSim
    s_cpu = synth.config_snapshot(3)
    assert s_cpu.n_agents == 20_000_000
    assert int(s_cpu.params["quarantine_policy"]) == 3 and int(s_cpu.params["testing_enabled"]) == 1
    s_gpu = s_cpu.copy()
    o = ob.Oracle(s_cpu)
    g = GpuSim(s_gpu)
    # new cases above 0.05% of the population close work, schools and shops
    rules = [dict(name="lockdown", conditionType="newCasesFraction", threshold=0.0005, threshold2=0.00025,
                  closeAfter=1, openAfter=7, parameter=0,
                  locationTypesToClose=[synth.WORK, synth.SCHOOL, synth.SHOP])]
    hdr = closures.stats_header(synth.STATE_NAMES)
    eng = oc.OracleClosures(o, rules, hdr)
    g.closures_init(rules, hdr)
    # 50k doses a day in a 6-category order, from the first midnight on
    opt = immunization.options(immunizations_per_week=350_000, immunizationStart=0,
                               immunizationOrder="1,2,3,4,5,6,0,0,0,0", boosterStart="1000",
                               boosters_per_week=[([0], [1.0] * 10)])
    o.immunization_init(opt)
    g.immunization_init(opt)
    vac_col = len(synth.STATE_NAMES) + 9
    vaccinated = 0
    for d in range(2):
        ro = stats_rows(_oracle_day(o, eng, d))
        rg = stats_rows(g.run_day(d))
        assert ro == rg, d
        vaccinated += ro[0][vac_col]
        act_o, open_o = eng.status()
        act_g, open_g = g.closures_status()
        assert np.array_equal(act_o, act_g) and np.array_equal(open_o, open_g), d
    assert vaccinated > 0
    # testing ran at the second midnight and quarantined someone
    assert (s_cpu.agents["st_quarantined_ts"] > 0).any() or (s_cpu.agents["last_test"] > 0).any()
    _compare_state(o, g, s_cpu, s_gpu, "end of day 1")
    o.close()
    g.close()


def test_eight_uneven_replicas_batched(gpu_lib):
    n, ks, seeds = synth.batch_sizes(64)
    pick = [int(x) for x in np.argsort(n)[np.linspace(0, 63, 8).astype(int)]]  # smallest .. largest
    parts = []
    for r in pick:
        p = synth.make_snapshot(int(n[r]), int(n[r]) // 4, seed=int(seeds[r]), pop_seed=0x5EED0004 + r, k=float(ks[r]))
        parts.append(p)
    batch = snp.concat(parts, [int(seeds[r]) for r in pick], [float(ks[r]) for r in pick])
    assert batch.n_replicas == 8
    _run_plain(batch, 2)
