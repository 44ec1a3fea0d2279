"""GPU parity against the CPU oracle through the C ABI (gpu).

Bit-exact: movement, location assignment, CSR (canonical order), per-location
counts, fixed-point sums and hazards, infection outcomes, state transitions,
daily plan, testing, statistics.  Hazards additionally within 1e-5 relative
of the oracle's FP64 evaluation.
"""
import numpy as np
import pytest

from oracle import binding as ob
from pansim_gb300.native import GpuSim
from tests.helpers import diff_state, small_snapshot, stats_rows

pytestmark = pytest.mark.gpu


def _pair(**kw):
    s_cpu = small_snapshot(**kw)
    s_gpu = s_cpu.copy()
    return s_cpu, s_gpu, ob.Oracle(s_cpu), GpuSim(s_gpu)


def test_initial_csr(gpu_lib):
    s_cpu, s_gpu, o, g = _pair(n=8000, locs=2000)
    off_o, ag_o = o.csr()
    off_g, ag_g = g.csr(canonical=True)
    assert np.array_equal(off_o, off_g)
    assert np.array_equal(ag_o, ag_g)


def test_one_day_phase_by_phase(gpu_lib):
    s_cpu, s_gpu, o, g = _pair(n=20000, locs=5000, initial_infected_frac=0.02)
    st_o = o.midnight(0)
    st_g = g.midnight(0)
    assert stats_rows(st_o) == stats_rows(st_g)
    for t in range(144):
        o.movement(t)
        g.movement(t)
        o.regroup()
        g.regroup()
        out = o.infect(t)
        g.infect(t)
        if t % 24 == 5:
            g.download()
            assert diff_state(s_cpu, s_gpu) == [], t
            off_o, ag_o = o.csr()
            off_g, ag_g = g.csr(canonical=True)
            assert np.array_equal(off_o, off_g), t
            assert np.array_equal(ag_o, ag_g), t
            hz = g.hazard()
            assert np.array_equal(hz, out["hazard"]), t
            nz = out["r64"] > 0
            if nz.any():
                rel = np.abs(hz[nz].astype(np.float64) - out["r64"][nz]) / out["r64"][nz]
                assert rel.max() < 1e-5
    g.download()
    assert diff_state(s_cpu, s_gpu) == []
    # next midnight: progression + stats + plan
    o.progress(144)
    g.progress(144)
    g.download()
    assert diff_state(s_cpu, s_gpu) == []
    assert stats_rows(o.stats(144)) == stats_rows(g.stats(144))
    o.plan(144)
    g.plan(144)
    g.download()
    assert diff_state(s_cpu, s_gpu) == []


def test_week_graph_bit_exact(gpu_lib):
    s_cpu, s_gpu, o, g = _pair(n=30000, locs=7500, initial_infected_frac=0.01)
    for d in range(7):
        ro = stats_rows(o.run_day(d))
        rg = stats_rows(g.run_day(d))
        assert ro == rg, d
    g.download()
    assert diff_state(s_cpu, s_gpu) == []


def test_quarantine_testing_policies_bit_exact(gpu_lib):
    """quarantinePolicy 3, DetailedTesting with high probabilities."""
    s_cpu, s_gpu, o, g = _pair(n=20000, locs=5000, initial_infected_frac=0.02, quarantine_policy=3, testing=True)
    for s in (s_cpu, s_gpu):
        s.params.update(t_random=0.02, t_home=0.3, t_work=0.1, t_school=0.1, t_hospital=0.2)
    o.set_params()
    g.set_params()
    for d in range(6):
        ro = stats_rows(o.run_day(d))
        rg = stats_rows(g.run_day(d))
        assert ro == rg, d
    g.download()
    assert diff_state(s_cpu, s_gpu) == []
    assert s_cpu.agents["quarantined"].sum() > 0
    assert (s_cpu.agents["last_test"] != 0xFFFFFFFF).sum() > 0


def test_curfew_and_closures_bit_exact(gpu_lib):
    s_cpu, s_gpu, o, g = _pair(n=15000, locs=4000, initial_infected_frac=0.02)
    rng = np.random.default_rng(3)
    closed = rng.random(s_cpu.n_locations) < 0.2
    for s in (s_cpu, s_gpu):
        s.params.update(enable_curfew=1, curfew_begin=120, curfew_end=30, school_age_restriction=12)
        s.locs["open"][closed] = 0
    o = ob.Oracle(s_cpu)
    g = GpuSim(s_gpu)
    for d in range(3):
        assert stats_rows(o.run_day(d)) == stats_rows(g.run_day(d)), d
    g.download()
    assert diff_state(s_cpu, s_gpu) == []


def test_replicas_batch_equals_single(gpu_lib):
    """A replica gives the same trajectory alone and inside a batch."""
    from pansim_gb300 import snapshot as snp, synth
    parts = [synth.make_snapshot(n, n // 4, seed=1, pop_seed=100 + i, initial_infected_frac=0.01)
             for i, n in enumerate([6000, 9000, 4000])]
    seeds = [11, 22, 33]
    ks = [2e-4, 5e-4, 9e-4]
    batch = snp.concat(parts, seeds, ks)
    gb = GpuSim(batch)
    singles = []
    for i, p in enumerate(parts):
        q = p.copy()
        q.params["seed"] = seeds[i]
        q.params["k"] = ks[i]
        q.reps["seed"][:] = seeds[i]
        q.reps["k"][:] = ks[i]
        singles.append((q, GpuSim(q)))
    for d in range(3):
        rb = stats_rows(gb.run_day(d))
        for i, (q, gs) in enumerate(singles):
            assert rb[i] == stats_rows(gs.run_day(d))[0], (d, i)
    # the oracle agrees on the batch too
    batch2 = snp.concat(parts, seeds, ks)
    ob_ = ob.Oracle(batch2)
    gb2 = GpuSim(batch2.copy())
    for d in range(2):
        assert stats_rows(ob_.run_day(d)) == stats_rows(gb2.run_day(d))


def test_location_type_ids_beyond_the_packed_lists(gpu_lib):
    """The per-agent location lists go to the device in 4-byte entries when
    every type id is below 64 and every location below 2^26, else in 8-byte
    entries: the shop type renumbered 7 -> 100 wherever it appears takes the
    8-byte form and gives the oracle's days bit for bit."""
    s_cpu = small_snapshot(n=12000, locs=3000, initial_infected_frac=0.02)
    shop, new = int(s_cpu.params["public_type"]), 100
    for arr in (s_cpu.locs["type"], s_cpu.agents["poss_type"], s_cpu.model["ev_loc_type"]):
        assert (arr == shop).any()
        arr[arr == shop] = new
    s_cpu.params["public_type"] = new
    s_gpu = s_cpu.copy()
    o, g = ob.Oracle(s_cpu), GpuSim(s_gpu)
    for d in range(3):
        assert stats_rows(o.run_day(d)) == stats_rows(g.run_day(d)), d
    g.download()
    assert diff_state(s_cpu, s_gpu) == []


def test_bounded_wait_reports_error_and_context_survives(gpu_lib):
    s = small_snapshot(n=2000, locs=500)
    g = GpuSim(s)
    rc = g.bounded_wait_selftest(1 << 16)
    assert rc == -5  # PSIM_ERR_DEVICE
    assert "bounded wait expired" in g.last_error()
    g.run_day(0)  # still usable


@pytest.mark.parametrize("tuning", [dict(agg_count=0, agg_slot=0, blocks_per_sm=0),
                                    dict(agg_count=1, agg_slot=1, blocks_per_sm=3),
                                    dict(agg_count=0, agg_slot=1, blocks_per_sm=16),
                                    dict(agg_count=0, agg_slot=0, blocks_per_sm=5),
                                    dict(agg_count=0, agg_slot=0, blocks_per_sm=0, scan_items=2, scan_mode=1),
                                    dict(agg_count=0, agg_slot=1, blocks_per_sm=3, scan_items=4, scan_mode=0),
                                    dict(agg_count=0, agg_slot=0, blocks_per_sm=4, scan_items=2, scan_mode=1),
                                    dict(agg_count=0, agg_slot=0, blocks_per_sm=0, scan_items=8, scan_mode=1),
                                    dict(agg_count=0, agg_slot=0, blocks_per_sm=4, scan_items=4, scan_mode=2),
                                    dict(agg_count=0, agg_slot=1, blocks_per_sm=0, scan_items=8, scan_mode=2),
                                    dict(agg_count=0, agg_slot=0, blocks_per_sm=4, scan_items=8, scan_mode=0),
                                    dict(agg_count=0, agg_slot=0, blocks_per_sm=8, scan_items=4, scan_mode=3),
                                    dict(agg_count=0, agg_slot=1, blocks_per_sm=0, scan_items=8, scan_mode=3),
                                    dict(agg_count=0, agg_slot=0, blocks_per_sm=8, scan_items=2, scan_mode=3),
                                    dict(agg_count=0, agg_slot=0, blocks_per_sm=0, variant=4),
                                    dict(agg_count=0, agg_slot=1, blocks_per_sm=2, variant=4)])
def test_tuning_choices_do_not_change_results(gpu_lib, tuning):
    """Every tuning against the oracle over three days: statistics, state and
    the agent list at the end of each day.  Most steps of a day move nobody
    and keep the agent list of the step before (incremental CSR); the
    canonical read also reorders the kept segments in place."""
    s_cpu, s_gpu, o, g = _pair(n=12000, locs=3000, initial_infected_frac=0.02)
    g.set_tuning(**tuning)
    for d in range(3):
        assert stats_rows(o.run_day(d)) == stats_rows(g.run_day(d)), (d, tuning)
        off_o, ag_o = o.csr()
        off_g, ag_g = g.csr(canonical=True)
        assert np.array_equal(off_o, off_g) and np.array_equal(ag_o, ag_g), (d, tuning)
    g.download()
    assert diff_state(s_cpu, s_gpu) == []


def test_profiled_graph_same_results_and_kernel_times(gpu_lib):
    s_cpu, s_gpu, o, g = _pair(n=12000, locs=3000, initial_infected_frac=0.02)
    g.set_profiling(True)
    for d in range(2):
        assert stats_rows(o.run_day(d)) == stats_rows(g.run_day(d)), d
        ms = g.day_kernel_ms()
        assert (ms[:4] > 0).all() and ms[4] >= 0, ms
        assert ms.sum() <= g.last_day_ms() * 1.01, (ms, g.last_day_ms())
        entries, hazard, movers, queues, rebuilds, listed_locs, listed_agents = g.day_counts()
        assert entries > 0 and 0 < hazard <= entries and movers > 0 and 0 < queues < 143 and 0 < rebuilds <= 144
        # the rebuilds list the agents at locations with a nonzero sum, a
        # part of all; every step draws the entries of the last rebuild
        assert 0 < listed_locs <= listed_agents < rebuilds * 12000 and entries >= listed_agents
        # per step: spans, the steps that rebuilt and queued, the gaps
        tl = g.day_timeline()
        assert tl.shape == (144, 7) and (tl >= 0).all()
        assert (tl[:, 0] > 0).all()
        assert rebuilds - 2 <= (tl[:, 1:3].sum(axis=1) > 0).sum() <= rebuilds
        assert queues - 2 <= (tl[:, 5] > 0).sum() <= queues
        assert (tl[:, 0].sum() + tl[:, 6].sum()) * 1e-3 <= g.last_day_ms() * 1.01
    g.set_profiling(False)
    assert stats_rows(o.run_day(2)) == stats_rows(g.run_day(2))
    g.download()
    assert diff_state(s_cpu, s_gpu) == []


@pytest.mark.parametrize("n,locs,frac", [(1, 4, 1.0), (3, 5, 0.0), (257, 64, 0.5), (5000, 1200, 0.0)])
def test_tiny_ragged_and_uninfected_populations(gpu_lib, n, locs, frac):
    """A single agent, a few agents, sizes off the warp/block multiples, and
    days with no infectious agent at all (empty hazard masks)."""
    s_cpu, s_gpu, o, g = _pair(n=n, locs=locs, initial_infected_frac=frac)
    for d in range(2):
        assert stats_rows(o.run_day(d)) == stats_rows(g.run_day(d)), d
    g.download()
    assert diff_state(s_cpu, s_gpu) == []
    off_o, ag_o = o.csr()
    off_g, ag_g = g.csr(canonical=True)
    assert np.array_equal(off_o, off_g) and np.array_equal(ag_o, ag_g)


def test_uneven_tiny_replicas_match_single_runs(gpu_lib):
    from pansim_gb300 import snapshot as snp
    from tests.helpers import small_snapshot
    parts = [small_snapshot(n=n, locs=max(4, n // 4), seed=10 + i, initial_infected_frac=0.2)
             for i, n in enumerate([1, 33, 700])]
    batch = snp.concat([p.copy() for p in parts], [10, 11, 12], [3.74e-4] * 3)
    gb = GpuSim(batch)
    singles = [GpuSim(p.copy()) for p in parts]
    for d in range(2):
        rows_b = stats_rows(gb.run_day(d))
        for r, gs in enumerate(singles):
            assert stats_rows(gs.run_day(d))[0] == rows_b[r], (d, r)


def test_restored_day_rebuilds_the_agent_list(gpu_lib):
    """A day replayed from a checkpoint (as the autotuner and the adjoint do)
    gives the oracle's state, statistics and agent list: the restore forces
    the next step to rebuild the CSR, which the checkpoint does not hold."""
    s_cpu, s_gpu, o, g = _pair(n=12000, locs=3000, initial_infected_frac=0.02)
    for d in range(2):
        assert stats_rows(o.run_day(d)) == stats_rows(g.run_day(d)), d
    g.checkpoint_save(7)
    g.run_day(2)
    g.run_day(3)
    g.checkpoint_restore(7)
    assert stats_rows(o.run_day(2)) == stats_rows(g.run_day(2))
    g.download()
    assert diff_state(s_cpu, s_gpu) == []
    off_o, ag_o = o.csr()
    off_g, ag_g = g.csr(canonical=True)
    assert np.array_equal(off_o, off_g) and np.array_equal(ag_o, ag_g)
    g.checkpoint_drop(7)


def test_timestep_timing_leaves_a_consistent_agent_list(gpu_lib):
    """psim_time_step_kernels (one timestep and the decisions of the next, the
    step kernels timed) runs the rebuild, draw, queue and decision kernels in
    sequence; afterwards the agent list is the stable grouping of the agents'
    current locations."""
    for agg in (0, 1):
        s_gpu = small_snapshot(n=12000, locs=3000, initial_infected_frac=0.02)
        g = GpuSim(s_gpu)
        g.set_tuning(agg_count=0, agg_slot=agg, blocks_per_sm=4, variant=3, scan_items=4, scan_mode=3)
        g.run_day(0)
        spd = s_gpu.steps_per_day
        for step in (40, 47, 48):
            ms = g.time_step_kernels(spd + step)
            assert (np.asarray(ms) > 0).all(), ms
            g.download()
            loc = s_gpu.agents["location"]
            off, ag = g.csr(canonical=True)
            order = np.argsort(loc, kind="stable").astype(np.uint32)
            counts = np.bincount(loc, minlength=s_gpu.n_locations)
            assert np.array_equal(off, np.concatenate([[0], np.cumsum(counts)]).astype(np.uint32))
            assert np.array_equal(ag, order)


@pytest.mark.parametrize("time_step", [96, 160])
def test_odd_steps_per_day(gpu_lib, time_step):
    """Days of an odd number of timesteps (15 of 96 minutes, 9 of 160): the
    step kernel reads its two copies of the sums by step parity, so a day
    ends on the second copy and the next day starts afresh; every row, the
    end state and the canonical agent list equal the oracle's."""
    from pansim_gb300.native import GpuSim
    s_cpu = small_snapshot(n=12000, locs=3000, initial_infected_frac=0.02)
    s_cpu.params["time_step"] = time_step
    assert (1440 // time_step) % 2 == 1
    s_gpu = s_cpu.copy()
    o, g = ob.Oracle(s_cpu), GpuSim(s_gpu)
    for d in range(3):
        assert stats_rows(o.run_day(d)) == stats_rows(g.run_day(d)), d
    g.download()
    assert diff_state(s_cpu, s_gpu) == []
    off_o, ag_o = o.csr()
    off_g, ag_g = g.csr(canonical=True)
    assert np.array_equal(off_o, off_g) and np.array_equal(ag_o, ag_g)
