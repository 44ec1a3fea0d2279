"""Autotuner of the step kernel.

Times each candidate tuning (warp aggregation of the agent-list slot
atomics, resident blocks per SM of the persistent step kernel) on the live
workload: every candidate runs the same whole day (the day graph, all its
steps) from the same checkpoint taken after that day's midnight phases,
timed with CUDA events, and the fastest is kept.  Steps at different times
of day differ several-fold in cost (movers, infectious locations), so
candidates are never compared on different steps.  The choice depends on the
device and on the population, so it is made per context.
"""
import itertools

DEFAULT_GRID = [0, 2, 3]
LARGE_AGENTS = 8_000_000


def candidates(grid=None):
    """blocks_per_sm 0 = as many as the step kernel's occupancy allows (the
    library caps every value there: its grid barriers need every block
    resident)."""
    for agg_slot, bps in itertools.product([1, 0], grid or DEFAULT_GRID):
        yield dict(agg_count=0, agg_slot=agg_slot, blocks_per_sm=bps, variant=3, scan_items=4, scan_mode=3)


TUNE_SLOT = 1 << 16


def autotune(sim, day, reps=2, grid=None, verbose=False):
    """Tries the candidates on the steps of `day` (the simulation must be at
    the start of that day); returns (best tuning, table of (tuning, day ms)).
    The simulation state is saved first and restored afterwards, so tuning
    leaves no trace.  Populations above LARGE_AGENTS get a reduced candidate
    set and one repetition (a day there takes a good fraction of a second)."""
    if sim.snap.n_agents > LARGE_AGENTS:
        grid = grid or [0, 2]
        reps = 1
    spd = sim.snap.steps_per_day
    sim.checkpoint_save(TUNE_SLOT)
    # the midnight phases without closure rules, whose host-side state a
    # checkpoint does not hold
    t = day * spd
    if t > 0 and int(sim.snap.params.get("testing_enabled", 0)):
        sim.test(t)
    if t > 0:
        sim.progress(t)
    sim.stats(t)
    sim.plan(t)
    sim.checkpoint_save(TUNE_SLOT + 1)
    table = []
    for cand in candidates(grid):
        sim.set_tuning(**cand)
        ms = []
        for _ in range(reps):
            sim.checkpoint_restore(TUNE_SLOT + 1)
            sim.run_steps(day)
            ms.append(sim.last_day_ms())
        table.append((cand, float(min(ms))))
        if verbose:
            print("tune", cand, "%.3f ms/day" % table[-1][1])
    best = min(table, key=lambda x: x[1])[0]
    sim.set_tuning(**best)
    sim.checkpoint_restore(TUNE_SLOT)
    sim.checkpoint_drop(TUNE_SLOT)
    sim.checkpoint_drop(TUNE_SLOT + 1)
    return best, table
