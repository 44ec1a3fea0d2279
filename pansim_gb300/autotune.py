"""Autotuner of the per-step kernels.

Times each candidate tuning (warp aggregation of the count reductions and of
the CSR slot atomics, blocks per SM of the per-agent kernels) on the live
workload with CUDA events (psim_time_step_kernels: scan + fused
scatter/draw/movement, as the day graph runs them) and keeps the fastest.
The choice depends on the device and on the population (location sizes,
household structure), so it is made per context.
"""
import itertools

import numpy as np

DEFAULT_GRID = [0, 4, 8, 16]


def candidates(grid=None):
    """variant: register cap of the fused kernel (64 / 40 / 32 registers) or
    3 = hot/cold split;
    blocks_per_sm 0 = one occupancy wave of that variant."""
    for variant, agg_count, agg_slot, bps in itertools.product([0, 1, 2, 3], [1, 0], [1, 0], grid or DEFAULT_GRID):
        yield dict(agg_count=agg_count, agg_slot=agg_slot, blocks_per_sm=bps, variant=variant)


TUNE_SLOT = 1 << 16


def autotune(sim, day, reps=3, grid=None, verbose=False, keep_state=True):
    """Tries the candidates on steps of `day`; returns (best tuning, table of
    (tuning, step ms)).  With keep_state the simulation state is saved to a
    checkpoint first and restored afterwards, so tuning leaves no trace."""
    if keep_state:
        sim.checkpoint_save(TUNE_SLOT)
    table = []
    t = day * sim.snap.steps_per_day
    for cand in candidates(grid):
        sim.set_tuning(**cand)
        ms = []
        for _ in range(reps):
            if t % sim.snap.steps_per_day + 1 >= sim.snap.steps_per_day:
                t += 2
            k = sim.time_step_kernels(t)
            ms.append(float(k[1] + k[2]))
            t += 2
        table.append((cand, float(np.median(ms))))
        if verbose:
            print("tune", cand, "%.2f us" % (1000 * table[-1][1]))
    best = min(table, key=lambda x: x[1])[0]
    sim.set_tuning(**best)
    if keep_state:
        sim.checkpoint_restore(TUNE_SLOT)
        sim.checkpoint_drop(TUNE_SLOT)
    return best, table
