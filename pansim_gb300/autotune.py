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
    """variant: register cap of the fused kernel (64 / 40 / 32 registers);
    blocks_per_sm 0 = one occupancy wave of that variant."""
    for variant, agg_count, agg_slot, bps in itertools.product([0, 1, 2], [1, 0], [1, 0], grid or DEFAULT_GRID):
        yield dict(agg_count=agg_count, agg_slot=agg_slot, blocks_per_sm=bps, variant=variant)


def autotune(sim, day, reps=3, grid=None, verbose=False):
    """Tries the candidates on the steps of `day` (the state advances by those
    steps); returns (best tuning, table of (tuning, step ms))."""
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
    return best, table
