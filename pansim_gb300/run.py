"""Command-line runner: a seeded synthetic population stepped on the GPU.

  python -m pansim_gb300.run --agents 2000000 --locs 500000 --days 2
  python -m pansim_gb300.run --agents 2000000 --locs 500000 --steps 20   # individual psim_step launches

Prints the daily statistics row (the reference's TSV columns,
simulation.h:754) and the wall time.  --steps runs the timesteps of day 0
one psim_step call at a time (no graph), which is the form used for kernel
profiles.  --timeline FILE runs the days with the kernels' timeline stamps
and writes, per day and step, the step kernel's span, the rebuild's listing
and slots, the draws, the queue, the decisions and the time since the
previous kernel (us, tab-separated), with the day's counters.
"""
import argparse
import sys
import time

from . import native, synth


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--agents", type=int, default=100_000)
    ap.add_argument("--locs", type=int, default=20_000)
    ap.add_argument("--days", type=int, default=0)
    ap.add_argument("--steps", type=int, default=0)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--pop-seed", type=int, default=0x5EED0002)
    ap.add_argument("--quarantine-policy", type=int, default=0)
    ap.add_argument("--testing", action="store_true")
    ap.add_argument("--quiet", action="store_true")
    ap.add_argument("--tune", action="store_true", help="set the tuning below (else the context's default)")
    ap.add_argument("--agg-slot", type=int, default=0)
    ap.add_argument("--blocks-per-sm", type=int, default=4)
    ap.add_argument("--scan-items", type=int, default=4)
    ap.add_argument("--scan-mode", type=int, default=3)
    ap.add_argument("--timeline", default="")
    a = ap.parse_args(argv)
    snap = synth.make_snapshot(a.agents, a.locs, seed=a.seed, pop_seed=a.pop_seed,
                               quarantine_policy=a.quarantine_policy, testing=a.testing)
    g = native.GpuSim(snap)
    if a.tune:
        g.set_tuning(agg_count=0, agg_slot=a.agg_slot, blocks_per_sm=a.blocks_per_sm, variant=3,
                     scan_items=a.scan_items, scan_mode=a.scan_mode)
    tl_out = open(a.timeline, "w") if a.timeline else None
    if tl_out:
        g.set_profiling(True)
        tl_out.write("day\tstep\tspan_us\treb_listing_us\treb_slots_us\tdraw_us\tqueue_us\tdecide_us\tgap_us\n")
    t0 = time.perf_counter()
    for d in range(a.days):
        st = g.run_day(d)
        if not a.quiet:
            print("day %d\t" % d + "\t".join(str(x) for x in list(st[0].v)[: st[0].n]))
        if tl_out:
            for s, row in enumerate(g.day_timeline()):
                tl_out.write("%d\t%d\t" % (d, s) + "\t".join("%.2f" % x for x in row) + "\n")
            tl_out.write("# day %d: graph %.3f ms, counts %s\n" % (d, g.last_day_ms(),
                                                                     " ".join(str(int(x)) for x in g.day_counts())))
    if tl_out:
        tl_out.close()
    if a.steps:
        g.midnight(a.days * 144)
        for s in range(a.steps):
            g.step(a.days * 144 + s)
    dt = time.perf_counter() - t0
    print("agents %d locations %d days %d steps %d wall %.3f s launches %d" % (
        snap.n_agents, snap.n_locations, a.days, a.steps, dt, g.launch_count()))
    return 0


if __name__ == "__main__":
    sys.exit(main())
