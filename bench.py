#!/usr/bin/env python3
"""Benchmark of the PanSim per-timestep agent loop on GB300.

Metric: agent-steps/s on the 2M-agent workload (2,000,000 agents, 500,000
non-home locations plus homes, dt = 10 min, FP32 infectiousness, uint32
location ids, seeded synthetic population).  One bench step = one simulated
day: the midnight phases (progression, statistics, daily plan) and the 144
timesteps of movement -> regrouping -> infection, launched as one CUDA graph.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Under torchrun every rank runs its own replica of the workload (replicas only:
the path does not shard a single population), value = all ranks' agent-steps
/ the slowest rank's time.
"""
import argparse
import json
import socket
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_AGENTS = 2_000_000
N_OTHER_LOCS = 500_000
METRIC = "agent-steps/s at 2M agents"
UNIT = "agent-steps/s"
# The reference's step: per agent the countdown (read and write, 8), the
# agent list (12) and the infection inputs (12); per location the offsets (8)
# and the reduction's inputs and output (12): 32*N + 20*L bytes per timestep.
# Our step touches much less (most timesteps move nobody); this figure over
# our timestep time is the step-rate fraction, a rate and not a bandwidth.
STEP_BYTES = (32, 20)


def kernel_bytes(N, L, V, spd, counts):
    """Algorithmic bytes per simulated day of each phase of the step kernel,
    from the profiled day's counters (entries E, entries at a location with a
    nonzero ratio EH, queued agents M, queue passes Q, rebuilds R, listed
    locations LL and agents LA, summed over the rebuilds and steps):
      rebuild   per rebuild the hazard mask read twice (L / 4) and every
                agent's location (4 N); per listed location its sums read
                (8 V), its count read twice and its first slot written (12);
                per listed agent its age band and susceptibilities read, its
                slot's atomic, id, location and susceptibility products
                written (17 + 8 V)
      draw      per entry its slot's location, agent and susceptibility
                products (8 + 4 V) and its location's count, weight, replica
                and sums (10 + 8 V)
      decide    per queue pass the decision timestamps (4 N); per decision
                76: its work-list entry written and read (8), the agent's
                location, decision timestamp, state, type, age, flags and
                timestamps (38), its location-list entries (12), the new
                location's flags (5), the location and timestamp written (8),
                the histogram deltas (8)
    """
    E, EH, M, Q, R, LL, LA = (float(x) for x in counts)
    return {"rebuild": R * (L / 4.0 + 4.0 * N) + (12 + 8 * V) * LL + (17 + 8 * V) * LA,
            "draw": (18 + 12 * V) * E,
            "decide": 4.0 * N * Q + 76.0 * M}


KERNEL_LABELS = {"rebuild": "k_step rebuild phase", "draw": "k_step draw phase", "decide": "k_step queue + decide phase"}


def step_kinds(tl):
    """The profiled day's steps by kind (tl: per step the kernel span, the
    rebuild's listing and slots, the draws, the queue, the decisions, the
    time since the previous kernel, us): count and mean span, gap and phase
    times of the draw-only steps, the steps with a rebuild and no decisions,
    with decisions and no rebuild, with both."""
    reb, dec = tl[:, 1:3].sum(axis=1) > 0, tl[:, 5] > 0
    out = {}
    cols = ["span_us", "rebuild_listing_us", "rebuild_slots_us", "draw_us", "queue_us", "decide_us", "gap_us"]
    for name, sel in [("draw_only", ~reb & ~dec), ("rebuild", reb & ~dec), ("decide", ~reb & dec),
                      ("rebuild_and_decide", reb & dec)]:
        n = int(sel.sum())
        out[name] = {"steps": n}
        for j, c in enumerate(cols):
            out[name][c] = float(tl[sel, j].mean()) if n else None
    return out


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def whole_job(total_ms, agents_per_rank, timesteps_per_step, steps, ws, dist=None, device="cuda"):
    """(max over ranks of the timed milliseconds, whole-job agent-steps/s):
    every rank runs its own replica of the same size (weak scaling), so the
    job processes ws times the per-rank agent-steps in the slowest rank's time."""
    t_max = float(total_ms)
    if dist is not None and ws > 1:
        import torch
        tt = torch.tensor([float(total_ms)], device=device, dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_max = float(tt.item())
    value = agents_per_rank * ws * timesteps_per_step * steps / (t_max / 1000.0)
    return t_max, value


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic():
    """dram bytes per launch of the dominant kernel from the committed ncu summary, or None."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as f:
            return json.load(f)
    except Exception:
        return None


class ClockSampler:
    def __init__(self, gpu_index):
        self.f = tempfile.NamedTemporaryFile(prefix="clocks_", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), "--query-gpu=" + q,
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
        self.f.close()
        rows = []
        try:
            for line in open(self.f.name):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except Exception:
            pass
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


WORKLOAD = "2M agents, 500k non-home locations (+homes), dt 10 min, 1 day per step"


def workload_config(snap, ws):
    """The `config` of both arms' lines (identical, so the two runs read as
    the same workload)."""
    return {"workload": WORKLOAD, "agents": snap.n_agents, "locations": snap.n_locations,
            "timesteps_per_step": snap.steps_per_day,
            "l2": "GB300 arm: flushed between timed steps (256 MiB write)",
            "parallelism": "replicas" if ws > 1 else "1 gpu"}


def make_snapshot(rank):
    from pansim_gb300 import synth
    return synth.make_snapshot(N_AGENTS, N_OTHER_LOCS, seed=1 + rank, model_seed=0x5EED0000, pop_seed=0x5EED0002)


def pinned_copy(snap):
    """Snapshot whose mutable arrays live in one block of pinned host memory
    (torch.pin_memory), laid out as the library's device state
    (native.state_layout), so that an upload or a download is one copy."""
    import torch
    from pansim_gb300 import native
    from pansim_gb300.snapshot import AGENT_MUTABLE, LOC_MUTABLE
    s = snap.copy()
    fields = [(s.agents, k) for k in AGENT_MUTABLE] + [(s.locs, k) for k in LOC_MUTABLE]
    off = native.state_layout(s.n_agents, s.n_locations, int(s.model["n_variants"]))
    assert len(off) == len(fields) + 1
    t = torch.empty(max(int(off[-1]), 1), dtype=torch.uint8, pin_memory=True)
    buf = t.numpy()
    for j, (part, k) in enumerate(fields):
        a = part[k]
        assert a.nbytes <= int(off[j + 1] - off[j]), k
        v = buf[int(off[j]): int(off[j]) + a.nbytes].view(a.dtype).reshape(a.shape)
        v[...] = a
        part[k] = v
    s._pins = [t]
    return s


def mutable_bytes(snap):
    from pansim_gb300.snapshot import AGENT_MUTABLE, LOC_MUTABLE
    return sum(snap.agents[k].nbytes for k in AGENT_MUTABLE) + sum(snap.locs[k].nbytes for k in LOC_MUTABLE)


def cpu_baseline(snap, min_seconds=8.0):
    """The oracle port on all host threads (OpenMP): whole days (midnight
    phases + 144 timesteps) of the same workload until `min_seconds` elapsed."""
    from oracle import binding as ob
    s = snap.copy()
    o = ob.Oracle(s)
    spd = s.steps_per_day
    days = 0
    rows = []
    t0 = time.perf_counter()
    while True:
        rows.append([list(x.v)[: x.n] for x in o.run_day(days)])
        days += 1
        dt = time.perf_counter() - t0
        if dt >= min_seconds:
            break
    o.close()
    res = {"value": s.n_agents * spd * days / dt, "unit": UNIT, "cores": ob.threads(), "kind": "port",
           "sample": "%d whole days (midnight + %d timesteps) of the 2M-agent workload from day 0, "
                     "oracle port on %d threads" % (days, spd, ob.threads()),
           "seconds": round(dt, 3)}
    return res, rows, s


def parity_check(snap, cpu_rows, cpu_state, best, device):
    """The GB300 arm on the same snapshot from day 0, for the days the CPU
    baseline ran: every daily statistics row and, at the end, every mutable
    agent and location array compared with the oracle's."""
    import numpy as np
    from pansim_gb300 import native
    from pansim_gb300.snapshot import AGENT_MUTABLE, LOC_MUTABLE
    s = snap.copy()
    g = native.GpuSim(s, device=device)
    g.set_tuning(**best)
    rows_equal = True
    first_diff = None
    for d, row in enumerate(cpu_rows):
        got = [list(x.v)[: x.n] for x in g.run_day(d)]
        if got != row and first_diff is None:
            first_diff = d
        rows_equal = rows_equal and got == row
    g.download()
    g.close()
    diff = [k for k in AGENT_MUTABLE if not np.array_equal(s.agents[k], cpu_state.agents[k])]
    diff += ["loc." + k for k in LOC_MUTABLE if not np.array_equal(s.locs[k], cpu_state.locs[k])]
    return {"days": len(cpu_rows), "rows_equal": bool(rows_equal), "state_equal": not diff,
            "differing_arrays": diff, "first_differing_day": first_diff,
            "against": "oracle port, same snapshot from day 0 (the cpu_baseline run)"}


def run_reference(args, ws, rank):
    """The reference path's CPU implementation on the host cores: the oracle
    port (OpenMP over agents and locations), one bench step = one simulated
    day (midnight phases + 144 timesteps), as in the GPU arm."""
    if rank != 0:
        return 0
    from oracle import binding as ob
    snap = make_snapshot(0)
    o = ob.Oracle(snap)
    spd = snap.steps_per_day
    day = 0
    for _ in range(args.warmup):
        o.run_day(day)
        day += 1
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.run_day(day)
        day += 1
    dt = time.perf_counter() - t0
    value = snap.n_agents * spd * args.steps / dt
    cores = ob.threads()
    # n_gpus: the job's, as in the GB300 arm's line (the work runs on rank 0's host cores)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1000 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(snap, ws),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "%d simulated days after %d warm-up days, oracle port on %d threads"
                                       % (args.steps, args.warmup, cores)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def measure_policy(days=28, warmup=2, scale=1.0):
    """Config 3: 20M agents, 5M locations, quarantine policy 3 (10 days),
    testing (5e-5 / 1e-2 / 5e-4 / 5e-4 / 5e-3, PCR), closures of work, school
    and shops while daily new infections exceed 0.05% of the population, and
    immunization of 50k a day from day 7 in a 6-category order."""
    import torch
    from pansim_gb300 import closures, immunization, native, synth
    snap = synth.config_snapshot(3, scale=scale)
    N = snap.n_agents
    g = native.GpuSim(snap)
    rules = [dict(name="lockdown", conditionType="newCasesFraction", threshold=0.0005, threshold2=0.00025,
                  closeAfter=1, openAfter=7, parameter=0,
                  locationTypesToClose=[synth.WORK, synth.SCHOOL, synth.SHOP])]
    g.closures_init(rules, closures.stats_header(synth.STATE_NAMES))
    g.immunization_init(immunization.options(immunizations_per_week=int(350_000 * scale), immunizationStart=7,
                                             immunizationOrder="1,2,3,4,5,6,0,0,0,0", boosterStart="1000",
                                             boosters_per_week=[([0], [1.0] * 10)]))
    spd = snap.steps_per_day
    for d in range(warmup):
        g.run_day(d)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    graph_ms = 0.0
    rows = []
    for d in range(warmup, days):
        st = g.run_day(d)
        graph_ms += g.last_day_ms()
        rows.append(list(st[0].v)[: st[0].n])
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    n_days = days - warmup
    act, op = g.closures_status()
    vac_col = len(synth.STATE_NAMES) + 9
    g.close()
    return {"metric": "agent-steps/s at 20M agents, policy-heavy", "value": N * spd * n_days / dt,
            "unit": UNIT, "higher_is_better": True, "days": n_days, "warmup_days": warmup,
            "graph_ms_per_day": graph_ms / n_days, "ms_per_day": dt * 1000 / n_days,
            "immunized_total": int(sum(r[vac_col] for r in rows)),
            "closure_rule_active_at_end": bool(act[0]) if len(act) else None,
            "config": {"workload": "20M agents, 5M non-home locations (+homes), quarantine 3, testing, closures, "
                                   "immunization", "agents": N, "locations": snap.n_locations, "scale": scale}}


def measure_batched(days=28, scale=1.0):
    """64 replicas, agent counts log-uniform on [250k, 2M], k log-uniform on
    [1e-4, 1e-3], independent seeds: one context over the concatenation vs
    the same 64 runs one after another (same days, same per-replica rows).
    Each arm is autotuned on its own workload: the batch once, every
    sequential replica separately."""
    import numpy as np
    import torch
    from pansim_gb300 import autotune, native, snapshot as snp, synth
    n, ks, seeds = synth.batch_sizes(64)
    n = np.maximum((n * scale).astype(np.int64), 1000)
    parts = [synth.make_snapshot(int(n[r]), int(n[r]) // 4, seed=int(seeds[r]), pop_seed=0x5EED0004 + r, k=float(ks[r]))
             for r in range(len(n))]
    batch = snp.concat(parts, seeds, ks)
    g = native.GpuSim(batch)
    g.run_day(0)
    best, _ = autotune.autotune(g, 1)
    g.run_day(1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rows_b = []
    for d in range(2, 2 + days):
        rows_b.append([list(x.v)[: x.n] for x in g.run_day(d)])
    tb = time.perf_counter() - t0
    g.close()
    del g, batch
    ts = 0.0
    same = True
    tunings = {}
    for r, p in enumerate(parts):
        gs = native.GpuSim(p)
        gs.run_day(0)
        best_r, _ = autotune.autotune(gs, 1)
        tunings[json.dumps(best_r, sort_keys=True)] = tunings.get(json.dumps(best_r, sort_keys=True), 0) + 1
        gs.run_day(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for j, d in enumerate(range(2, 2 + days)):
            row = [list(x.v)[: x.n] for x in gs.run_day(d)][0]
            same = same and row == rows_b[j][r]
        ts += time.perf_counter() - t0
        gs.close()
    tot = int(n.sum()) * 144 * days
    return {"metric": "64-replica batched vs sequential", "value": ts / tb, "unit": "x", "higher_is_better": True,
            "batched_agent_steps_per_s": tot / tb, "sequential_agent_steps_per_s": tot / ts,
            "batched_s": tb, "sequential_s": ts, "days": days, "replicas": int(len(n)), "agents_total": int(n.sum()),
            "identical_per_replica_statistics": bool(same), "batch_tuning": best,
            "sequential_tunings": [dict(json.loads(k), replicas=v) for k, v in tunings.items()],
            "config": {"workload": "64 replicas, agents log-uniform 250k-2M x%g, k log-uniform 1e-4..1e-3, "
                                   "days 3-%d (after 2 warm-up days and the autotuner)" % (scale, 2 + days)}}


def measure_adjoint(days=28, scale=1.0):
    """16 replicas x 1M agents, 28 days: forward with per-day checkpoints,
    backward replay with the adjoint accumulation."""
    import numpy as np
    import torch
    from pansim_gb300 import adjoint, snapshot as snp, synth
    R, n = 16, int(1_000_000 * scale)
    parts = [synth.make_snapshot(n, n // 4, seed=100 + r, pop_seed=0x5EED0005 + r) for r in range(R)]
    batch = snp.concat(parts, [100 + r for r in range(R)], [3.74e-4] * R)
    runner = adjoint.CalibrationRunner(batch, days)
    theta = adjoint.theta_of(batch)
    runner.set_theta(theta)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    E = runner.forward()
    tf = time.perf_counter() - t0
    target = E.mean(axis=0) * 0.9
    gE = 2.0 * (E - target[None, :])
    t0 = time.perf_counter()
    grad = runner.backward(gE)
    tbw = time.perf_counter() - t0
    cb = runner.g.checkpoint_bytes()
    runner.g.close()
    return {"metric": "adjoint grad time", "value": tf + tbw, "unit": "s", "higher_is_better": False,
            "forward_s": tf, "backward_s": tbw, "replicas": R, "agents_per_replica": n, "days": days,
            "checkpoint_bytes_per_day": cb, "grad_norm": float(np.linalg.norm(grad)),
            "config": {"workload": "16 replicas x 1M agents x %d days, theta = k, 5 type weights, "
                                   "9 band susceptibilities" % days}}


def extras(args):
    """The other two parts of the headline metric (64-replica batched vs
    sequential, adjoint gradient time) and the 20M-agent policy workload, on
    the same GPU after the main measurement."""
    out = {}
    for name, fn in (("batched", measure_batched), ("adjoint", measure_adjoint), ("policy", measure_policy)):
        t0 = time.perf_counter()
        try:
            out[name] = fn(days=args.days or 28, scale=args.scale)
        except Exception as e:  # reported, not hidden: the main figure stands on its own
            out[name] = {"error": "%s: %s" % (type(e).__name__, e)}
        out[name]["wall_s"] = round(time.perf_counter() - t0, 2)
    return out


def free_port():
    sk = socket.socket()
    sk.bind(("127.0.0.1", 0))
    port = sk.getsockname()[1]
    sk.close()
    return port


def launch_ranks(n, argv, script=None):
    """Starts `script` (this file) as n ranks on this node, one per GPU,
    under torch.distributed.run with a rendezvous on 127.0.0.1 (each rank
    reads RANK / LOCAL_RANK / WORLD_SIZE from its environment and runs its
    own replica).  Returns the launcher's exit status."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(n),
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), script or os.path.abspath(__file__)]
    return subprocess.call(cmd + list(argv))


def _print(d):
    print(json.dumps(d, default=float))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=40)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="step", choices=["step", "batched", "adjoint", "policy"])
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--days", type=int, default=0)
    ap.add_argument("--no-extras", action="store_true")
    args = ap.parse_args()
    if args.workload == "batched":
        return _print(measure_batched(days=args.days or 28, scale=args.scale)) or 0
    if args.workload == "adjoint":
        return _print(measure_adjoint(days=args.days or 28, scale=args.scale)) or 0
    if args.workload == "policy":
        return _print(measure_policy(days=args.days or 28, warmup=min(args.warmup, 2), scale=args.scale)) or 0
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, max(ws, args.gpus) if "WORLD_SIZE" not in os.environ else ws, rank)
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one process per GPU: the same command under torch.distributed.run
        return launch_ranks(args.gpus, sys.argv[1:])

    import numpy as np
    import torch
    from pansim_gb300 import native

    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    snap = make_snapshot(rank)
    host_snap = snap.copy() if (rank == 0 and not args.no_cpu_baseline) else None
    g = native.GpuSim(snap, device=local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    ext = torch.cuda.ExternalStream(g.stream())
    day = 0
    for _ in range(args.warmup):
        g.run_day(day)
        day += 1
    # autotune the step kernels on this workload (part of the warm-up)
    from pansim_gb300 import autotune
    best, table = autotune.autotune(g, day)
    g.run_day(day)
    day += 1
    # the state at the start of the timed days, for the end-to-end pass
    ps = None
    if rank == 0 and args.e2e_steps > 0:
        g.download()
        ps = pinned_copy(snap)
    day_timed0 = day
    sampler = ClockSampler(local)
    launches0 = g.launch_count()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    total_ms = 0.0
    graph_ms = 0.0  # the day graphs alone (CUDA events around the graph launch, library stream)
    for _ in range(args.steps):
        flush.fill_(1.0)  # L2 flush between timed days (buffer 2x L2)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        g.run_day(day)
        e1.record(ext)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
        graph_ms += g.last_day_ms()
        day += 1
    torch.cuda.synchronize()
    launches = g.launch_count() - launches0
    clocks = sampler.stop()
    spd = snap.steps_per_day
    t_max, value = whole_job(total_ms, snap.n_agents, spd, args.steps, ws, dist, "cuda")
    # per-phase durations (roofline): the same days again with the kernels'
    # timeline stamps (global timer at every block's entry, phase ends and
    # exit, one atomic per block and stamp) and the day's counters (entries
    # drawn, decisions, rebuilds).  Kept out of the timed region above.
    g.set_profiling(True)
    g.run_day(day)  # captures the profiled graph
    day += 1
    n_prof = min(args.steps, 10)
    kms_sum = np.zeros(5)
    cnt_sum = np.zeros(7)
    tl_sum = None
    prof_day_ms = 0.0
    for _ in range(n_prof):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        g.run_day(day)
        kms_sum += g.day_kernel_ms()
        cnt_sum += g.day_counts().astype(np.float64)
        tl = g.day_timeline().astype(np.float64)
        tl_sum = tl if tl_sum is None else tl_sum + tl
        prof_day_ms += g.last_day_ms()
        day += 1
    g.set_profiling(False)

    # end to end through the C ABI with pinned host buffers: per step, the
    # full mutable state host->device, one day, the full state device->host
    # (the same simulated days as the timed region, from the same state: a new
    # context on pinned host buffers; every step uploads the whole mutable
    # state, runs the day and downloads the whole state, which is the next
    # step's input)
    e2e = None
    if ps is not None:
        ge = native.GpuSim(ps, device=local)
        ge.set_tuning(**best)
        ge.run_day(day_timed0)  # warm-up (graph capture); the first upload restores the state
        nb = mutable_bytes(ps)
        n_e2e = min(args.e2e_steps, args.steps)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for j in range(n_e2e):
            ge.upload()
            ge.run_day(day_timed0 + j)
            ge.download()
        te = time.perf_counter() - t0
        e2e = {"value": ps.n_agents * spd * n_e2e / te, "unit": UNIT,
               "h2d_bytes_per_step": nb, "d2h_bytes_per_step": nb, "steps": n_e2e,
               "days": "the timed days, from the same state"}
        ge.close()

    if rank == 0:
        peak, peak_kind = peaks()
        N, L = snap.n_agents, snap.n_locations
        V = int(snap.model["n_variants"])
        counts = cnt_sum / n_prof
        kb = kernel_bytes(N, L, V, spd, counts)
        kms_day = kms_sum / n_prof  # per simulated day: movement(0), rebuild, draw, queue + decide, between kernels
        launches_per_day = {"rebuild": max(counts[4], 1.0), "draw": float(spd), "decide": max(counts[3], 1.0)}
        kern = {"movement": {"ms_per_day": float(kms_day[0])}}
        for j, name in enumerate(["rebuild", "draw", "decide"]):
            ms = float(kms_day[1 + j])
            kern[name] = {"ms_per_day": ms, "alg_bytes_per_day": kb[name],
                          "launches_with_work_per_day": launches_per_day[name],
                          "gbs": kb[name] / (ms * 1e-3) / 1e9 if ms > 0 else None,
                          "frac": kb[name] / (ms * 1e-3) / 1e9 / peak if ms > 0 else None}
        kern["between_kernels"] = {"ms_per_day": float(kms_day[4])}
        tot_k = sum(kern[n]["ms_per_day"] for n in KERNEL_LABELS) or 1.0
        for name in KERNEL_LABELS:
            kern[name]["share_of_steps"] = kern[name]["ms_per_day"] / tot_k
        steps_by_kind = step_kinds(tl_sum / n_prof)
        # The step kernel (one launch per timestep, its phases fused with
        # grid barriers) is the kernel of the day graph: its algorithmic
        # bytes per launch are the phases' bytes of a day over the day's
        # timesteps, its launch time the timed days' graph time (less the
        # day's first movement pass) over their timesteps.
        step_alg = sum(kb.values()) / spd
        step_ms = (graph_ms / args.steps - float(kms_day[0])) / spd
        ach = step_alg / (step_ms * 1e-3) / 1e9
        tr = committed_traffic()
        traffic = tr.get("k_step") if tr else None
        # the step-rate figure: the reference's per-step bytes over our
        # average timestep time
        step_bytes = STEP_BYTES[0] * N + STEP_BYTES[1] * L
        counts_d = {"draw_entries": counts[0], "draw_entries_with_hazard": counts[1], "decisions": counts[2],
                    "queue_passes": counts[3], "rebuilds": counts[4], "listed_locations": counts[5],
                    "listed_agents": counts[6]}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": workload_config(snap, ws),
            "roofline": {"bound": "hbm", "kernel": "k_step (one launch per timestep: rebuild, draw, decide phases)",
                         "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak, "traffic": traffic,
                         "peak_kind": peak_kind, "alg_bytes_per_launch": step_alg, "launch_ms": step_ms,
                         "launch_ms_source": "day-graph CUDA events over the timed days, less the first movement "
                                             "pass, over their timesteps",
                         "dominant": "k_step", "dominant_phase": max(KERNEL_LABELS, key=lambda n: kern[n]["ms_per_day"]),
                         "per_phase": kern, "day_counts": counts_d, "steps_by_kind": steps_by_kind,
                         "step_rate": {"reference_bytes_per_timestep": step_bytes, "timestep_ms": step_ms,
                                       "gbs": step_bytes / (step_ms * 1e-3) / 1e9,
                                       "frac": step_bytes / (step_ms * 1e-3) / 1e9 / peak,
                                       "note": "the reference's step bytes (32 N + 20 L) over our timestep "
                                               "time: a rate, not a bandwidth"}},
            "clocks": clocks, "gpu_launches": int(launches), "e2e": e2e,
            "kernel_timing": {"days": n_prof, "graph_ms_per_day_with_stamps": prof_day_ms / n_prof,
                              "note": "per-phase durations from the kernels' timeline stamps in a separate pass"},
            "tuning": {"best": best, "candidates": len(table),
                       "worst_step_ms": max(x[1] for x in table), "best_step_ms": min(x[1] for x in table)},
        }
        if host_snap is not None:
            line["cpu_baseline"], cpu_rows, cpu_state = cpu_baseline(host_snap)
            line["parity"] = parity_check(make_snapshot(0), cpu_rows, cpu_state, best, local)
        if ws == 1 and not args.no_extras:
            line["extras"] = extras(args)
        print(json.dumps(line, default=float))
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
