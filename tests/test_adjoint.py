"""Adjoint of the expected daily new infections (gpu).

The GPU gradient (checkpoint replay, FP64 accumulation in the draw kernels)
is checked against an FP64 torch autograd evaluation of the same expected
curve along the same sampled trajectory (recorded with the oracle), and
against central finite differences (h = 1e-3 relative) of that FP64
function: within 1e-4 relative per component, with an absolute floor of 1e-9
of the largest component for components that are zero.
"""
import math

import numpy as np
import pytest

from oracle import binding as ob
from pansim_gb300 import adjoint, synth

pytestmark = pytest.mark.gpu
DAYS = 2


def _snapshot():
    return synth.make_snapshot(5000, 1250, seed=17, pop_seed=0x5EED0300, initial_infected_frac=0.06)


def _record(snap, days):
    """The sampled trajectory, step by step, from the oracle."""
    s = snap.copy()
    o = ob.Oracle(s)
    N = s.n_agents
    recs = []
    for d in range(days):
        o.midnight(d * 144)
        season = ob.seasonality(s, d * 144)
        for t in range(d * 144, (d + 1) * 144):
            o.movement(t)
            o.regroup()
            loc = s.agents["location"].copy()
            su = s.agents["susceptible"][:N].copy()
            out = o.infect(t)
            off, _ = o.csr()
            recs.append((d, loc, su, out["fix"].copy(), np.diff(off.astype(np.int64)), season))
    return recs


def _expected_ref(theta, recs, snap, days, torch):
    """FP64 expected daily new infections along the recorded trajectory."""
    k, w, sig = theta[0], theta[1:6], theta[6:15]
    ltype = snap.locs["type"]
    slot = np.full(256, -1)
    for t, sl in adjoint.TYPE_SLOTS.items():
        slot[t] = sl
    lslot = torch.from_numpy(slot[ltype])
    base = torch.from_numpy(np.array([synth.TYPE_W.get(int(t), 0.0) for t in ltype], np.float64))
    w_l = torch.where(lslot >= 0, w[lslot.clamp(min=0)], base)
    band = torch.from_numpy(snap.agents["band"].astype(np.int64))
    dt = float(snap.params["time_step"])
    E = [torch.zeros((), dtype=torch.float64) for _ in range(days)]
    for d, loc, su, fix, n, season in recs:
        fix_t = torch.from_numpy(fix.astype(np.float64)) * 2.0 ** -40
        n_t = torch.from_numpy(np.maximum(n, 1).astype(np.float64))
        x = k * (fix_t / n_t) * w_l * season * dt
        r = -torch.expm1(-x)
        r = torch.where(torch.from_numpy(fix != 0), r, torch.zeros_like(r))
        su_t = torch.from_numpy(su.astype(np.float64))
        p = r[torch.from_numpy(loc.astype(np.int64))] * su_t * sig[band]
        E[d] = E[d] + torch.clamp(p, max=1.0).sum()
    return torch.stack(E)


def test_adjoint_matches_fp64_autograd_and_finite_differences(gpu_lib):
    torch = pytest.importorskip("torch")
    snap = _snapshot()
    theta0 = adjoint.theta_of(snap)
    runner = adjoint.CalibrationRunner(snap.copy(), DAYS)
    runner.set_theta(theta0)
    E_gpu = runner.forward()[0]
    recs = _record(snap, DAYS)
    th = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
    E_ref = _expected_ref(th, recs, snap, DAYS, torch)
    assert E_ref.detach().numpy().min() > 5.0
    np.testing.assert_allclose(E_gpu, E_ref.detach().numpy(), rtol=1e-5)
    target = 0.8 * E_ref.detach()
    L = ((E_ref - target) ** 2).sum()
    L.backward()
    g_ref = th.grad.numpy()
    g_gpu = runner.backward((2.0 * (E_gpu - target.numpy()))[None, :])
    # per component: within 1e-4 relative of the FP64 reference, with an
    # absolute floor of 1e-9 of the largest component for components that
    # are zero (the parameters differ in scale by orders of magnitude, so a
    # bound relative to the largest component would not test the others)
    scale = np.abs(g_ref).max()
    floor = 1e-9 * scale
    tol = 1e-4 * np.abs(g_ref) + floor
    assert (np.abs(g_gpu - g_ref) <= tol).all(), (g_gpu, g_ref)
    assert (np.abs(g_ref) > floor).sum() >= 12  # k, the weights and the populated bands

    def loss(theta):
        with torch.no_grad():
            e = _expected_ref(torch.tensor(theta, dtype=torch.float64), recs, snap, DAYS, torch)
            return float(((e - target) ** 2).sum())

    fd = np.zeros_like(theta0)
    for j in range(len(theta0)):
        h = 1e-3 * abs(theta0[j])
        tp, tm = theta0.copy(), theta0.copy()
        tp[j] += h
        tm[j] -= h
        fd[j] = (loss(tp) - loss(tm)) / (2 * h)
    assert (np.abs(g_gpu - fd) <= 1e-4 * np.abs(fd) + floor).all(), (g_gpu, fd)


def test_autograd_function_and_replica_sum(gpu_lib):
    """The torch.autograd.Function over a 2-replica batch equals the sum of
    the single-replica gradients."""
    torch = pytest.importorskip("torch")
    from pansim_gb300 import snapshot as snp
    parts = [synth.make_snapshot(3000, 750, seed=1, pop_seed=0x5EED0400 + i, initial_infected_frac=0.05)
             for i in range(2)]
    seeds, ks = [5, 6], [3.74e-4, 3.74e-4]
    batch = snp.concat(parts, seeds, ks)
    theta0 = adjoint.theta_of(batch)
    Fn = adjoint.expected_curve_function()
    rb = adjoint.CalibrationRunner(batch, DAYS)
    th = torch.tensor(theta0, requires_grad=True)
    E = Fn.apply(th, rb)
    assert E.shape == (2, DAYS)
    (E ** 2).sum().backward()
    g_batch = th.grad.numpy().copy()
    total = np.zeros_like(theta0)
    for i, p in enumerate(parts):
        q = p.copy()
        q.reps["seed"][:] = seeds[i]
        q.reps["k"][:] = ks[i]
        r1 = adjoint.CalibrationRunner(q, DAYS)
        t1 = torch.tensor(theta0, requires_grad=True)
        e1 = Fn.apply(t1, r1)
        np.testing.assert_allclose(e1.detach().numpy()[0], E.detach().numpy()[i], rtol=1e-9)
        (e1 ** 2).sum().backward()
        total += t1.grad.numpy()
    np.testing.assert_allclose(g_batch, total, rtol=1e-9, atol=1e-12 * np.abs(total).max())


def test_adjoint_identities_at_16_replicas_of_1m_agents(gpu_lib):
    """The calibration workload, 16 replicas x 1M agents x 28 days, through
    two identities that hold at any size.  The ratio's argument is
    proportional to k times the location's weight, so k dL/dk equals
    sum_j w_j dL/dw_j (every location type with a nonzero weight has a slot);
    and p is linear in the band susceptibility, so sum_b sigma_b dL/dsigma_b
    equals sum_{r,d} dL/dE[r, d] E[r, d] when no probability reaches 1: the
    backward replay accumulates the forward pass's own expected curve."""
    from pansim_gb300 import snapshot as snp
    R, n, D = 16, 1_000_000, 28
    parts = [synth.make_snapshot(n, n // 4, seed=100 + r, pop_seed=0x5EED0005 + r) for r in range(R)]
    batch = snp.concat(parts, [100 + r for r in range(R)], [3.74e-4] * R)
    runner = adjoint.CalibrationRunner(batch, D)
    theta = adjoint.theta_of(batch)
    runner.set_theta(theta)
    E = runner.forward()
    assert E.shape == (R, D) and (E > 0).all()
    wE = np.random.default_rng(5).uniform(0.5, 1.5, size=E.shape)
    g = runner.backward(wE)
    runner.g.close()
    th = theta.astype(np.float32).astype(np.float64)  # the values the device holds
    nw = adjoint.N_W
    k_term = th[0] * g[0]
    w_term = float((th[1:1 + nw] * g[1:1 + nw]).sum())
    # every term is positive, so FP64 accumulation errors stay relative
    assert k_term > 0 and abs(k_term - w_term) <= 1e-8 * k_term, (k_term, w_term)
    s_term = float((th[1 + nw:] * g[1 + nw:]).sum())
    e_term = float((wE * E).sum())
    # p is rounded to FP32 in the forward pass (two roundings per term)
    assert abs(s_term - e_term) <= 2.5e-7 * e_term, (s_term, e_term)
