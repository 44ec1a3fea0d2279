"""Differentiable calibration: expected daily new infections and their
gradient with respect to theta = (k, 5 location-type weights, 9 age-band
susceptibilities), as a torch.autograd.Function.

E[r, d] is the expected number of new infections of replica r on day d given
the sampled state: the sum over the day's steps of min(1, p_i) over
susceptible agents, p_i = r_l * s_i * sigma_band(i) (the Bernoulli draws stay
as they are).  Forward: the days run on the GPU with a checkpoint of the
mutable state saved at the start of every day.  Backward: every day is
restored from its checkpoint and replayed (movement and draws recompute
bit-identically from the counter-based streams) while the draw kernels add
dL/dE[r, d] * dp/dtheta in FP64 (psim_set_adjoint).
"""
import numpy as np

from . import native, synth

# parameter layout of theta
TYPE_SLOTS = {synth.HOME: 0, synth.WORK: 1, synth.SCHOOL: 2, synth.SHOP: 3, synth.HOSPITAL: 4}
N_W = 5
N_BANDS = synth.N_BANDS
N_THETA = 1 + N_W + N_BANDS


def theta_of(snap):
    """theta of a snapshot: k, the weights of the slotted location types, sigma per band."""
    w = np.zeros(N_W)
    for t, sl in TYPE_SLOTS.items():
        w[sl] = synth.TYPE_W[t]
    sig = np.asarray(snap.params.get("sigma_band", np.ones(16)), np.float64)[:N_BANDS]
    return np.concatenate([[float(snap.reps["k"][0])], w, sig])


class CalibrationRunner:
    def __init__(self, snap, days, device=0):
        self.snap = snap
        self.days = int(days)
        self.R = snap.n_replicas
        self.g = native.GpuSim(snap, device=device)
        self.g.set_tracking(True)
        self.slot_of_type = np.full(256, -1, np.int8)
        for t, sl in TYPE_SLOTS.items():
            self.slot_of_type[t] = sl
        self.w_base = np.zeros(256, np.float32)
        for t, v in synth.TYPE_W.items():
            self.w_base[t] = v
        self.initial_slot = self.days + 1
        self.g.checkpoint_save(self.initial_slot)
        self.theta = None

    def set_theta(self, theta):
        theta = np.asarray(theta, np.float64)
        assert theta.shape == (N_THETA,)
        self.theta = theta.copy()
        self.g.set_replica_k(np.full(self.R, theta[0]))
        w = self.w_base.copy()
        for t, sl in TYPE_SLOTS.items():
            w[t] = theta[1 + sl]
        self._w = w
        self.g.set_type_weights(w, self.slot_of_type)
        sig = np.ones(16, np.float32)
        sig[:N_BANDS] = theta[1 + N_W:]
        self.snap.params["sigma_band"] = sig
        self.g.set_params()

    def forward(self):
        """E[r, d] for d < days, from the initial state; saves the day checkpoints."""
        g, D, spd = self.g, self.days, self.snap.steps_per_day
        g.checkpoint_restore(self.initial_slot)
        if self.theta is not None:
            g.set_type_weights(self._w, self.slot_of_type)  # the checkpoint holds the old weights
        g.set_adjoint(False)
        E = np.zeros((self.R, D))
        for d in range(D):
            g.checkpoint_save(d)
            st = g.run_day(d)
            if d > 0:
                E[:, d - 1] = [st[r].expected_new_infections for r in range(self.R)]
        st = g.stats(D * spd)
        E[:, D - 1] = [st[r].expected_new_infections for r in range(self.R)]
        g.checkpoint_save(D)
        return E

    def backward(self, dL_dE):
        """dL/dtheta given dL/dE[r, d]: replays every day from its checkpoint."""
        dL_dE = np.asarray(dL_dE, np.float64).reshape(self.R, self.days)
        g = self.g
        g.gradient(reset=True)
        total = np.zeros(25)
        for d in reversed(range(self.days)):
            g.checkpoint_restore(d)
            g.set_adjoint(True, dL_dE[:, d])
            g.run_day(d)
            total += g.gradient(reset=True)
        g.set_adjoint(False)
        g.checkpoint_restore(self.days)
        return np.concatenate([[total[0]], total[1:1 + N_W], total[9:9 + N_BANDS]])


def expected_curve_function():
    """torch.autograd.Function computing E[r, d](theta) with the GPU adjoint."""
    import torch

    class ExpectedCurve(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta, runner):
            runner.set_theta(theta.detach().cpu().numpy())
            E = runner.forward()
            ctx.runner = runner
            return torch.from_numpy(E)

        @staticmethod
        def backward(ctx, grad_E):
            g = ctx.runner.backward(grad_E.detach().cpu().numpy())
            return torch.from_numpy(g), None

    return ExpectedCurve
