"""ctypes wrapper of the C oracle — TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
checker; the product never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from pansim_gb300 import cabi

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libpsim_oracle.so")


def build(force=False):
    """gcc -O2 -ffp-contract=off -fopenmp: no FMA contraction, so FP results
    match the device; the per-step loops run on all host threads (the results
    do not depend on their number)."""
    src = os.path.join(HERE, "psim_oracle.c")
    deps = [src, os.path.join(HERE, "psim_oracle.h"),
            os.path.join(HERE, "..", "pansim_gb300", "csrc", "psim_rng.h"),
            os.path.join(HERE, "..", "pansim_gb300", "csrc", "psim_immunity.h"),
            os.path.join(HERE, "..", "include", "pansim_gb300.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".%d.tmp" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-o", tmp, src, "-lm"])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        P, U32, D = C.c_void_p, C.c_uint32, C.c_double
        L = _lib
        L.psim_oracle_create.restype = P
        L.psim_oracle_create.argtypes = [P, P, P, P, P]
        L.psim_oracle_destroy.argtypes = [P]
        L.psim_oracle_set_params.argtypes = [P, P]
        for f in ["psim_oracle_movement", "psim_oracle_progress", "psim_oracle_plan"]:
            getattr(L, f).argtypes = [P, U32]
        L.psim_oracle_regroup.argtypes = [P]
        L.psim_oracle_infect.argtypes = [P, U32, U32, P, P, P, P, P, P]
        L.psim_oracle_step.argtypes = [P, U32, P]
        L.psim_oracle_test.argtypes = [P, U32, P]
        L.psim_oracle_stats.argtypes = [P, U32, P]
        L.psim_oracle_midnight.argtypes = [P, U32, P]
        L.psim_oracle_run_day.argtypes = [P, U32, P]
        L.psim_oracle_expose.argtypes = [P, U32, U32, D]
        L.psim_oracle_threads.restype = C.c_int
        L.psim_oracle_threads.argtypes = []
        L.psim_oracle_immunization_init.argtypes = [P, P]
        L.psim_oracle_immunize.restype = U32
        L.psim_oracle_immunize.argtypes = [P, U32]
        L.psim_oracle_other_disease_init.argtypes = [P, P]
        L.psim_oracle_other_disease.argtypes = [P, U32]
        L.psim_oracle_csr_offsets.restype = C.POINTER(C.c_uint32)
        L.psim_oracle_csr_offsets.argtypes = [P]
        L.psim_oracle_csr_agents.restype = C.POINTER(C.c_uint32)
        L.psim_oracle_csr_agents.argtypes = [P]
        L.psim_oracle_philox.argtypes = [P, P, P]
        L.psim_oracle_one_minus_exp.restype = D
        L.psim_oracle_one_minus_exp.argtypes = [D]
        L.psim_oracle_one_minus_expf.restype = C.c_float
        L.psim_oracle_one_minus_expf.argtypes = [C.c_float]
        L.psim_oracle_seasonality.restype = D
        L.psim_oracle_seasonality.argtypes = [P, U32, U32]
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Oracle:
    """Runs the oracle in place on a Snapshot's host arrays."""

    def __init__(self, snap):
        self.snap = snap
        self.structs = snap.structs()
        m, a, lo, p, r = self.structs
        self.h = lib().psim_oracle_create(C.byref(m), C.byref(a), C.byref(lo), C.byref(p), C.byref(r))

    def close(self):
        if self.h:
            lib().psim_oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_params(self):
        p = self.snap.params_struct()
        self.structs = self.structs[:3] + (p,) + self.structs[4:]
        lib().psim_oracle_set_params(self.h, C.byref(p))

    def movement(self, t):
        lib().psim_oracle_movement(self.h, t)

    def regroup(self):
        lib().psim_oracle_regroup(self.h)

    def csr(self):
        L, N = self.snap.n_locations, self.snap.n_agents
        off = np.ctypeslib.as_array(lib().psim_oracle_csr_offsets(self.h), shape=(L + 1,)).copy()
        ag = np.ctypeslib.as_array(lib().psim_oracle_csr_agents(self.h), shape=(max(N, 1),))[:N].copy()
        return off, ag

    def infect(self, t, v=0):
        L, N, R = self.snap.n_locations, self.snap.n_agents, self.snap.n_replicas
        out = dict(hazard=np.zeros(L, np.float32), fix=np.zeros(L, np.int64), sum64=np.zeros(L),
                   r64=np.zeros(L), p64=np.zeros(N), expected=np.zeros(R))
        lib().psim_oracle_infect(self.h, t, v, _p(out["hazard"]), _p(out["fix"]), _p(out["sum64"]),
                                 _p(out["r64"]), _p(out["p64"]), _p(out["expected"]))
        return out

    def step(self, t):
        lib().psim_oracle_step(self.h, t, None)

    def test(self, t):
        tpp = np.zeros(3 * self.snap.n_replicas, np.uint32)
        lib().psim_oracle_test(self.h, t, _p(tpp))
        return tpp

    def progress(self, t):
        lib().psim_oracle_progress(self.h, t)

    def plan(self, t):
        lib().psim_oracle_plan(self.h, t)

    def stats(self, t):
        out = (cabi.PsimDayStats * self.snap.n_replicas)()
        lib().psim_oracle_stats(self.h, t, out)
        return out

    def midnight(self, t):
        out = (cabi.PsimDayStats * self.snap.n_replicas)()
        lib().psim_oracle_midnight(self.h, t, out)
        return out

    def run_day(self, day):
        out = (cabi.PsimDayStats * self.snap.n_replicas)()
        lib().psim_oracle_run_day(self.h, day, out)
        return out

    def immunization_init(self, imm):
        self._imm = imm
        lib().psim_oracle_immunization_init(self.h, C.byref(imm) if imm is not None else None)

    def immunize(self, t):
        return lib().psim_oracle_immunize(self.h, t)

    def other_disease_init(self, od):
        self._od = od
        lib().psim_oracle_other_disease_init(self.h, C.byref(od) if od is not None else None)

    def other_disease(self, t):
        lib().psim_oracle_other_disease(self.h, t)


def threads():
    """Host threads the oracle's parallel loops use."""
    return lib().psim_oracle_threads()


def philox(ctr, key):
    c = np.array(ctr, np.uint32)
    k = np.array(key, np.uint32)
    o = np.zeros(4, np.uint32)
    lib().psim_oracle_philox(_p(c), _p(k), _p(o))
    return o


def one_minus_exp(x):
    return lib().psim_oracle_one_minus_exp(float(x))


def one_minus_expf(x):
    return lib().psim_oracle_one_minus_expf(float(x))


def seasonality(snap, t):
    p = snap.params_struct()
    return lib().psim_oracle_seasonality(C.byref(p), t, snap.steps_per_day)
