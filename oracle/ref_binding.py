"""ctypes wrapper of the reference-compiled harness (oracle/_ref) — TEST
INFRASTRUCTURE ONLY.  Available where the reference tree is (this is where
the pinning tests and golden fixtures are produced)."""
import ctypes as C
import os

import numpy as np

from . import ref_build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = ref_build.build()
        if path is None:
            raise RuntimeError("reference tree not available")
        L = C.CDLL(path)
        P, U32 = C.c_void_p, C.c_uint32
        L.ref_create.restype = P
        L.ref_create.argtypes = [P, P, P, P, C.c_int, C.c_ulonglong]
        L.ref_destroy.argtypes = [P]
        L.ref_set_params.argtypes = [P, P]
        for f in ["ref_midnight", "ref_movement", "ref_step", "ref_run_day"]:
            getattr(L, f).argtypes = [P, U32]
        L.ref_sync_out.argtypes = [P]
        L.ref_csr.argtypes = [P, P, P]
        L.ref_event_minutes.argtypes = [P, P, P, P]
        L.ref_threads.restype = C.c_int
        _lib = L
    return _lib


def available():
    try:
        lib()
        return True
    except Exception:
        return False


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class RefSim:
    """The reference's hot path on a Snapshot (single replica).  native=False:
    Philox streams (pins the oracle bit for bit); native=True: the reference's
    own RNG, FP32 reduction and OpenMP loops."""

    def __init__(self, snap, native=False, native_seed=1):
        assert snap.n_replicas == 1
        self.snap = snap
        self.structs = snap.structs()
        m, a, lo, p, r = self.structs
        self.h = lib().ref_create(C.byref(m), C.byref(a), C.byref(lo), C.byref(p), 1 if native else 0, native_seed)

    def close(self):
        if self.h:
            lib().ref_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_params(self):
        p = self.snap.params_struct()
        self.structs = self.structs[:3] + (p,) + self.structs[4:]
        lib().ref_set_params(self.h, C.byref(p))

    def midnight(self, t):
        lib().ref_midnight(self.h, t)

    def movement(self, t):
        lib().ref_movement(self.h, t)

    def step(self, t):
        lib().ref_step(self.h, t)

    def run_day(self, day):
        lib().ref_run_day(self.h, day)

    def sync(self):
        lib().ref_sync_out(self.h)
        return self.snap

    def csr(self):
        off = np.zeros(self.snap.n_locations + 1, np.uint32)
        ag = np.zeros(self.snap.n_agents, np.uint32)
        lib().ref_csr(self.h, _p(off), _p(ag))
        return off, ag

    def event_minutes(self):
        n = len(self.snap.model["ev_start"])
        s, e, d = (np.zeros(n, np.uint16) for _ in range(3))
        lib().ref_event_minutes(self.h, _p(s), _p(e), _p(d))
        return s, e, d
