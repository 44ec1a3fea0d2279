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
        L.ref_midnight_pre.argtypes = [P, U32]
        L.ref_plan.argtypes = [P, U32]
        L.ref_get_params.argtypes = [P, P]
        L.ref_closures_init.restype = C.c_int
        L.ref_closures_init.argtypes = [P, P, U32, C.c_char_p, C.c_int]
        L.ref_closures_midnight.argtypes = [P, U32, P, U32]
        L.ref_closures_status.argtypes = [P, P, P, P]
        L.ref_immunization_init.restype = C.c_int
        L.ref_immunization_init.argtypes = [P, P, C.c_char_p]
        L.ref_immunize.restype = U32
        L.ref_immunize.argtypes = [P, U32]
        L.ref_events.restype = U32
        L.ref_events.argtypes = [P, P, P, P, U32]
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

    # closure rules through the reference's RuleClosure
    def midnight_pre(self, t):
        lib().ref_midnight_pre(self.h, t)

    def plan(self, t):
        lib().ref_plan(self.h, t)

    def params(self):
        from pansim_gb300 import cabi
        p = cabi.PsimParams()
        lib().ref_get_params(self.h, C.byref(p))
        return p

    def closures_init(self, rules, header, enable=True):
        from pansim_gb300 import closures
        self._rules = closures.rule_array(rules)
        rc = lib().ref_closures_init(self.h, self._rules, len(rules), header.encode(), 1 if enable else 0)
        if rc:
            raise ValueError("reference RuleClosure::init threw")

    def closures_midnight(self, t, row):
        v = np.array(list(row.v)[: row.n], np.uint32)
        lib().ref_closures_midnight(self.h, t, _p(v), len(v))

    def closures_status(self):
        n = C.c_uint32(0)
        a = np.zeros(64, np.uint8)
        o = np.zeros(64, np.uint8)
        lib().ref_closures_status(self.h, _p(a), _p(o), C.byref(n))
        return a[: n.value].astype(bool), o[: n.value].astype(bool)

    def events(self):
        off = np.zeros(int(self.snap.model["n_agent_types"]) * 28 + 1, np.uint32)
        cap = 4 * len(self.snap.model["ev_loc_type"]) + 64
        ty = np.zeros(cap, np.uint32)
        ch = np.zeros(cap, np.float32)
        n = lib().ref_events(self.h, _p(off), _p(ty), _p(ch), cap)
        s, e, d = (np.zeros(max(n, cap), np.uint16) for _ in range(3))
        lib().ref_event_minutes(self.h, _p(s), _p(e), _p(d))
        return dict(event_offset=off, ev_loc_type=ty[:n], ev_chance=ch[:n], ev_start=s[:n], ev_end=e[:n],
                    ev_duration=d[:n])

    # immunization through the reference's Immunization
    def immunization_init(self, imm, workdir):
        self._imm = imm
        if lib().ref_immunization_init(self.h, C.byref(imm), str(workdir).encode()):
            raise ValueError("reference Immunization::initializeArgs threw")

    def immunize(self, t):
        return lib().ref_immunize(self.h, t)
