"""ctypes binding of libpansim_gb300.so (the C ABI in include/pansim_gb300.h).

The library is built in-tree by pansim_gb300.build; there is no CPU
fallback: a missing library or a missing GPU raises.
"""
import ctypes as C
import os
import re

import numpy as np

from . import cabi
from .build import LIB, ROOT, build

_lib = None


class PsimError(RuntimeError):
    pass


def header_symbols():
    """Function names declared in include/pansim_gb300.h."""
    txt = open(os.path.join(ROOT, "include", "pansim_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(psim_[a-z_0-9]+)\s*\(", txt)))


def lib(auto_build=True):
    global _lib
    if _lib is None:
        path = build() if auto_build else LIB
        if not os.path.exists(path):
            raise PsimError("libpansim_gb300.so is not built (run __graft_entry__.build())")
        L = C.CDLL(path)
        P, U32, I = C.c_void_p, C.c_uint32, C.c_int
        L.psim_version.restype = C.c_char_p
        L.psim_last_error.restype = C.c_char_p
        L.psim_last_error.argtypes = [P]
        L.psim_abi_sizes.argtypes = [P, I]
        L.psim_device_count.argtypes = [P]
        L.psim_create.argtypes = [I, P, P, P, P, P, C.POINTER(P)]
        L.psim_destroy.argtypes = [P]
        L.psim_upload.argtypes = [P, P, P]
        L.psim_download.argtypes = [P, P, P]
        L.psim_set_params.argtypes = [P, P]
        L.psim_set_tracking.argtypes = [P, I]
        for f in ["psim_movement", "psim_step", "psim_progress_day", "psim_plan_day", "psim_run_steps"]:
            getattr(L, f).argtypes = [P, U32]
        L.psim_regroup.argtypes = [P]
        L.psim_infect.argtypes = [P, U32, U32]
        L.psim_test_day.argtypes = [P, U32, P]
        L.psim_stats_day.argtypes = [P, U32, P]
        L.psim_midnight.argtypes = [P, U32, P]
        L.psim_run_day.argtypes = [P, U32, P]
        L.psim_get_csr.argtypes = [P, I, P, P]
        L.psim_get_hazard.argtypes = [P, P, P]
        L.psim_last_day_ms.argtypes = [P, C.POINTER(C.c_float)]
        L.psim_set_profiling.argtypes = [P, C.c_int]
        L.psim_closures_init.argtypes = [P, P, U32, C.c_char_p, I]
        L.psim_closures_midnight.argtypes = [P, U32, P]
        L.psim_closures_status.argtypes = [P, P, P, P]
        L.psim_set_types_open.argtypes = [P, P, U32, I]
        L.psim_scale_location_weights.argtypes = [P, C.c_double, I]
        L.psim_get_params.argtypes = [P, P]
        L.psim_immunization_init.argtypes = [P, P]
        L.psim_immunize_day.argtypes = [P, U32, P]
        L.psim_other_disease_init.argtypes = [P, P]
        L.psim_other_disease_day.argtypes = [P, U32]
        L.psim_get_events.argtypes = [P, P, P, P, P, P, P, U32, P]
        L.psim_day_kernel_ms.argtypes = [P, C.c_void_p]
        L.psim_day_timeline.argtypes = [P, C.c_void_p]
        L.psim_day_counts.argtypes = [P, C.c_void_p]
        L.psim_set_alloc_fault.argtypes = [C.c_longlong]
        L.psim_launch_count.argtypes = [P, C.POINTER(C.c_uint64)]
        L.psim_stream_handle.argtypes = [P, C.POINTER(P)]
        L.psim_bounded_wait_selftest.argtypes = [P, U32]
        L.psim_time_step_kernels.argtypes = [P, U32, P]
        L.psim_set_tuning.argtypes = [P, P]
        L.psim_csr_build_noalloc.argtypes = [P, U32, U32, P, P, P]
        L.psim_set_type_weights.argtypes = [P, P, P]
        L.psim_set_replica_k.argtypes = [P, P]
        L.psim_set_adjoint.argtypes = [P, I, P]
        L.psim_get_gradient.argtypes = [P, P, I]
        L.psim_checkpoint_save.argtypes = [P, U32]
        L.psim_checkpoint_restore.argtypes = [P, U32]
        L.psim_checkpoint_free.argtypes = [P]
        L.psim_checkpoint_drop.argtypes = [P, U32]
        L.psim_checkpoint_bytes.argtypes = [P, C.POINTER(C.c_uint64)]
        L.psim_noalloc_last_error.restype = C.c_char_p
        L.psim_get_tuning.argtypes = [P, P]
        L.psim_state_layout.argtypes = [U32, U32, U32, P, P]
        _lib = L
    return _lib


def abi_sizes():
    out = np.zeros(6, np.uint64)
    lib().psim_abi_sizes(out.ctypes.data_as(C.c_void_p), 6)
    return [int(x) for x in out]


def state_layout(n_agents, n_locations, n_variants):
    """Byte offsets of the mutable state fields (snapshot.AGENT_MUTABLE then
    LOC_MUTABLE; the last entry is the total) as the library lays them out in
    one device allocation: host arrays in this layout move in one copy."""
    n = C.c_uint32(0)
    lib().psim_state_layout(n_agents, n_locations, n_variants, None, C.byref(n))
    off = np.zeros(n.value + 1, np.uint64)
    lib().psim_state_layout(n_agents, n_locations, n_variants, _p(off), None)
    return off


def device_count():
    n = C.c_int(0)
    lib().psim_device_count(C.byref(n))
    return n.value


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class GpuSim:
    """One pansim_gb300 context on a snapshot.  Host arrays of the snapshot
    are read at creation; download() writes the device state back into them."""

    def __init__(self, snap, device=0):
        self.snap = snap
        self._structs = snap.structs()
        m, a, lo, p, r = self._structs
        h = C.c_void_p()
        rc = lib().psim_create(device, C.byref(m), C.byref(a), C.byref(lo), C.byref(p), C.byref(r), C.byref(h))
        self.h = h
        if rc != 0:
            msg = lib().psim_last_error(h).decode() if h else "psim_create failed"
            if h:
                lib().psim_destroy(h)
                self.h = None
            raise PsimError("psim_create: %d %s" % (rc, msg))

    def _ck(self, rc, what):
        if rc != 0:
            raise PsimError("%s: %d %s" % (what, rc, lib().psim_last_error(self.h).decode()))

    def close(self):
        if getattr(self, "h", None):
            lib().psim_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # phases
    def movement(self, t):
        self._ck(lib().psim_movement(self.h, t), "movement")

    def regroup(self):
        self._ck(lib().psim_regroup(self.h), "regroup")

    def infect(self, t, v=0):
        self._ck(lib().psim_infect(self.h, t, v), "infect")

    def step(self, t):
        self._ck(lib().psim_step(self.h, t), "step")

    def test(self, t):
        tpp = np.zeros(3 * self.snap.n_replicas, np.uint32)
        self._ck(lib().psim_test_day(self.h, t, _p(tpp)), "test")
        return tpp

    def progress(self, t):
        self._ck(lib().psim_progress_day(self.h, t), "progress")

    def stats(self, t):
        out = (cabi.PsimDayStats * self.snap.n_replicas)()
        self._ck(lib().psim_stats_day(self.h, t, out), "stats")
        return out

    def plan(self, t):
        self._ck(lib().psim_plan_day(self.h, t), "plan")

    def midnight(self, t):
        out = (cabi.PsimDayStats * self.snap.n_replicas)()
        self._ck(lib().psim_midnight(self.h, t, out), "midnight")
        return out

    def run_steps(self, day):
        self._ck(lib().psim_run_steps(self.h, day), "run_steps")

    def run_day(self, day):
        out = (cabi.PsimDayStats * self.snap.n_replicas)()
        self._ck(lib().psim_run_day(self.h, day, out), "run_day")
        return out

    def set_params(self):
        p = self.snap.params_struct()
        self._structs = self._structs[:3] + (p,) + self._structs[4:]
        self._ck(lib().psim_set_params(self.h, C.byref(p)), "set_params")

    def set_tracking(self, expected=True):
        self._ck(lib().psim_set_tracking(self.h, 1 if expected else 0), "set_tracking")

    def download(self):
        _, a, lo, _, _ = self._structs
        self._ck(lib().psim_download(self.h, C.byref(a), C.byref(lo)), "download")
        return self.snap

    def upload(self):
        _, a, lo, _, _ = self._structs
        self._ck(lib().psim_upload(self.h, C.byref(a), C.byref(lo)), "upload")

    def csr(self, canonical=True):
        L, N = self.snap.n_locations, self.snap.n_agents
        off = np.zeros(L + 1, np.uint32)
        ag = np.zeros(max(N, 1), np.uint32)
        self._ck(lib().psim_get_csr(self.h, 1 if canonical else 0, _p(off), _p(ag)), "csr")
        return off, ag[:N]

    def hazard(self):
        V = int(self.snap.model["n_variants"])
        out = np.zeros(self.snap.n_locations * V, np.float32)
        self._ck(lib().psim_get_hazard(self.h, _p(out), None), "hazard")
        return out

    def last_day_ms(self):
        ms = C.c_float(0)
        lib().psim_last_day_ms(self.h, C.byref(ms))
        return ms.value

    # closure rules (RuleClosure)
    def closures_init(self, rules, header, enable_closures=True):
        """rules: closures.Rule list or dicts with the closureRules.json keys."""
        from . import closures
        arr = closures.rule_array(rules)
        self._rules = arr
        self._ck(lib().psim_closures_init(self.h, arr, len(arr), header.encode(), 1 if enable_closures else 0),
                 "closures_init")

    def closures_midnight(self, t, row):
        """The closure rules on a statistics row (a psim_day_stats)."""
        self._ck(lib().psim_closures_midnight(self.h, t, C.byref(row)), "closures_midnight")

    def set_types_open(self, types, open_):
        ty = np.ascontiguousarray(types, dtype=np.uint32)
        self._ck(lib().psim_set_types_open(self.h, _p(ty), len(ty), 1 if open_ else 0), "set_types_open")

    def scale_location_weights(self, coef, divide):
        self._ck(lib().psim_scale_location_weights(self.h, float(coef), 1 if divide else 0), "scale_location_weights")

    def closures_status(self):
        n = C.c_uint32(0)
        lib().psim_closures_status(self.h, None, None, C.byref(n))
        act = np.zeros(max(n.value, 1), np.uint8)
        op = np.zeros(max(n.value, 1), np.uint8)
        self._ck(lib().psim_closures_status(self.h, _p(act), _p(op), C.byref(n)), "closures_status")
        return act[: n.value].astype(bool), op[: n.value].astype(bool)

    # immunization
    def immunization_init(self, imm):
        """imm: cabi.PsimImmunization (pansim_gb300.immunization.options) or None."""
        self._imm = imm
        self._ck(lib().psim_immunization_init(self.h, C.byref(imm) if imm is not None else None),
                 "immunization_init")

    def immunize(self, t):
        n = C.c_uint32(0)
        self._ck(lib().psim_immunize_day(self.h, t, C.byref(n)), "immunize")
        return n.value

    # non-COVID hospitalization and death
    def other_disease_init(self, od):
        """od: cabi.PsimOtherDisease (cabi.other_disease_options) or None."""
        self._od = od
        self._ck(lib().psim_other_disease_init(self.h, C.byref(od) if od is not None else None),
                 "other_disease_init")

    def other_disease(self, t):
        self._ck(lib().psim_other_disease_day(self.h, t), "other_disease")

    def get_params(self):
        p = cabi.PsimParams()
        self._ck(lib().psim_get_params(self.h, C.byref(p)), "get_params")
        return p

    def get_events(self):
        n = C.c_uint32(0)
        off = np.zeros(int(self.snap.model["n_agent_types"]) * 28 + 1, np.uint32)
        self._ck(lib().psim_get_events(self.h, _p(off), None, None, None, None, None, 0, C.byref(n)), "get_events")
        ne = n.value
        ev = dict(event_offset=off, ev_loc_type=np.zeros(ne, np.uint32), ev_chance=np.zeros(ne, np.float32),
                  ev_start=np.zeros(ne, np.uint16), ev_end=np.zeros(ne, np.uint16), ev_duration=np.zeros(ne, np.uint16))
        self._ck(lib().psim_get_events(self.h, _p(off), _p(ev["ev_loc_type"]), _p(ev["ev_chance"]), _p(ev["ev_start"]),
                                       _p(ev["ev_end"]), _p(ev["ev_duration"]), ne, C.byref(n)), "get_events")
        return ev

    def set_profiling(self, on=True):
        self._ck(lib().psim_set_profiling(self.h, 1 if on else 0), "set_profiling")

    def day_kernel_ms(self):
        """Of the last profiled day, from the kernels' timeline stamps: the
        first movement kernel, the step kernel's rebuilds, draws, queues +
        decisions, and the time between the kernels (ms, summed)."""
        ms = np.zeros(5, np.float32)
        self._ck(lib().psim_day_kernel_ms(self.h, _p(ms)), "day_kernel_ms")
        return ms

    def day_timeline(self):
        """Per step of the last profiled day (rows), microseconds: the step
        kernel's span, its rebuild's listing and slots, the draws, the queue,
        the decisions (0 where the phase did not run), the time since the
        previous kernel ended."""
        us = np.zeros((self.snap.steps_per_day, 7), np.float32)
        self._ck(lib().psim_day_timeline(self.h, _p(us)), "day_timeline")
        return us

    def day_counts(self):
        """Of the last profiled day: agent-list entries the draws expanded,
        those at a location with a nonzero ratio, agents queued for a
        decision, steps whose queue passed over the agents, steps that rebuilt
        the agent list, locations and agents those rebuilds listed."""
        out = np.zeros(7, np.uint64)
        self._ck(lib().psim_day_counts(self.h, _p(out)), "day_counts")
        return out

    def launch_count(self):
        n = C.c_uint64(0)
        lib().psim_launch_count(self.h, C.byref(n))
        return n.value

    def stream(self):
        s = C.c_void_p()
        lib().psim_stream_handle(self.h, C.byref(s))
        return s.value

    def time_step_kernels(self, t):
        ms = np.zeros(3, np.float32)
        self._ck(lib().psim_time_step_kernels(self.h, t, _p(ms)), "time_step_kernels")
        return ms

    def set_tuning(self, agg_count=0, agg_slot=0, blocks_per_sm=4, variant=3, scan_items=4, scan_mode=2):
        t = cabi.PsimTuning(agg_count, agg_slot, blocks_per_sm, variant, scan_items, scan_mode)
        self._ck(lib().psim_set_tuning(self.h, C.byref(t)), "set_tuning")

    def get_tuning(self):
        t = cabi.PsimTuning()
        self._ck(lib().psim_get_tuning(self.h, C.byref(t)), "get_tuning")
        return dict(agg_count=t.agg_count, agg_slot=t.agg_slot, blocks_per_sm=t.blocks_per_sm, variant=t.variant,
                    scan_items=t.scan_items, scan_mode=t.scan_mode)

    # differentiable calibration
    def set_type_weights(self, w_by_type, slot_of_type=None):
        w = np.ascontiguousarray(w_by_type, np.float32)
        assert w.shape == (256,)
        sl = None if slot_of_type is None else np.ascontiguousarray(slot_of_type, np.int8)
        self._ck(lib().psim_set_type_weights(self.h, _p(w), _p(sl)), "set_type_weights")

    def set_replica_k(self, k):
        kk = np.ascontiguousarray(k, np.float64)
        self._ck(lib().psim_set_replica_k(self.h, _p(kk)), "set_replica_k")

    def set_adjoint(self, on, weights=None):
        w = None if weights is None else np.ascontiguousarray(weights, np.float64)
        self._ck(lib().psim_set_adjoint(self.h, 1 if on else 0, _p(w)), "set_adjoint")

    def gradient(self, reset=True):
        out = np.zeros(25, np.float64)
        self._ck(lib().psim_get_gradient(self.h, _p(out), 1 if reset else 0), "get_gradient")
        return out

    def checkpoint_save(self, slot):
        self._ck(lib().psim_checkpoint_save(self.h, slot), "checkpoint_save")

    def checkpoint_restore(self, slot):
        self._ck(lib().psim_checkpoint_restore(self.h, slot), "checkpoint_restore")

    def checkpoint_drop(self, slot):
        self._ck(lib().psim_checkpoint_drop(self.h, slot), "checkpoint_drop")

    def checkpoint_free(self):
        self._ck(lib().psim_checkpoint_free(self.h), "checkpoint_free")

    def checkpoint_bytes(self):
        n = C.c_uint64(0)
        lib().psim_checkpoint_bytes(self.h, C.byref(n))
        return n.value

    def bounded_wait_selftest(self, iters):
        return lib().psim_bounded_wait_selftest(self.h, iters)

    def last_error(self):
        return lib().psim_last_error(self.h).decode()
