"""The reference's policy concept over the C ABI (include/gb300_policies.h).

CPU: the reference's own Simulation (include/simulation.h), instantiated with
Gb300Movement / Gb300Infection / Gb300Testing / Gb300Closure through
include/gb300_config_types.h, compiles against the reference's headers
(runSimulation and every policy member instantiated).

GPU: the four policies in a stand-in Simulation with the reference's
container names and element layouts (tests/adapter/adapter_run.cpp), run in
runSimulation's order -- the device steps, and Simulation::updateAgents on the
host containers between them -- end bit for bit where the oracle's run of the
same days ends.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from oracle import binding as ob
from tests.helpers import diff_state, small_snapshot

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_adapters_compile_inside_the_reference_simulation():
    from oracle import ref_build
    res = ref_build.check_adapters()
    if res is None:
        pytest.skip("reference tree not available")
    ok, out = res
    assert ok, out


def _driver():
    from pansim_gb300 import build as pb
    lib = pb.build()
    olib = ob.build()
    out_dir = os.path.join(ROOT, "tests", "adapter", "_build")
    os.makedirs(out_dir, exist_ok=True)
    so = os.path.join(out_dir, "libadapter_run.so")
    src = os.path.join(ROOT, "tests", "adapter", "adapter_run.cpp")
    deps = [src, os.path.join(ROOT, "include", "gb300_policies.h"), lib, olib]
    if not os.path.exists(so) or any(os.path.getmtime(d) > os.path.getmtime(so) for d in deps):
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-o", so, src,
               "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "oracle"),
               "-L", os.path.dirname(lib), "-lpansim_gb300", "-Wl,-rpath," + os.path.dirname(lib),
               "-L", os.path.dirname(olib), "-lpsim_oracle", "-Wl,-rpath," + os.path.dirname(olib)]
        subprocess.run(cmd, check=True, capture_output=True, text=True)
    d = C.CDLL(so)
    d.adapter_run.argtypes = [C.c_void_p] * 4 + [C.c_uint32, C.c_char_p, C.c_int]
    return d


@pytest.mark.gpu
@pytest.mark.parametrize("policy", [0, 3])
def test_adapters_in_run_simulation_order_match_the_oracle(gpu_lib, policy):
    days = 3
    snap = small_snapshot(n=12000, locs=3000, initial_infected_frac=0.02, quarantine_policy=policy,
                          testing=policy > 0)
    s_ad, s_or = snap.copy(), snap.copy()
    o = ob.Oracle(s_or)
    for d in range(days):
        o.run_day(d)
    o.close()
    m, a, lo, p, r = s_ad.structs()
    err = C.create_string_buffer(512)
    rc = _driver().adapter_run(C.addressof(m), C.addressof(a), C.addressof(lo), C.addressof(p), days, err, 512)
    assert rc == 0, err.value
    # the policies' own state (countdowns, last tests, no-work flags) lives in
    # the policies, not in the reference's containers: compared through its
    # effects on the next days
    fields = [k for k in s_or.agents if k not in ("steps_until_move", "last_test", "no_work", "imm_round")
              and k in s_ad.agents and isinstance(s_ad.agents[k], np.ndarray) and k not in
              ("type", "age", "band", "prog_id", "symptom_scaling", "loc_offset", "poss_loc", "poss_type", "precond",
               "sex", "symptom_scaling_v")]
    assert diff_state(s_or, s_ad, fields) == []
