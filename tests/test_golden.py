"""Golden fixtures produced by the reference's own C++ (tests/golden/make_golden.py).

CPU: the oracle reproduces them bit for bit.  GPU: the CUDA path through the
C ABI reproduces them bit for bit, including the final CSR in canonical order.
"""
import os

import numpy as np
import pytest

from oracle import binding as ob
from pansim_gb300 import snapshot as snp
from pansim_gb300.snapshot import AGENT_MUTABLE, LOC_MUTABLE

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SCENARIOS = ["plain", "policies", "curfew_closures"]


def _load(name):
    s = snp.load(os.path.join(HERE, name + "_input.npz"))
    ref = np.load(os.path.join(HERE, name + "_reference.npz"))
    return s, ref


def _neutral(s, k):
    """Fields newer than the fixtures (immunization) keep their neutral values
    in these scenarios, which run no immunization."""
    if k == "imm_round":
        return np.zeros(s.n_agents, np.uint8)
    V = int(s.model["n_variants"])
    return np.tile(s.agents["symptom_scaling"], V)


def _check(s, ref):
    bad = []
    for k in AGENT_MUTABLE:
        want = ref["agents/" + k] if "agents/" + k in ref.files else _neutral(s, k)
        if not np.array_equal(s.agents[k], want):
            bad.append(k)
    for k in LOC_MUTABLE:
        if not np.array_equal(s.locs[k], ref["locs/" + k]):
            bad.append("loc." + k)
    return bad


@pytest.mark.parametrize("name", SCENARIOS)
def test_oracle_matches_reference_golden(name):
    s, ref = _load(name)
    o = ob.Oracle(s)
    for d in range(int(ref["days"])):
        o.run_day(d)
    assert _check(s, ref) == []
    _, ag = o.csr()
    assert np.array_equal(ag, ref["csr_agents"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", SCENARIOS)
def test_gpu_matches_reference_golden(gpu_lib, name):
    from pansim_gb300.native import GpuSim
    s, ref = _load(name)
    g = GpuSim(s)
    for d in range(int(ref["days"])):
        g.run_day(d)
    g.download()
    assert _check(s, ref) == []
    _, ag = g.csr(canonical=True)
    assert np.array_equal(ag, ref["csr_agents"])
