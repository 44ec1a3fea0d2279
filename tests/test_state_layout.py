"""The mutable state's one-block layout (psim_state_layout): host arrays laid
out this way move in one copy each way (psim_upload / psim_download), with
the same results as the per-field copies."""
import numpy as np
import pytest

from pansim_gb300 import native
from pansim_gb300.snapshot import AGENT_MUTABLE, LOC_MUTABLE
from tests.helpers import diff_state, small_snapshot, stats_rows


def packed_copy(snap):
    """A copy whose mutable arrays are views into one host block in the library's layout."""
    s = snap.copy()
    fields = [(s.agents, k) for k in AGENT_MUTABLE] + [(s.locs, k) for k in LOC_MUTABLE]
    off = native.state_layout(s.n_agents, s.n_locations, int(s.model["n_variants"]))
    buf = np.zeros(int(off[-1]), np.uint8)
    for j, (part, k) in enumerate(fields):
        a = part[k]
        v = buf[int(off[j]): int(off[j]) + a.nbytes].view(a.dtype).reshape(a.shape)
        v[...] = a
        part[k] = v
    s._block = buf
    return s


@pytest.mark.parametrize("n,locs,v", [(1, 4, 1), (3000, 800, 1), (4097, 1031, 3)])
def test_layout_covers_every_field_aligned(n, locs, v):
    snap = small_snapshot(n=n, locs=locs, n_variants=v)
    off = native.state_layout(snap.n_agents, snap.n_locations, v)
    fields = [snap.agents[k] for k in AGENT_MUTABLE] + [snap.locs[k] for k in LOC_MUTABLE]
    assert len(off) == len(fields) + 1 == 35
    assert off[0] == 0 and (off % 256 == 0).all() and (np.diff(off.astype(np.int64)) > 0).all()
    for j, a in enumerate(fields):
        assert a.nbytes <= off[j + 1] - off[j]
        assert off[j + 1] - off[j] < a.nbytes + 256


@pytest.mark.gpu
def test_packed_state_moves_in_one_copy_with_the_same_results(gpu_lib):
    snap = small_snapshot(n=12000, locs=3000, initial_infected_frac=0.02, n_variants=2)
    s_plain, s_packed = snap.copy(), packed_copy(snap)
    g_plain, g_packed = native.GpuSim(s_plain), native.GpuSim(s_packed)
    for d in range(2):
        assert stats_rows(g_plain.run_day(d)) == stats_rows(g_packed.run_day(d)), d
    g_plain.download()
    g_packed.download()
    assert diff_state(s_plain, s_packed) == []
    # an upload of the packed block restores a state, as the per-field one does
    g_packed.upload()
    g_plain.upload()
    assert stats_rows(g_plain.run_day(2)) == stats_rows(g_packed.run_day(2))
    g_plain.download()
    g_packed.download()
    assert diff_state(s_plain, s_packed) == []
