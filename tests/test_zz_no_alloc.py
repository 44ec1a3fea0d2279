"""psim_csr_build_noalloc against the context path's CSR (gpu).

The entry point serves callers that cannot call cudaMalloc (device memory
owned by another allocator, plug-ins that must not grow the footprint,
loops where an allocation would synchronize the device): it builds the
location CSR into caller-owned buffers using a fixed scratch array compiled
into the library.  Two calls in a row, on two different location arrays,
must each give the CSR that psim_regroup + psim_get_csr give: identical
offsets and, location by location, the same agents (the order inside a
location is unspecified, so each segment is compared sorted, which is the
canonical order of the context path).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib, loc_host, n_locations, torch):
    dev = torch.device("cuda", 0)
    d_loc = torch.from_numpy(loc_host.astype(np.uint32).view(np.int32)).to(dev)
    d_off = torch.zeros(n_locations + 1, dtype=torch.int32, device=dev)
    d_ag = torch.full((len(loc_host),), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = lib.psim_csr_build_noalloc(C.c_void_p(d_loc.data_ptr()), len(loc_host), n_locations,
                                    C.c_void_p(d_off.data_ptr()), C.c_void_p(d_ag.data_ptr()),
                                    C.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.psim_noalloc_last_error()
    torch.cuda.synchronize(dev)
    off = d_off.cpu().numpy().view(np.uint32).copy()
    ag = d_ag.cpu().numpy().view(np.uint32).copy()
    return off, ag


def _segments_sorted(off, ag):
    out = ag.copy()
    for l in np.nonzero(np.diff(off.astype(np.int64)) > 1)[0]:
        out[off[l]:off[l + 1]] = np.sort(ag[off[l]:off[l + 1]])
    return out


def test_noalloc_csr_matches_context_path_on_two_calls(gpu_lib):
    torch = pytest.importorskip("torch")
    from pansim_gb300 import native, synth
    lib = native.lib()
    s = synth.make_snapshot(50000, 12000, seed=4, initial_infected_frac=0.02)
    g = native.GpuSim(s)
    L = s.n_locations
    assert L <= (1 << 21)
    # call 1: the initial positions
    off_ref, ag_ref = g.csr(canonical=True)
    off, ag = _noalloc(lib, s.agents["location"], L, torch)
    assert np.array_equal(off, off_ref)
    assert np.array_equal(_segments_sorted(off, ag), ag_ref)
    # call 2: positions after half a day of steps (the scratch keeps call 1's contents)
    g.midnight(0)
    for t in range(70):
        g.step(t)
    g.download()
    off_ref2, ag_ref2 = g.csr(canonical=True)
    off2, ag2 = _noalloc(lib, s.agents["location"], L, torch)
    assert not np.array_equal(off_ref2, off_ref)
    assert np.array_equal(off2, off_ref2)
    assert np.array_equal(_segments_sorted(off2, ag2), ag_ref2)


def _numpy_csr(loc, L):
    """Offsets and agents (ascending id inside a location) of the in-range entries."""
    loc = loc.astype(np.int64)
    keep = np.nonzero(loc < L)[0]
    counts = np.bincount(loc[keep], minlength=L)
    off = np.zeros(L + 1, np.uint64)
    off[1:] = np.cumsum(counts)
    order = keep[np.argsort(loc[keep], kind="stable")]
    return off.astype(np.uint32), order.astype(np.uint32)


def test_noalloc_edge_cases(gpu_lib):
    """Maximum location count, out-of-range locations left out, and no agents."""
    torch = pytest.importorskip("torch")
    from pansim_gb300 import native
    lib = native.lib()
    rng = np.random.default_rng(11)
    Lmax = 1 << 21
    # the largest location count: the per-tile prefix loop of the scan is longest
    loc = rng.integers(0, Lmax, 5000).astype(np.uint32)
    loc[:3] = [0, Lmax - 1, Lmax - 1]
    off, ag = _noalloc(lib, loc, Lmax, torch)
    off_ref, ag_ref = _numpy_csr(loc, Lmax)
    assert np.array_equal(off, off_ref)
    assert np.array_equal(_segments_sorted(off, ag), ag_ref)
    # some agents at locations >= n_locations: left out, offsets[L] < n_agents,
    # only the prefix of the agent list is written
    L = 3000
    loc = rng.integers(0, L, 20000).astype(np.uint32)
    loc[rng.random(20000) < 0.1] = L + 7
    loc[5] = 0xFFFFFFFF
    off, ag = _noalloc(lib, loc, L, torch)
    off_ref, ag_ref = _numpy_csr(loc, L)
    assert off[L] == int(np.sum(loc < L)) < len(loc)
    assert np.array_equal(off, off_ref)
    assert np.array_equal(_segments_sorted(off, ag)[: off[L]], ag_ref)
    assert np.all(ag[off[L]:] == 0xFFFFFFFF)  # untouched: the buffer's fill value
    # no agents: every offset is 0
    off, ag = _noalloc(lib, np.zeros(0, np.uint32), 1000, torch)
    assert off.shape == (1001,) and not off.any()
