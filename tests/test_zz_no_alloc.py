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
    d_loc = torch.from_numpy(loc_host.astype(np.int32).view(np.int32)).to(dev)
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


def test_noalloc_rejects_oversize(gpu_lib):
    from pansim_gb300 import native
    lib = native.lib()
    rc = lib.psim_csr_build_noalloc(None, 0, (1 << 21) + 1, None, None, None)
    assert rc == -1
    assert b"n_locations must be" in lib.psim_noalloc_last_error()
