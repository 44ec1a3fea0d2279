"""Device allocation failures (gpu): psim_create and psim_checkpoint_save
report PSIM_ERR_ALLOC and leave nothing allocated behind.

The reference raises only at initialization and keeps going without checks
afterwards (simulation.h:762-765); here every device allocation of the
library goes through one place, and the test hook psim_set_alloc_fault makes
the n-th one fail as if the device were full.  For a range of n, creation
fails cleanly (the context is returned for psim_last_error, psim_destroy
frees what it took) until n exceeds what a context needs; the device's free
memory ends where it started.  A checkpoint whose allocation fails leaves the
context usable.
"""
import ctypes as C

import pytest

from tests.helpers import small_snapshot

pytestmark = pytest.mark.gpu


def _create(lib, snap):
    m, a, lo, p, r = snap.structs()
    h = C.c_void_p()
    rc = lib.psim_create(0, C.byref(m), C.byref(a), C.byref(lo), C.byref(p), C.byref(r), C.byref(h))
    msg = lib.psim_last_error(h).decode() if h else ""
    return rc, msg, h, (m, a, lo, p, r)


def test_create_and_checkpoint_fail_cleanly(gpu_lib):
    torch = pytest.importorskip("torch")
    from pansim_gb300 import native
    lib = native.lib()
    snap = small_snapshot(n=4000, locs=1000, initial_infected_frac=0.02)
    # a first context brings up the CUDA context itself (not counted below)
    rc, msg, h, keep = _create(lib, snap)
    assert rc == 0, msg
    lib.psim_destroy(h)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    failed = 0
    for n in [0, 1, 2, 5, 9, 17, 33, 48, 64, 96, 128, 4096]:
        lib.psim_set_alloc_fault(n)
        try:
            rc, msg, h, keep = _create(lib, snap)
        finally:
            lib.psim_set_alloc_fault(-1)
        if rc == 0:
            assert n >= 17  # a context takes dozens of allocations
            lib.psim_destroy(h)
            break
        assert rc == -3 and "cudaMalloc" in msg, (n, rc, msg)
        failed += 1
        lib.psim_destroy(h)
    assert failed >= 5
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert abs(free1 - free0) <= 2 << 20, (free0, free1)
    # a checkpoint that cannot be allocated: error, and the context runs on
    g = native.GpuSim(snap.copy())
    g.run_day(0)
    lib.psim_set_alloc_fault(0)
    try:
        rc = lib.psim_checkpoint_save(g.h, 3)
    finally:
        lib.psim_set_alloc_fault(-1)
    assert rc == -3 and b"checkpoint" in lib.psim_last_error(g.h)
    g.run_day(1)
    g.checkpoint_save(3)
    g.run_day(2)
    g.checkpoint_restore(3)
    g.close()
