"""The C ABI library builds, loads and exports every declared symbol (CPU; no GPU calls)."""
import ctypes
import subprocess

from pansim_gb300 import cabi, native
from pansim_gb300.build import build


def test_library_builds_and_exports_header_symbols():
    path = build()
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    declared = native.header_symbols()
    assert len(declared) >= 25
    missing = [s for s in declared if s not in exported]
    assert not missing, missing


def test_struct_layout_matches_bindings():
    sizes = native.abi_sizes()
    mine = [ctypes.sizeof(s) for s in cabi.ABI_STRUCTS]
    assert sizes == mine, (sizes, mine)


def test_version_string():
    assert b"sm_103a" in native.lib().psim_version()


def _create(snap):
    from pansim_gb300.native import lib
    m, a, lo, p, r = snap.structs()
    h = ctypes.c_void_p()
    rc = lib().psim_create(0, ctypes.byref(m), ctypes.byref(a), ctypes.byref(lo), ctypes.byref(p), ctypes.byref(r),
                           ctypes.byref(h))
    msg = lib().psim_last_error(h).decode() if h else ""
    if h:
        lib().psim_destroy(h)
    return rc, msg


def test_create_validates_snapshot_on_host():
    """psim_create rejects inconsistent snapshots before touching a device."""
    import numpy as np
    from tests.helpers import small_snapshot
    s = small_snapshot(500, 120)
    bad = s.copy()
    bad.agents["location"][3] = bad.n_locations + 5
    rc, msg = _create(bad)
    assert rc == -4 and "location out of range" in msg
    bad = s.copy()
    bad.agents["poss_loc"][7] = np.uint32(0xFFFFFFF0)
    rc, msg = _create(bad)
    assert rc == -4
    bad = s.copy()
    bad.model["tr_next"][0] = 99
    rc, msg = _create(bad)
    assert rc == -4 and "transition" in msg
    bad = s.copy()
    bad.reps["cemetery"][0] = 0
    rc, msg = _create(bad)
    assert rc == -4 and "cemetery" in msg


def test_create_without_device_fails_cleanly():
    """A valid snapshot passes validation; without a GPU the call reports a CUDA error."""
    from pansim_gb300.native import device_count
    from tests.helpers import small_snapshot
    if device_count() > 0:
        return
    rc, msg = _create(small_snapshot(500, 120))
    assert rc == -2, (rc, msg)


def test_create_rejects_empty_population_and_shared_replica_locations():
    import numpy as np
    from pansim_gb300 import snapshot as snp
    from tests.helpers import small_snapshot
    s = small_snapshot(300, 80)
    empty = s.copy()
    for k in list(empty.agents):
        if k == "loc_offset":
            empty.agents[k] = np.zeros(1, np.uint32)
        else:
            empty.agents[k] = empty.agents[k][:0]
    empty.reps["agent_offset"][:] = [0, 0]
    rc, msg = _create(empty)
    assert rc == -1 and "no agents" in msg
    a, b = small_snapshot(300, 80, seed=1), small_snapshot(200, 60, seed=2)
    batch = snp.concat([a, b], [1, 2], [3e-4, 3e-4])
    batch.agents["location"][5] = batch.reps["loc_offset"][1] + 3  # an agent of replica 0 placed in replica 1
    rc, msg = _create(batch)
    assert rc == -4 and "outside its replica" in msg


def test_noalloc_limit_checks_on_host():
    """psim_csr_build_noalloc rejects sizes beyond its fixed scratch before any CUDA call,
    and its message describes the last call only."""
    L = native.lib()
    rc = L.psim_csr_build_noalloc(None, 0, (1 << 21) + 1, None, None, None)
    assert rc == -1
    assert b"n_locations must be" in L.psim_noalloc_last_error()
    rc = L.psim_csr_build_noalloc(None, 0, 0, None, None, None)
    assert rc == -1
    rc = L.psim_csr_build_noalloc(None, 0xFFFFFFFF, 16, None, None, None)
    assert rc == -1 and b"n_agents must be" in L.psim_noalloc_last_error()
    rc = L.psim_csr_build_noalloc(None, 10, 16, None, None, None)
    assert rc == -1 and b"null device pointer" in L.psim_noalloc_last_error()
