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
