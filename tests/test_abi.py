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
