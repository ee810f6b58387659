"""The C-ABI library loads and exports every function include/mantiis_gpu.h
declares; the Python binding covers the header.  No GPU calls."""
import re
import subprocess

from conftest import ROOT

from mantiis_gb300 import lib, native

HEADER = ROOT / "include" / "mantiis_gpu.h"


def declared():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(mgpu_[a-z_0-9]+)\s*\(", text)
    return sorted(set(names))


def test_library_loads_and_exports_all_symbols():
    L = lib()
    names = declared()
    assert len(names) >= 30
    for n in names:
        assert hasattr(L, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", str(native.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (mgpu_\w+)", out))
    assert set(names) <= exported, set(names) - exported


def test_binding_covers_header():
    assert set(declared()) == set(native.SIGNATURES)


def test_no_device_needed_for_defaults():
    p = native.default_params()
    assert p.collision == 2 and p.wall == 2 and p.max_allowed_level == 2
    assert p.tol == 1e-10 and p.dx == 1e-9 and p.fbody == 1e-8
