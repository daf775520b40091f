"""Host-side checks of the C ABI library that need no GPU: it builds, loads,
and exports every symbol include/bem.h declares (and nothing else)."""
import os
import re
import subprocess

from conftest import ROOT


def _declared():
    text = open(os.path.join(ROOT, "include", "bem.h")).read()
    return sorted(set(re.findall(r"BEM_API\s+[^;(]*?\b(bem_\w+)\s*\(", text)))


def test_library_builds_and_exports():
    from cc_abstemious_gb300 import build
    lib = build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    exported = sorted(set(l.split()[-1] for l in out.splitlines() if " T " in l))
    declared = _declared()
    assert declared, "no declarations parsed"
    assert set(declared) <= set(exported), set(declared) - set(exported)
    assert all(e.startswith("bem_") for e in exported), [e for e in exported if not e.startswith("bem_")]


def test_ctypes_binding_covers_header():
    from cc_abstemious_gb300 import _lib
    assert set(_declared()) == set(_lib.SIGNATURES), set(_declared()) ^ set(_lib.SIGNATURES)
    lib = _lib.load()
    assert lib.bem_version().startswith(b"bem_gb300")


def test_no_device_reports_error():
    """Without a GPU (this container) context creation fails with a status,
    not a crash; on a GPU machine it succeeds."""
    import ctypes as C
    from cc_abstemious_gb300 import _lib
    lib = _lib.load()
    h = C.c_void_p()
    st = lib.bem_ctx_create(0, C.byref(h))
    if st == 0:
        lib.bem_ctx_destroy(h)
    else:
        assert st == 6 and not h.value
