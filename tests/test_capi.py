"""CPU tests of the C ABI library: it builds, loads, and exports every symbol the header declares."""
import ctypes
import re
import subprocess
from pathlib import Path

import pytest

from phasefield_gb300 import build, capi

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols() -> set[str]:
    syms = set()
    for hdr in (ROOT / "include").glob("*.h"):
        text = hdr.read_text()
        for m in re.finditer(r"\b(ppf_[a-z0-9_]+)\s*\(", text):
            syms.add(m.group(1))
    return syms


@pytest.fixture(scope="module")
def lib_path():
    return build.build()


def test_library_exports_every_declared_symbol(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib_path)], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = declared_symbols() - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"


def test_library_loads_and_binds(lib_path):
    lib = capi.load()
    for name in declared_symbols():
        assert hasattr(lib, name)


def test_python_binding_list_matches_header():
    assert set(capi.EXPORTED) <= declared_symbols()
    assert declared_symbols() <= set(capi.EXPORTED) | {"ppf_last_error"}


def test_create_rejects_bad_arguments_without_gpu(lib_path):
    lib = capi.load()
    h = ctypes.c_void_p()
    m = capi.MeshDesc()
    m.dim = 5  # invalid
    rc = lib.ppf_create(ctypes.byref(m), None, 0, None, 0, b"allen_cahn", None, 0, 0.0, ctypes.byref(h))
    assert rc == capi.PPF_ERR_ARG
    assert not h.value
    assert b"dim" in lib.ppf_last_error(None)
