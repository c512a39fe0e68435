"""The C ABI library loads and exports every function include/onesolver.h
declares (CPU; no compute calls)."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def declared_functions() -> list[str]:
    text = (ROOT / "include" / "onesolver.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(os_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(native):
    lib = ctypes.CDLL(str(native.LIB_PATH))
    names = declared_functions()
    assert len(names) > 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(native):
    assert set(declared_functions()) <= set(native.SIGNATURES), \
        set(declared_functions()) - set(native.SIGNATURES)


def test_abi_version_and_status_names(native):
    L = native.lib()
    assert L.os_abi_version() == 1
    assert L.os_status_string(native.OVERFLOW_MINIMISERS) == b"OVERFLOW_MINIMISERS"
