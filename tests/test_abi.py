"""The C-ABI library loads without a GPU and exports every entry point the
headers in include/ declare; the ABI table matches the header."""
import ctypes
import os
import re

import lsmlib_gb300 as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    syms = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?(?:void|int|long long|char)\s*\*?\s*(\w+)\s*\(", text, re.M):
            syms.add(m.group(1))
    return syms


def test_library_builds_and_loads():
    from lsmlib_gb300 import build as B
    B.build()
    h = L.lib()
    assert h.lsmgpu_version().startswith(b"lsmgpu")


def test_every_declared_symbol_is_exported():
    h = L.lib()
    syms = header_symbols()
    assert len(syms) > 30
    missing = [s for s in sorted(syms) if not hasattr(h, s)]
    assert not missing, missing


def test_abi_table_matches_header():
    syms = header_symbols()
    for s in L.ABI:
        assert s in syms, s
        spec = L.ABI[s]
        assert spec["ref"].startswith(("src/", "NEW")), spec["ref"]


def test_error_channel_without_gpu():
    h = L.lib()
    code, msg = L.last_error(h)
    assert code == 0
