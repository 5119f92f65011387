"""CPU checks of the drop-in boundary: the library builds, loads and
exports every function that include/fmd.h and include/fmdg.h declare."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    txt = re.sub(r"#define[^\n]*(\\\n[^\n]*)*", "", txt)
    names = set(re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", txt))
    keep = {n for n in names if n.startswith(("fmd_", "_fmd_", "fmdg_"))}
    return keep - {"fmd_EventHandler_t"}


@pytest.mark.parametrize("header", ["fmd.h", "fmdg.h"])
def test_exports(lib, header):
    names = declared(header)
    assert len(names) > 10
    missing = [n for n in sorted(names) if not lib.has(n)]
    assert not missing, missing


def test_version(lib):
    import ctypes
    assert lib.fmd_version_getMajor() == 0 and lib.fmd_version_getMinor() == 4
    p = lib.fmd_version_getString()
    assert ctypes.string_at(p).decode().startswith("0.4.0")
