"""CPU-only checks of the C-ABI library: it builds, loads and exports every
entry point that include/vx3g.h declares (no compute calls without a GPU)."""

import ctypes
import os
import re

from vx3g import abi, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "vx3g.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(vx3g_[a-z_0-9]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib_path = build.build()
    lib = ctypes.CDLL(lib_path)
    names = declared_functions()
    assert len(names) >= 19
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(abi.EXPORTS) <= set(names)


def test_loader_is_loud_when_library_missing(tmp_path):
    import pytest
    saved = abi._lib
    abi._lib = None
    try:
        with pytest.raises(RuntimeError):
            abi.load(str(tmp_path / "nope.so"))
    finally:
        abi._lib = saved
