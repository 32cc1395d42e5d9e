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


def test_ctypes_structs_match_the_header(tmp_path):
    """The ctypes mirrors in abi.py have the C structs' sizes and field offsets."""
    import subprocess
    fields = {"vx3g_material": (abi.Material, ["E", "fail_stress", "model", "is_measured", "thermal_on_after",
                                                "cilia", "cilia_on_after", "remove_after"]),
              "vx3g_robot_desc": (abi.RobotDesc, ["lattice", "materials", "vox_size", "floor_enabled",
                                                  "volume_effects", "slow_damping", "log10E", "force_field",
                                                  "enable_cilia", "cilia_base", "cilia_shift", "enable_detach",
                                                  "secondary_experiment"]),
              "vx3g_batch_desc": (abi.BatchDesc, ["robots", "precision", "graph_chunk"])}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "vx3g.h"', "int main(void) {"]
    for st, (_, names) in fields.items():
        lines.append(f'printf("%zu\\n", sizeof({st}));')
        lines += [f'printf("%zu\\n", offsetof({st}, {n}));' for n in names]
    lines.append('printf("%zu\\n", sizeof(vx3g_math_token));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    want = []
    for st, (cls, names) in fields.items():
        want.append(ctypes.sizeof(cls))
        want += [getattr(cls, n).offset for n in names]
    from vx3g import workloads as wl
    want.append(wl.math_tokens(("mtCONST", 0.0)).dtype.itemsize)
    assert got == want
