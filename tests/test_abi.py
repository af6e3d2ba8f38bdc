"""The struct layouts of include/flam3_gpu.h and flam3_gb300/abi.py match
the reference's flam3.h (offsets printed from the real header and committed
as tests/golden/abi_offsets.txt)."""
import ctypes as C
import os
import subprocess

import pytest

from flam3_gb300 import abi

GOLD = os.path.join(os.path.dirname(__file__), "golden", "abi_offsets.txt")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def golden():
    out = {}
    for line in open(GOLD):
        kind, name, val = line.split()
        out[(kind, name)] = int(val)
    return out


def test_python_mirror_matches_reference_layout():
    g = golden()
    types = {t.__name__: t for t in (abi.randctx, abi.flam3_palette_entry, abi.stat_struct, abi.flam3_xform,
                                     abi.flam3_genome, abi.flam3_frame)}
    n = 0
    for (kind, name), val in g.items():
        if kind == "sizeof":
            assert C.sizeof(types[name]) == val, name
        else:
            t, f = name.split(".")
            assert getattr(types[t], f).offset == val, name
        n += 1
    assert n > 60


def test_c_mirror_matches_reference_layout(tmp_path):
    exe = tmp_path / "abi_mine"
    subprocess.run(["gcc", "-O0", "-I", os.path.join(ROOT, "include"), "-o", str(exe),
                    os.path.join(ROOT, "oracle", "abi_offsets.c")], check=True)
    mine = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    assert mine == open(GOLD).read()
