"""libflam3gpu.so loads without a GPU and exports every function that
include/*.h declares; option validation needs no device."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in sorted(f for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")):
        txt = open(os.path.join(ROOT, "include", h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"\b(flam3gpu_\w+)\s*\(", txt):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_function():
    from flam3_gb300 import _build, render

    if not os.path.exists(render._LIB_PATH):
        _build.build()
    syms = subprocess.run(["nm", "-D", "--defined-only", render._LIB_PATH], capture_output=True, text=True,
                          check=True).stdout
    exported = {line.split()[-1] for line in syms.splitlines() if " T " in line}
    names = declared_functions()
    assert len(names) >= 28
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    lib = render.load()
    for n in names:
        assert hasattr(lib, n)


def test_options_validation_without_gpu():
    from flam3_gb300 import render

    lib = render.load()
    o = render.Options()
    lib.flam3gpu_default_options(C.byref(o))
    assert o.iter_mode == 1 and o.iter_precision == 32 and o.threads_per_block == 256
    bad = render.Options.from_buffer_copy(o)
    bad.iter_precision = 16
    assert lib.flam3gpu_set_options(C.byref(bad)) != 0
    assert b"iter_precision" in lib.flam3gpu_last_error()
    bad = render.Options.from_buffer_copy(o)
    bad.threads_per_block = 100
    assert lib.flam3gpu_set_options(C.byref(bad)) != 0
    assert lib.flam3gpu_set_options(C.byref(o)) == 0
    assert render.version().startswith("flam3-gb300")


def test_service_config_defaults_without_gpu():
    from flam3_gb300 import service

    c = service.config()
    assert c.tail_graphs == 1 and c.streams == 1 and c.use_tuning == 1 and c.tail_branches == 1
    assert c.round_samples == 0 and c.hbm_budget_bytes == 0.0
    c = service.config(round_samples=-1, streams=3)
    assert c.round_samples == -1 and c.streams == 3



def test_strip_planning_without_gpu():
    """calc_nstrips against a given budget and the strip loop's argument
    checks are host logic (flam3-render.c:35-101, 276-283)"""
    from flam3_gb300 import genome as gm, render

    F = gm.Frame(gm.small_genome(3, width=64, height=40), bits=33, seed="s")
    need = render.memory_required(F)
    assert need > 0
    assert render.calc_nstrips(F, need) == 1
    assert render.calc_nstrips(F, need / 3.5) == 4
    with pytest.raises(render.Flam3GpuError, match="more strips than rows"):
        render.render_strips(F, 41)


def test_analysis_helpers_need_a_random_context():
    """flam3gpu_dimension / flam3gpu_lyapunov refuse a NULL context before
    touching the device"""
    from flam3_gb300 import genome as gm, render

    lib = render.load()
    G = gm.small_genome(3)
    assert lib.flam3gpu_dimension(C.byref(G.g), 1000, 0, None) == -1.0
    assert b"ISAAC" in lib.flam3gpu_last_error()
    assert lib.flam3gpu_lyapunov(C.byref(G.g), 10, None) == -1.0


def test_struct_mirrors_match_the_library_without_gpu():
    """The Python mirrors of flam3gpu_options and flam3gpu_service_config are
    at least as large as the library's structs (its default writers stop
    inside them: canary bytes after the mirror stay untouched) and the
    defaults land in the mirrored fields."""
    from flam3_gb300 import render, service

    lib = render.load()
    for cls, fill in ((render.Options, lib.flam3gpu_default_options),
                      (service.ServiceConfig, service._lib().flam3gpu_service_default_config)):
        n = C.sizeof(cls)
        buf = (C.c_ubyte * (n + 64))(*([0xAB] * (n + 64)))
        fill(C.cast(buf, C.POINTER(cls)))
        assert bytes(buf[n:]) == b"\xab" * 64, cls.__name__
    o = render.Options()
    lib.flam3gpu_default_options(C.byref(o))
    assert (o.shuffle_every, o.chain_samples, o.tail_chain_samples, o.tail_wave_pct, o.test_exchange_stall) == \
        (3, 0, 0, 0, 0)
    c = service.config()
    assert c.order == 1 and c.max_inflight == 2


def test_pass_record_mirror_without_gpu():
    """The tests' ctypes mirror of the iterate kernel's pass record has the
    library's size (flam3gpu_pass_bytes is host code)."""
    from flam3_gb300 import render
    from test_gpu_plan import F3GPass

    assert C.sizeof(F3GPass) == render.load().flam3gpu_pass_bytes()
