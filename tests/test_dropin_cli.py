"""The reference's command-line programs run unchanged on this library.

oracle/dropin/flam3_render_forward.c is the binding a libflam3 maintainer
adds: flam3_render and flam3_render_memory_required hand the call to
libflam3gpu.  `make -C oracle dropin` compiles the reference's library and
its unmodified flam3-render.c and flam3-animate.c with that binding in place
of the reference's own flam3_render (flam3-render.c:345,
flam3-animate.c:234-248).  The programs are built where the reference tree
is; the GPU hosts have none (and no cross-compiler for them is here), so they
run in this container, without a GPU: each program's first flam3_render
call reaches libflam3gpu, which reports the missing device, and the program
takes the reference's error path.  The same programs linked to the
reference's CPU library render the same genome file."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "oracle", "_ref")
GPU_RENDER = os.path.join(REF, "flam3-render-gpu")
GPU_ANIMATE = os.path.join(REF, "flam3-animate-gpu")

pytestmark = pytest.mark.skipif(not os.path.exists(GPU_RENDER), reason="drop-in CLIs not built on this machine")

FLAMES = """<flames>
<flame name="a" time="0" size="64 48" center="0 0" scale="20" quality="5" oversample="1" filter="0.5" estimator_radius="0">
  <xform weight="0.5" color="0" linear="1" coefs="0.5 0 0 0.5 0 0"/>
  <xform weight="0.5" color="1" spherical="1" coefs="0.5 0 0 0.5 0.5 0"/>
  <color index="0" rgb="255 0 0"/><color index="255" rgb="0 0 255"/>
</flame>
<flame name="b" time="2" size="64 48" center="0 0" scale="20" quality="5" oversample="1" filter="0.5" estimator_radius="0">
  <xform weight="0.5" color="0" linear="1" coefs="0.4 0.1 -0.1 0.4 0 0"/>
  <xform weight="0.5" color="1" spherical="1" coefs="0.5 0 0 0.5 0.4 0.1"/>
  <color index="0" rgb="0 255 0"/><color index="255" rgb="255 255 0"/>
</flame>
</flames>
"""


def run(prog, tmp_path, **env):
    inp = tmp_path / "in.flam3"
    inp.write_text(FLAMES)
    e = dict(os.environ, format="ppm", verbose="0", **env)
    with open(inp) as f:
        return subprocess.run([prog], stdin=f, env=e, cwd=tmp_path, capture_output=True, text=True, timeout=120)


def symbols(prog):
    out = subprocess.run(["nm", prog], capture_output=True, text=True, check=True).stdout
    return {line.split()[-1]: line.split()[-2] for line in out.splitlines() if len(line.split()) >= 2}


@pytest.mark.parametrize("prog", [GPU_RENDER, GPU_ANIMATE])
def test_relinked_cli_binds_flam3_render_to_libflam3gpu(prog):
    sym = symbols(prog)
    # the forwarder defines flam3_render; the reference's own is renamed aside
    assert sym.get("flam3_render") == "T" and sym.get("flam3_render_cpu") == "T"
    assert sym.get("flam3_render_memory_required") == "T"
    assert sym.get("flam3gpu_render") == "U" and sym.get("flam3gpu_render_memory_required") == "U"
    ldd = subprocess.run(["ldd", prog], capture_output=True, text=True).stdout
    assert "libflam3gpu.so" in ldd and "not found" not in ldd


def test_relinked_flam3_render_reaches_the_library(tmp_path):
    r = run(GPU_RENDER, tmp_path, out=str(tmp_path / "o.ppm"))
    if "no CUDA device" not in r.stderr:
        pytest.skip("a GPU is present: the relinked program renders instead")
    assert r.returncode == 1
    assert "flam3gpu: no CUDA device available" in r.stderr
    assert "error rendering image" in r.stderr


def test_relinked_flam3_animate_reaches_the_library(tmp_path):
    r = run(GPU_ANIMATE, tmp_path, begin="0", end="1", prefix=str(tmp_path / "f"))
    if "no CUDA device" not in r.stderr:
        pytest.skip("a GPU is present: the relinked program renders instead")
    assert r.returncode != 0
    assert "flam3gpu: no CUDA device available" in r.stderr


def test_cpu_linked_cli_renders_the_same_file(tmp_path):
    r = run(os.path.join(REF, "flam3-render"), tmp_path, out=str(tmp_path / "o.ppm"))
    assert r.returncode == 0, r.stderr
    data = (tmp_path / "o.ppm").read_bytes()
    assert data.startswith(b"P6") and len(data) > 64 * 48 * 3
