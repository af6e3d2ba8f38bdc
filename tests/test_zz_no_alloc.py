"""flam3gpu_render_noalloc -- the render for callers that cannot call
cudaMalloc -- against the allocating drop-in flam3gpu_render, called through
the C ABI twice in a row (the static scratch array keeps the previous call's
contents, so the second call also checks that the histogram is cleared).
Tolerance as for the tail tests: every channel within one 8-bit level on at
least 99.9% of pixels (atomic-add order differs between the two renders)."""
import ctypes as C

import numpy as np
import pytest

from flam3_gb300 import abi, genome as gm, render

pytestmark = pytest.mark.gpu


def _frame(seed, est, bits=33, w=160, h=120, q=60.0):
    G = gm.small_genome(seed)
    gm.resize(G, w, h)
    G.g.sample_density = q
    G.g.estimator = est
    return gm.Frame(G, bits=bits, seed="noalloc-%d" % seed)


def _noalloc(lib, F, nchan=3):
    out = F.out_buffer(nchan)
    st = abi.stat_struct()
    r = lib.flam3gpu_render_noalloc(C.byref(F.f), out.ctypes.data, 0, nchan, 0, C.byref(st))
    return r, out, st


def _close(a, b):
    d = np.abs(a.astype(np.int64) - b.astype(np.int64))
    return float(np.mean(d <= 1))


@pytest.mark.parametrize("est,bits", [(0.0, 33), (3.0, 33), (2.0, 64)])
def test_noalloc_matches_allocating_render_twice(gpulib, est, bits):
    lib = gpulib
    lib.flam3gpu_render_noalloc.argtypes = [C.POINTER(abi.flam3_frame), C.c_void_p, C.c_int, C.c_int, C.c_int,
                                            C.POINTER(abi.stat_struct)]
    ref, st_ref = render.render(_frame(3, est, bits))
    assert ref.mean() > 1.0
    for call in range(2):
        F = _frame(3, est, bits)
        r, out, st = _noalloc(lib, F)
        assert r == 0, lib.flam3gpu_last_error()
        assert st.num_iters == st_ref.num_iters
        assert _close(out, ref) >= 0.999, (call, _close(out, ref))


def test_noalloc_refuses_renders_beyond_its_scratch(gpulib):
    lib = gpulib
    lib.flam3gpu_noalloc_capacity.restype = C.c_size_t
    cap = lib.flam3gpu_noalloc_capacity()
    assert cap == 48 << 20
    F = _frame(1, 0.0, w=2400, h=1800, q=1.0)
    r, out, st = _noalloc(lib, F)
    assert r == 1
    msg = lib.flam3gpu_last_error().decode()
    assert "scratch" in msg and str(cap) in msg
