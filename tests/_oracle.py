"""ctypes bindings of the test oracle (oracle/liboracle.so, the plain-C
restatement of the reference render path) and, where it was built, of the
reference itself (oracle/_ref).  Test infrastructure only."""
import ctypes as C
import os
import subprocess

import numpy as np

from flam3_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
REF_DIR = os.path.join(ORACLE_DIR, "_ref")
GOLDEN = os.path.join(ROOT, "tests", "golden")

_cache = {}


def _build_port():
    subprocess.run(["make", "-C", ORACLE_DIR, "port", "liboracle_fast.so"], check=True, capture_output=True)


def _bind(lib, prefix):
    F = C.POINTER(abi.flam3_frame)
    G = C.POINTER(abi.flam3_genome)
    S = C.POINTER(abi.stat_struct)
    dp = C.POINTER(C.c_double)
    getattr(lib, prefix + "render").argtypes = [F, C.c_void_p, C.c_int, C.c_int, C.c_int, S]
    return lib


class RenderIO(C.Structure):
    _fields_ = [("hist_in", C.POINTER(C.c_double)), ("hist_out", C.POINTER(C.c_double)),
                ("accum_out", C.POINTER(C.c_double)), ("hist_w", C.c_int), ("hist_h", C.c_int),
                ("nthreads_used", C.c_int)]


def oracle(fast=False):
    key = "fast" if fast else "port"
    if key in _cache:
        return _cache[key]
    path = os.path.join(ORACLE_DIR, "liboracle_fast.so" if fast else "liboracle.so")
    if not os.path.exists(path):
        _build_port()
    lib = C.CDLL(path)
    F = C.POINTER(abi.flam3_frame)
    G = C.POINTER(abi.flam3_genome)
    S = C.POINTER(abi.stat_struct)
    dp = C.POINTER(C.c_double)
    lib.f3o_render.argtypes = [F, C.c_void_p, C.c_int, C.c_int, C.c_int, S]
    lib.f3o_render_ex.argtypes = [F, C.c_void_p, C.c_int, C.c_int, C.c_int, S, C.POINTER(RenderIO)]
    lib.f3o_apply_xform.argtypes = [G, C.c_int, C.c_int, dp, C.POINTER(C.c_uint32), C.c_int, dp, C.POINTER(C.c_int)]
    lib.f3o_accumulate_points.argtypes = [F, C.c_int, dp, C.c_long, dp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.f3o_iterate_chains.argtypes = [G, C.c_int, C.c_int, C.c_int, dp, C.c_uint64, dp, C.POINTER(C.c_long)]
    lib.f3o_irand.argtypes = [C.POINTER(abi.randctx)]
    lib.f3o_irand.restype = C.c_ulong
    lib.f3o_init_rc.argtypes = [C.POINTER(abi.randctx), C.c_char_p]
    lib.f3o_create_de_filters.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int, C.POINTER(C.c_int),
                                          C.POINTER(C.c_int), C.POINTER(dp), C.POINTER(dp)]
    lib.f3o_create_spatial_filter.argtypes = [F, C.c_int, C.POINTER(dp)]
    lib.f3o_create_temporal_filter.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.POINTER(dp),
                                               C.POINTER(dp)]
    lib.f3o_create_temporal_filter.restype = C.c_double
    lib.f3o_create_xform_distrib.argtypes = [G]
    lib.f3o_create_xform_distrib.restype = C.POINTER(C.c_ushort)
    lib.f3o_prepare_precalc_flags.argtypes = [G]
    lib.f3o_philox4x32.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
    lib.f3o_set_interpolator.argtypes = [C.c_void_p]
    lib.f3o_set_interpolator.restype = None
    lib.oracle_png_filter.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
    lib.oracle_png_filter.restype = C.c_longlong
    lib.oracle_png_unfilter.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
    _cache[key] = lib
    return lib


_INTERP = C.CFUNCTYPE(C.c_int, C.POINTER(abi.flam3_genome), C.c_int, C.c_double, C.c_double,
                      C.POINTER(abi.flam3_genome))


def set_interpolator(which="product", fast=False):
    """Installs the oracle's multi-genome interpolator: libflam3gpu's
    flam3gpu_interpolate ("product", pinned against the reference by
    tests/test_interp_pin.py) or the reference's own flam3_interpolate
    ("reference", only where oracle/_ref was built)."""
    lib = oracle(fast)
    if which == "product":
        from flam3_gb300 import render
        gpu = render.load()
        lib.f3o_set_interpolator(C.cast(gpu.flam3gpu_interpolate, C.c_void_p))
    else:
        ref = reference(True)
        ref.flam3_interpolate.argtypes = [C.POINTER(abi.flam3_genome), C.c_int, C.c_double, C.c_double,
                                          C.POINTER(abi.flam3_genome)]
        ref.flam3_interpolate.restype = None

        def call(cps, n, t, stagger, out):
            ref.flam3_interpolate(cps, n, t, stagger, out)
            return 0

        cb = _INTERP(call)
        _cache["ref_interp_cb"] = cb  # keep the thunk alive
        lib.f3o_set_interpolator(C.cast(cb, C.c_void_p))
    _cache[("interp", fast)] = which


def reference(strict=True):
    """The reference library built from its sources (only where the reference
    tree was available at build time); None otherwise."""
    key = "ref_strict" if strict else "ref_fast"
    if key in _cache:
        return _cache[key]
    path = os.path.join(REF_DIR, "libflam3ref_strict.so" if strict else "libflam3ref.so")
    if not os.path.exists(path):
        _cache[key] = None
        return None
    lib = C.CDLL(path)
    F = C.POINTER(abi.flam3_frame)
    G = C.POINTER(abi.flam3_genome)
    S = C.POINTER(abi.stat_struct)
    dp = C.POINTER(C.c_double)
    lib.flam3_render.argtypes = [F, C.c_void_p, C.c_int, C.c_int, C.c_int, S]
    lib.prepare_precalc_flags.argtypes = [G]
    lib.xform_precalc.argtypes = [G, C.c_int]
    lib.apply_xform.argtypes = [G, C.c_int, dp, dp, C.POINTER(abi.randctx)]
    lib.flam3_create_xform_distrib.argtypes = [G]
    lib.flam3_create_xform_distrib.restype = C.POINTER(C.c_ushort)
    _cache[key] = lib
    return lib


def oracle_render(frame, field=0, nchan=3, transp=0, hist_in=None, want_hist=False, want_accum=False, fast=False):
    lib = oracle(fast)
    if frame.f.ngenomes > 1 and ("interp", fast) not in _cache:
        set_interpolator("product", fast)
    out = frame.out_buffer(nchan)
    st = abi.stat_struct()
    io = RenderIO()
    extras = {}
    keep = []
    if hist_in is not None:
        hi = np.ascontiguousarray(hist_in, dtype=np.float64)
        keep.append(hi)
        io.hist_in = hi.ctypes.data_as(C.POINTER(C.c_double))
    # geometry first (hist_out needs the size): a dry run is not available, so
    # size buffers from a render with outputs requested only when asked
    if want_hist or want_accum:
        probe = RenderIO()
        w, h = C.c_int(), C.c_int()
        lib.f3o_accumulate_points(C.byref(frame.f), field, None, 0, None, C.byref(w), C.byref(h))
        if want_hist:
            extras["hist"] = np.zeros((h.value, w.value, 5))
            io.hist_out = extras["hist"].ctypes.data_as(C.POINTER(C.c_double))
        if want_accum:
            extras["accum"] = np.zeros((h.value, w.value, 4))
            io.accum_out = extras["accum"].ctypes.data_as(C.POINTER(C.c_double))
        del probe
    r = lib.f3o_render_ex(C.byref(frame.f), out.ctypes.data, field, nchan, transp, C.byref(st), C.byref(io))
    if r:
        raise RuntimeError("oracle render failed")
    return out, st, extras


def oracle_apply_xform(genome, fn, points, words):
    lib = oracle()
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 4)
    n = pts.shape[0]
    w = np.ascontiguousarray(words, dtype=np.uint32).reshape(n, -1)
    q = np.zeros((n, 4))
    bad = np.zeros(n, dtype=np.int32)
    lib.f3o_apply_xform(C.byref(genome.g), fn, n, pts.ctypes.data_as(C.POINTER(C.c_double)),
                        w.ctypes.data_as(C.POINTER(C.c_uint32)), w.shape[1],
                        q.ctypes.data_as(C.POINTER(C.c_double)), bad.ctypes.data_as(C.POINTER(C.c_int)))
    return q, bad


def oracle_iterate_chains(genome, starts, n, fuse, seed):
    lib = oracle()
    st = np.ascontiguousarray(starts, dtype=np.float64).reshape(-1, 4)
    out = np.zeros((st.shape[0], n, 4))
    bad = C.c_long()
    lib.f3o_iterate_chains(C.byref(genome.g), st.shape[0], n, fuse, st.ctypes.data_as(C.POINTER(C.c_double)),
                           seed, out.ctypes.data_as(C.POINTER(C.c_double)), C.byref(bad))
    return out, bad.value


def oracle_accumulate(frame, points, field=0):
    lib = oracle()
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 4)
    w, h = C.c_int(), C.c_int()
    lib.f3o_accumulate_points(C.byref(frame.f), field, None, 0, None, C.byref(w), C.byref(h))
    hist = np.zeros((h.value, w.value, 5))
    lib.f3o_accumulate_points(C.byref(frame.f), field, pts.ctypes.data_as(C.POINTER(C.c_double)), pts.shape[0],
                              hist.ctypes.data_as(C.POINTER(C.c_double)), C.byref(w), C.byref(h))
    return hist


def ref_apply_xform(genome, fn, points, words):
    """The reference's apply_xform (variations.c:2129) with the random words
    fed through its ISAAC context (irand hands out randrsl from the top)."""
    lib = reference(True)
    g = genome.g
    lib.prepare_precalc_flags(C.byref(g))
    for i in range(g.num_xforms):
        lib.xform_precalc(C.byref(g), i)
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 4)
    n = pts.shape[0]
    w = np.ascontiguousarray(words, dtype=np.uint32).reshape(n, -1)
    if w.shape[1] > 16:
        raise ValueError("at most 16 words per call can be replayed")
    q = np.zeros((n, 4))
    bad = np.zeros(n, dtype=np.int32)
    for k in range(n):
        rc = abi.randctx()
        rc.randcnt = 16
        for j in range(w.shape[1]):
            rc.randrsl[15 - j] = int(w[k, j])
        p = (C.c_double * 4)(*pts[k])
        qq = (C.c_double * 4)()
        bad[k] = lib.apply_xform(C.byref(g), fn, p, qq, C.byref(rc))
        q[k] = list(qq)
    return q, bad


def png_filter(img, fast=False):
    """The filtered stream write_png's libpng call deflates (oracle restatement)."""
    img = np.ascontiguousarray(img)
    h, w, nchan = img.shape
    bpc = img.dtype.itemsize
    F = np.zeros(h * (1 + w * nchan * bpc), np.uint8)
    oracle(fast).oracle_png_filter(img.ctypes.data, w, h, nchan, bpc, F.ctypes.data)
    return F


def png_unfilter(F, shape, dtype):
    h, w, nchan = shape
    out = np.zeros(shape, dtype)
    F = np.ascontiguousarray(F, dtype=np.uint8)
    if oracle().oracle_png_unfilter(F.ctypes.data, w, h, nchan, np.dtype(dtype).itemsize, out.ctypes.data):
        raise ValueError("bad PNG filter type")
    return out
