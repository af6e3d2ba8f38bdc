"""Python view of libflam3gpu's C ABI (include/flam3_gpu.h).

`render(frame, ...)` is flam3_render (flam3.h:623) on the GPU: same frame,
same output layout, same stats.  The other functions expose the kernel-level
entry points used for parity work.  Every call goes through the native
library; if it is not built, `load()` raises -- there is no fallback.
"""
import ctypes as C
import os

import numpy as np

from . import abi

_LIB = None
# FLAM3GPU_LIB selects another build of the library (see flam3_gb300._build --out)
_LIB_PATH = os.environ.get("FLAM3GPU_LIB") or os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                            "libflam3gpu.so")


class Flam3GpuError(RuntimeError):
    pass


class RenderIO(C.Structure):
    _fields_ = [("hist_in", C.POINTER(C.c_double)), ("hist_out", C.POINTER(C.c_double)),
                ("accum_out", C.POINTER(C.c_double)), ("hist_w", C.c_int), ("hist_h", C.c_int),
                ("keep_on_device", C.c_int), ("image_w", C.c_int), ("image_h", C.c_int),
                ("reserved", C.c_int * 3)]


class Options(C.Structure):
    _fields_ = [("iter_mode", C.c_int), ("iter_precision", C.c_int), ("shuffle_every", C.c_int),
                ("threads_per_block", C.c_int), ("blocks", C.c_int), ("chain_samples", C.c_int),
                ("seed_salt", C.c_uint64), ("de_tile", C.c_int), ("de_kernel", C.c_int),
                ("de_stats", C.c_int), ("float_buckets", C.c_int), ("host_plan", C.c_int),
                ("tail_chain_samples", C.c_int), ("tail_wave_pct", C.c_int), ("test_exchange_stall", C.c_int)]


class PngText(C.Structure):
    _fields_ = [("key", C.c_char_p), ("text", C.c_char_p), ("compressed", C.c_int)]


class ImgComments(C.Structure):
    _fields_ = [("genome", C.c_char_p), ("badvals", C.c_char_p), ("numiters", C.c_char_p), ("rtime", C.c_char_p)]


def load():
    """Load libflam3gpu.so (built by flam3_gb300._build / __graft_entry__.build)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(_LIB_PATH):
        raise Flam3GpuError(f"{_LIB_PATH} is not built; run `python -m flam3_gb300._build`")
    lib = C.CDLL(_LIB_PATH)
    F = C.POINTER(abi.flam3_frame)
    G = C.POINTER(abi.flam3_genome)
    S = C.POINTER(abi.stat_struct)
    dp = C.POINTER(C.c_double)
    lib.flam3gpu_render.argtypes = [F, C.c_void_p, C.c_int, C.c_int, C.c_int, S]
    lib.flam3gpu_render_ex.argtypes = [F, C.c_void_p, C.c_int, C.c_int, C.c_int, S, C.POINTER(RenderIO)]
    lib.flam3gpu_render_memory_required.argtypes = [F]
    lib.flam3gpu_render_memory_required.restype = C.c_double
    lib.flam3gpu_calc_nstrips.argtypes = [F, C.c_double]
    lib.flam3gpu_render_strips.argtypes = [F, C.c_void_p, C.c_int, C.c_int, S, C.c_int]
    lib.flam3gpu_last_error.restype = C.c_char_p
    lib.flam3gpu_version.restype = C.c_char_p
    lib.flam3gpu_set_options.argtypes = [C.POINTER(Options)]
    lib.flam3gpu_get_options.argtypes = [C.POINTER(Options)]
    lib.flam3gpu_default_options.argtypes = [C.POINTER(Options)]
    lib.flam3gpu_last_timings.argtypes = [dp]
    lib.flam3gpu_last_de_work.argtypes = [dp]
    lib.flam3gpu_histogram_dims.argtypes = [F, C.c_int] + [C.POINTER(C.c_int)] * 5
    lib.flam3gpu_apply_xform.argtypes = [G, C.c_int, C.c_int, dp, C.POINTER(C.c_uint32), C.c_int, dp,
                                         C.POINTER(C.c_int), C.c_int]
    lib.flam3gpu_accumulate_points.argtypes = [F, C.c_int, dp, C.c_long, dp, C.POINTER(C.c_int),
                                               C.POINTER(C.c_int)]
    lib.flam3gpu_iterate_chains.argtypes = [G, C.c_int, C.c_int, C.c_int, dp, C.c_uint64, dp,
                                            C.POINTER(C.c_long), C.c_int]
    lib.flam3gpu_xform_choice_table.argtypes = [G, C.POINTER(C.c_uint16), C.POINTER(C.c_int)]
    lib.flam3gpu_plan_passes.argtypes = [F, C.c_int, C.c_void_p, C.c_int]
    lp = C.POINTER(C.c_longlong)
    ip = C.POINTER(C.c_int)
    lib.flam3gpu_chunk_plan.argtypes = [lp, C.c_int, C.c_int, C.c_int, C.c_int, ip, ip, lp, lp]
    lib.flam3gpu_choice_breakpoints.argtypes = [dp, dp, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_uint16),
                                                C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.flam3gpu_pass_bytes.restype = C.c_size_t
    lib.flam3gpu_interpolate.argtypes = [G, C.c_int, C.c_double, C.c_double, G]
    lib.flam3gpu_estimate_bounding_box.argtypes = [G, C.c_double, C.c_int, dp, dp, C.POINTER(abi.randctx)]
    lib.flam3gpu_colorhist.argtypes = [G, C.c_int, C.POINTER(abi.randctx), dp]
    lib.flam3gpu_measure_atomic_rate.argtypes = [C.c_longlong, C.c_longlong, dp]
    lib.flam3gpu_dimension.argtypes = [G, C.c_int, C.c_int, C.POINTER(abi.randctx)]
    lib.flam3gpu_dimension.restype = C.c_double
    lib.flam3gpu_lyapunov.argtypes = [G, C.c_int, C.POINTER(abi.randctx)]
    lib.flam3gpu_lyapunov.restype = C.c_double
    lib.flam3gpu_parse_xml2.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.POINTER(C.c_int)]
    lib.flam3gpu_parse_xml2.restype = C.POINTER(abi.flam3_genome)
    lib.flam3gpu_free_genome.argtypes = [G]
    lib.flam3gpu_free_genome.restype = None
    lib.flam3gpu_set_interpolator.argtypes = [C.c_void_p]
    lib.flam3gpu_set_interpolator.restype = None
    ucpp = C.POINTER(C.POINTER(C.c_ubyte))
    lib.flam3gpu_encode_png.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                        C.POINTER(PngText), C.c_int, ucpp, C.POINTER(C.c_size_t)]
    lib.flam3gpu_write_png.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.POINTER(ImgComments), C.c_int]
    lib.flam3gpu_render_png.argtypes = [F, C.c_int, S, C.c_char_p, ucpp, C.POINTER(C.c_size_t)]
    lib.flam3gpu_png_last_ms.argtypes = [dp]
    _LIB = lib
    return lib


def _err(lib, what):
    raise Flam3GpuError(f"{what} failed: {lib.flam3gpu_last_error().decode()}")


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def version():
    return load().flam3gpu_version().decode()


def histogram_dims(frame, field=0):
    lib = load()
    v = [C.c_int() for _ in range(5)]
    if lib.flam3gpu_histogram_dims(C.byref(frame.f), field, *[C.byref(x) for x in v]):
        _err(lib, "histogram_dims")
    w, h, gutter, de_offset, fw = (x.value for x in v)
    return {"w": w, "h": h, "gutter": gutter, "de_offset": de_offset, "filter_width": fw}


def render(frame, field=0, nchan=3, transp=0, out=None, hist_in=None, want_hist=False, want_accum=False):
    """flam3_render on the GPU.  Returns (image, stats[, extras])."""
    lib = load()
    if out is None:
        out = frame.out_buffer(nchan)
    st = abi.stat_struct()
    extras = {}
    if hist_in is None and not want_hist and not want_accum:
        if lib.flam3gpu_render(C.byref(frame.f), out.ctypes.data, field, nchan, transp, C.byref(st)):
            _err(lib, "flam3gpu_render")
        return out, st
    d = histogram_dims(frame, field)
    io = RenderIO()
    if hist_in is not None:
        hist_in = np.ascontiguousarray(hist_in, dtype=np.float64)
        if hist_in.size != d["w"] * d["h"] * 5:
            raise ValueError("hist_in has the wrong size")
        io.hist_in = _dptr(hist_in)
    if want_hist:
        extras["hist"] = np.zeros((d["h"], d["w"], 5))
        io.hist_out = _dptr(extras["hist"])
    if want_accum:
        extras["accum"] = np.zeros((d["h"], d["w"], 4))
        io.accum_out = _dptr(extras["accum"])
    if lib.flam3gpu_render_ex(C.byref(frame.f), out.ctypes.data, field, nchan, transp, C.byref(st), C.byref(io)):
        _err(lib, "flam3gpu_render_ex")
    return out, st, extras


def memory_required(frame):
    return load().flam3gpu_render_memory_required(C.byref(frame.f))


def calc_nstrips(frame, budget_bytes=0.0):
    """calc_nstrips of flam3-render against device memory (or budget_bytes)."""
    lib = load()
    n = lib.flam3gpu_calc_nstrips(C.byref(frame.f), float(budget_bytes))
    if n < 0:
        _err(lib, "flam3gpu_calc_nstrips")
    return n


def render_strips(frame, nstrips, nchan=3, transp=0, out=None):
    """flam3-render's strip loop on the GPU: (image, stats)."""
    lib = load()
    if out is None:
        out = frame.out_buffer(nchan)
    st = abi.stat_struct()
    if lib.flam3gpu_render_strips(C.byref(frame.f), out.ctypes.data, nchan, transp, C.byref(st), nstrips):
        _err(lib, "flam3gpu_render_strips")
    return out, st


def last_timings():
    """Measurements of the last render on this thread: kernel times (ms,
    CUDA events), wall time, kernel launches, host<->device bytes, samples
    plotted."""
    t = (C.c_double * 8)()
    load().flam3gpu_last_timings(t)
    return {"iterate_ms": t[0], "de_ms": t[1], "tail_ms": t[2], "wall_ms": t[3], "launches": int(t[4]),
            "h2d_bytes": int(t[5]), "d2h_bytes": int(t[6]), "plotted": int(t[7])}


def last_de_work():
    """Band density estimation work of the last render (set_options(de_stats=1)
    first): sources, source-band pairs, taps."""
    w = (C.c_double * 3)()
    load().flam3gpu_last_de_work(w)
    return {"sources": int(w[0]), "pairs": int(w[1]), "taps": int(w[2])}


def get_options():
    o = Options()
    load().flam3gpu_get_options(C.byref(o))
    return o


def set_options(**kw):
    lib = load()
    o = get_options()
    for k, v in kw.items():
        setattr(o, k, v)
    if lib.flam3gpu_set_options(C.byref(o)):
        _err(lib, "set_options")


def reset_options():
    lib = load()
    o = Options()
    lib.flam3gpu_default_options(C.byref(o))
    lib.flam3gpu_set_options(C.byref(o))


def apply_xform(genome, fn, points, words, precision=64):
    lib = load()
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 4)
    n = pts.shape[0]
    w = np.ascontiguousarray(words, dtype=np.uint32).reshape(n, -1)
    q = np.zeros((n, 4))
    bad = np.zeros(n, dtype=np.int32)
    if lib.flam3gpu_apply_xform(C.byref(genome.g), fn, n, _dptr(pts), w.ctypes.data_as(C.POINTER(C.c_uint32)),
                                w.shape[1], _dptr(q), bad.ctypes.data_as(C.POINTER(C.c_int)), precision):
        _err(lib, "apply_xform")
    return q, bad


def iterate_chains(genome, starts, n, fuse, seed, precision=64):
    lib = load()
    st = np.ascontiguousarray(starts, dtype=np.float64).reshape(-1, 4)
    out = np.zeros((st.shape[0], n, 4))
    bad = C.c_long()
    if lib.flam3gpu_iterate_chains(C.byref(genome.g), st.shape[0], n, fuse, _dptr(st), seed, _dptr(out),
                                   C.byref(bad), precision):
        _err(lib, "iterate_chains")
    return out, bad.value


def chunk_plan(samples, threads=256, blocks=608, sub_batch_size=10000):
    """The iterate launch's chunking on the host: (S, S_tail, chunk_tail,
    nchunks) for passes of the given sample counts."""
    lib = load()
    n = len(samples)
    smp = (C.c_longlong * n)(*[int(x) for x in samples])
    S, St = C.c_int(0), C.c_int(0)
    ct, nc = (C.c_longlong * n)(), (C.c_longlong * n)()
    if lib.flam3gpu_chunk_plan(smp, n, threads, blocks, sub_batch_size, C.byref(S), C.byref(St), ct, nc):
        _err(lib, "chunk_plan")
    return S.value, St.value, list(ct), list(nc)


def choice_breakpoints(weights, chaos=None, nstd=None, walk=False, moves=False):
    """Breakpoints of one choice row on the host: weights of every xform
    (the final one last), the row's chaos entries or None, built by the
    reference's loop or (walk=True) the device planner's binade walk.
    Returns the breakpoint list (and, with moves=True, the sequential steps
    taken); raises Flam3GpuError on the reference's errors."""
    lib = load()
    d = np.ascontiguousarray(weights, dtype=np.float64)
    nx = d.shape[0]
    nstd = nx if nstd is None else nstd
    c = None if chaos is None else np.ascontiguousarray(chaos, dtype=np.float64)
    brk = (C.c_uint16 * 32)()
    n, mv = C.c_int(0), C.c_int(0)
    if lib.flam3gpu_choice_breakpoints(_dptr(d), None if c is None else _dptr(c), nstd, nx, 1 if walk else 0, brk,
                                       C.byref(n), C.byref(mv)):
        _err(lib, "choice_breakpoints")
    return (list(brk)[:n.value], mv.value) if moves else list(brk)[:n.value]


def xform_choice_table(genome):
    """The GPU's xform choice for each 14-bit value of each choice row:
    an (rows, 16384) uint16 array, as flam3_create_xform_distrib's table."""
    lib = load()
    g = genome.g
    ns = g.num_xforms - (1 if g.final_xform_index >= 0 else 0)
    out = np.zeros((ns + 1) * 16384, np.uint16)
    rows = C.c_int(0)
    if lib.flam3gpu_xform_choice_table(C.byref(g), out.ctypes.data_as(C.POINTER(C.c_uint16)), C.byref(rows)):
        _err(lib, "flam3gpu_xform_choice_table")
    return out[:rows.value * 16384].reshape(rows.value, 16384)


def plan_passes(frame, on_device, max_passes=1024):
    """The first batch's passes of `frame` as flam3gpu_render plans them, on
    the device or on host threads: raw records of flam3gpu_pass_bytes() each
    (a uint8 array of shape (n, bytes))."""
    lib = load()
    size = lib.flam3gpu_pass_bytes()
    buf = np.zeros(max_passes * size, np.uint8)
    n = lib.flam3gpu_plan_passes(C.byref(frame.f), 1 if on_device else 0, buf.ctypes.data, max_passes)
    if n < 0:
        _err(lib, "flam3gpu_plan_passes")
    return buf[:n * size].reshape(n, size)


def accumulate_points(frame, points, field=0):
    lib = load()
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 4)
    w, h = C.c_int(), C.c_int()
    lib.flam3gpu_accumulate_points(C.byref(frame.f), field, _dptr(pts), 0, None, C.byref(w), C.byref(h))
    hist = np.zeros((h.value, w.value, 5))
    if lib.flam3gpu_accumulate_points(C.byref(frame.f), field, _dptr(pts), pts.shape[0], _dptr(hist), C.byref(w),
                                      C.byref(h)):
        _err(lib, "accumulate_points")
    return hist


class InterpolatedGenome:
    """A flam3_genome produced by flam3gpu_interpolate; owns its xform and
    chaos storage (released with flam3gpu_free_genome)."""

    def __init__(self, g):
        self.g = g

    def __del__(self):
        if _LIB is not None and self.g.xform:
            _LIB.flam3gpu_free_genome(C.byref(self.g))


def interpolate(genomes, time, stagger=0.0):
    """flam3_interpolate (flam3.c:717-802): the genome at `time` between the
    control points `genomes` (Genome objects or flam3_genome structs, sorted
    by time)."""
    lib = load()
    structs = [getattr(G, "g", G) for G in genomes]
    arr = (abi.flam3_genome * len(structs))(*structs)
    out = abi.flam3_genome()
    out.final_xform_index = -1
    if lib.flam3gpu_interpolate(arr, len(structs), float(time), float(stagger), C.byref(out)):
        _err(lib, "flam3gpu_interpolate")
    return InterpolatedGenome(out)


def estimate_bounding_box(genome, eps=0.01, nsamples=10000, rc=None):
    """flam3_estimate_bounding_box on the GPU: (bmin, bmax, bad values)."""
    lib = load()
    from .isaac import init_rc
    if rc is None:
        rc = abi.randctx()
        init_rc(rc, b"bbox")
    bmin = np.zeros(2)
    bmax = np.zeros(2)
    g = getattr(genome, "g", genome)
    bv = lib.flam3gpu_estimate_bounding_box(C.byref(g), eps, nsamples, _dptr(bmin), _dptr(bmax), C.byref(rc))
    if bv < 0:
        _err(lib, "flam3gpu_estimate_bounding_box")
    return bmin, bmax, bv


def dimension(genome, ntries=3000 * 1000, clip_to_camera=False, rc=None):
    """flam3_dimension on the GPU: the correlation dimension estimate."""
    lib = load()
    from .isaac import init_rc
    if rc is None:
        rc = abi.randctx()
        init_rc(rc, b"dimension")
    g = getattr(genome, "g", genome)
    d = lib.flam3gpu_dimension(C.byref(g), ntries, 1 if clip_to_camera else 0, C.byref(rc))
    if d == -1.0:
        _err(lib, "flam3gpu_dimension")
    return d


def lyapunov(genome, ntries=10000, rc=None):
    """flam3_lyapunov on the GPU."""
    lib = load()
    from .isaac import init_rc
    if rc is None:
        rc = abi.randctx()
        init_rc(rc, b"lyapunov")
    g = getattr(genome, "g", genome)
    v = lib.flam3gpu_lyapunov(C.byref(g), ntries, C.byref(rc))
    if v == -1.0 and load().flam3gpu_last_error():
        _err(lib, "flam3gpu_lyapunov")
    return v


def measure_atomic_rate(nbuckets, natomics=1 << 31):
    """float4 atomic adds per second at random buckets (roofline ceiling)."""
    lib = load()
    r = C.c_double()
    if lib.flam3gpu_measure_atomic_rate(int(nbuckets), int(natomics), C.byref(r)):
        _err(lib, "flam3gpu_measure_atomic_rate")
    return r.value


def colorhist(genome, num_batches=10, rc=None):
    """flam3_colorhist on the GPU: 256 normalised bins."""
    lib = load()
    from .isaac import init_rc
    if rc is None:
        rc = abi.randctx()
        init_rc(rc, b"colorhist")
    hist = np.zeros(256)
    g = getattr(genome, "g", genome)
    if lib.flam3gpu_colorhist(C.byref(g), num_batches, C.byref(rc), _dptr(hist)):
        _err(lib, "flam3gpu_colorhist")
    return hist



_libc = None


def _take_buffer(ptr, n):
    """Copies a malloc'd buffer of the library into bytes and frees it."""
    global _libc
    if _libc is None:
        _libc = C.CDLL(None)
        _libc.free.argtypes = [C.c_void_p]
    data = C.string_at(ptr, n)
    _libc.free(C.cast(ptr, C.c_void_p))
    return data


def encode_png(image, texts=(), on_device_ptr=None):
    """PNG bytes of an (h, w, 3|4) uint8 or uint16 image, encoded on the GPU
    (flam3gpu_encode_png).  texts: (key, text, compressed) tuples.  With
    on_device_ptr the pixels are read from that device address instead (the
    array then only gives shape and dtype)."""
    lib = load()
    img = np.ascontiguousarray(image)
    if img.ndim != 3 or img.shape[2] not in (3, 4) or img.dtype not in (np.uint8, np.uint16):
        raise ValueError("image must be (h, w, 3|4) uint8 or uint16")
    h, w, nchan = img.shape
    bpc = img.dtype.itemsize
    tt = (PngText * max(1, len(texts)))()
    keep = []
    for i, (k, t, z) in enumerate(texts):
        kb = k.encode("latin-1")
        tb = None if t is None else t.encode("latin-1")
        keep += [kb, tb]
        tt[i] = PngText(kb, tb, int(z))
    out = C.POINTER(C.c_ubyte)()
    n = C.c_size_t()
    src = on_device_ptr if on_device_ptr is not None else img.ctypes.data
    if lib.flam3gpu_encode_png(C.c_void_p(src), int(on_device_ptr is not None), w, h, nchan, bpc, tt, len(texts),
                               C.byref(out), C.byref(n)):
        _err(lib, "flam3gpu_encode_png")
    return _take_buffer(out, n.value)


def write_png(path, image, genome=None, badvals=None, numiters=None, rtime=None):
    """write_png (png.c:36) on the GPU: an (h, w, 4) uint8/uint16 image to `path`."""
    lib = load()
    img = np.ascontiguousarray(image)
    if img.ndim != 3 or img.shape[2] != 4 or img.dtype not in (np.uint8, np.uint16):
        raise ValueError("image must be (h, w, 4) uint8 or uint16")
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    libc.fclose.argtypes = [C.c_void_p]
    enc = (lambda v: None if v is None else v.encode("latin-1"))
    fpc = ImgComments(enc(genome), enc(badvals), enc(numiters), enc(rtime))
    fp = libc.fopen(path.encode(), b"wb")
    if not fp:
        raise OSError(f"cannot open {path}")
    try:
        rv = lib.flam3gpu_write_png(fp, img.ctypes.data, img.shape[1], img.shape[0], C.byref(fpc), img.dtype.itemsize)
    finally:
        libc.fclose(fp)
    if rv:
        _err(lib, "flam3gpu_write_png")


def render_png(frame, transp=0, genome_xml=None):
    """flam3gpu_render_png: (png bytes, stats) of an RGBA render that never
    leaves the device as raw pixels."""
    lib = load()
    st = abi.stat_struct()
    out = C.POINTER(C.c_ubyte)()
    n = C.c_size_t()
    if lib.flam3gpu_render_png(C.byref(frame.f), transp, C.byref(st),
                               None if genome_xml is None else genome_xml.encode("latin-1"), C.byref(out), C.byref(n)):
        _err(lib, "flam3gpu_render_png")
    return _take_buffer(out, n.value), st


def png_last_ms():
    """Kernel time (ms) of this thread's last PNG encode."""
    v = C.c_double()
    load().flam3gpu_png_last_ms(C.byref(v))
    return v.value
