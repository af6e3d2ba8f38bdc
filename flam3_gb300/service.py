"""Python view of the batched / served rendering API (include/flam3_gpu_service.h).

`Service` queues flam3_render requests (Frame objects) on a service thread
that packs every admitted job's temporal samples into shared persistent
iterate launches, runs per-round tails in CUDA graphs, and hands results
back per ticket.  `render_batch` renders a list of frames through a
temporary service in one go.  Everything goes through libflam3gpu; there is
no Python fallback.
"""
import ctypes as C

import numpy as np

from . import abi, render


class ServiceConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_double), ("round_samples", C.c_longlong), ("max_active", C.c_int),
                ("tail_graphs", C.c_int), ("streams", C.c_int), ("use_tuning", C.c_int),
                ("max_inflight", C.c_int), ("tail_branches", C.c_int), ("order", C.c_int),
                ("reserved", C.c_int * 5)]


_BOUND = False


def _lib():
    global _BOUND
    lib = render.load()
    if not _BOUND:
        F = C.POINTER(abi.flam3_frame)
        S = C.POINTER(abi.stat_struct)
        P = C.c_void_p
        lib.flam3gpu_service_default_config.argtypes = [C.POINTER(ServiceConfig)]
        lib.flam3gpu_service_default_config.restype = None
        lib.flam3gpu_service_create.argtypes = [C.POINTER(ServiceConfig)]
        lib.flam3gpu_service_create.restype = P
        lib.flam3gpu_service_submit.argtypes = [P, F, C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_uint64)]
        lib.flam3gpu_service_submit_many.argtypes = [P, F, C.c_int, C.POINTER(C.c_void_p), C.c_int, C.c_int,
                                                     C.c_int, C.POINTER(C.c_uint64)]
        lib.flam3gpu_service_wait.argtypes = [P, C.c_uint64, C.c_double, S, C.POINTER(C.c_double)]
        lib.flam3gpu_service_drain.argtypes = [P]
        lib.flam3gpu_service_counters.argtypes = [P, C.POINTER(C.c_double)]
        lib.flam3gpu_service_counters.restype = None
        lib.flam3gpu_service_destroy.argtypes = [P]
        lib.flam3gpu_service_destroy.restype = None
        lib.flam3gpu_render_batch.argtypes = [F, C.c_int, C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int, S,
                                              C.POINTER(ServiceConfig)]
        lib.flam3gpu_autotune.argtypes = [F, C.c_int, C.c_double]
        lib.flam3gpu_autotune_save.argtypes = [C.c_char_p]
        lib.flam3gpu_autotune_load.argtypes = [C.c_char_p]
        lib.flam3gpu_autotune_clear.argtypes = []
        lib.flam3gpu_autotune_clear.restype = None
        _BOUND = True
    return lib


def config(**kw):
    lib = _lib()
    c = ServiceConfig()
    lib.flam3gpu_service_default_config(C.byref(c))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


COUNTER_NAMES = ("jobs_done", "jobs_failed", "rounds", "launches", "tail_graphs", "graphs_instantiated",
                 "samples_plotted", "device_bytes", "peak_device_bytes", "busy_s", "h2d_bytes", "d2h_bytes",
                 "host_admit_s", "host_round_s", "host_tail_s", "host_complete_s", "host_wait_s",
                 "gpu_iterate_s", "gpu_tail_s")


class Service:
    """A render service on the current GPU."""

    def __init__(self, **cfg):
        self.lib = _lib()
        self.cfg = config(**cfg)
        self.h = self.lib.flam3gpu_service_create(C.byref(self.cfg))
        if not self.h:
            raise render.Flam3GpuError("service create failed: " + self.lib.flam3gpu_last_error().decode())
        self._keep = {}

    def submit(self, frame, field=0, nchan=3, transp=0, out=None):
        """Queues frame (a genome.Frame); returns a ticket.  The frame's ISAAC
        context advances as flam3_render would advance it."""
        if out is None:
            out = frame.out_buffer(nchan)
        t = C.c_uint64()
        if self.lib.flam3gpu_service_submit(self.h, C.byref(frame.f), out.ctypes.data, field, nchan, transp,
                                            C.byref(t)):
            raise render.Flam3GpuError("submit failed: " + self.lib.flam3gpu_last_error().decode())
        self._keep[t.value] = out
        return t.value

    def submit_many(self, frames, field=0, nchan=3, transp=0):
        """Queues a list of frames planned in parallel and admitted together;
        returns their tickets."""
        n = len(frames)
        arr = (abi.flam3_frame * n)(*[F.f for F in frames])
        outs = [F.out_buffer(nchan) for F in frames]
        ptrs = (C.c_void_p * n)(*[o.ctypes.data for o in outs])
        tk = (C.c_uint64 * n)()
        r = self.lib.flam3gpu_service_submit_many(self.h, arr, n, ptrs, field, nchan, transp, tk)
        for i, F in enumerate(frames):
            F.f.rc = arr[i].rc
            if tk[i]:
                self._keep[tk[i]] = outs[i]
        if r:
            raise render.Flam3GpuError("submit_many failed: " + self.lib.flam3gpu_last_error().decode())
        return list(tk)

    def wait(self, ticket, timeout_ms=-1.0):
        """(image, stats, times_ms) of a finished job; times_ms = [submit->admit,
        admit->first round, latency, rounds]."""
        st = abi.stat_struct()
        tm = (C.c_double * 4)()
        r = self.lib.flam3gpu_service_wait(self.h, ticket, float(timeout_ms), C.byref(st), tm)
        if r == 2:
            raise TimeoutError("job %d not done" % ticket)
        out = self._keep.pop(ticket)
        if r:
            raise render.Flam3GpuError("job failed: " + self.lib.flam3gpu_last_error().decode())
        return out, st, list(tm)

    def drain(self):
        self.lib.flam3gpu_service_drain(self.h)

    def counters(self):
        a = (C.c_double * 19)()
        self.lib.flam3gpu_service_counters(self.h, a)
        return dict(zip(COUNTER_NAMES, list(a)))

    def close(self):
        if self.h:
            self.lib.flam3gpu_service_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def render_batch(frames, field=0, nchan=3, transp=0, **cfg):
    """Renders a list of genome.Frame through one temporary service; returns
    a list of (image, stats)."""
    lib = _lib()
    n = len(frames)
    arr = (abi.flam3_frame * n)(*[F.f for F in frames])
    outs = [F.out_buffer(nchan) for F in frames]
    ptrs = (C.c_void_p * n)(*[o.ctypes.data for o in outs])
    stats = (abi.stat_struct * n)()
    c = config(**cfg) if cfg else None
    r = lib.flam3gpu_render_batch(arr, n, ptrs, field, nchan, transp, stats, C.byref(c) if c is not None else None)
    # the frames' ISAAC contexts advanced inside the array copy
    for i, F in enumerate(frames):
        F.f.rc = arr[i].rc
    if r:
        raise render.Flam3GpuError("render_batch failed: " + lib.flam3gpu_last_error().decode())
    return [(outs[i], stats[i]) for i in range(n)]


def render_batch_png(frames, transp=0):
    """flam3gpu_render_batch_png: the frames rendered as RGBA through one
    temporary service, each encoded as PNG on the device as it completes;
    returns a list of (png bytes, stats)."""
    lib = _lib()
    n = len(frames)
    arr = (abi.flam3_frame * n)(*[F.f for F in frames])
    stats = (abi.stat_struct * n)()
    pngs = (C.POINTER(C.c_ubyte) * n)()
    lens = (C.c_size_t * n)()
    lib.flam3gpu_render_batch_png.argtypes = [C.POINTER(abi.flam3_frame), C.c_int, C.c_int,
                                              C.POINTER(abi.stat_struct), C.POINTER(C.POINTER(C.c_ubyte)),
                                              C.POINTER(C.c_size_t)]
    r = lib.flam3gpu_render_batch_png(arr, n, transp, stats, pngs, lens)
    for i, F in enumerate(frames):
        F.f.rc = arr[i].rc
    out = [(render._take_buffer(pngs[i], lens[i]) if pngs[i] else None, stats[i]) for i in range(n)]
    if r:
        raise render.Flam3GpuError("render_batch_png failed: " + lib.flam3gpu_last_error().decode())
    return out


def autotune(frames, quality_scale=0.25):
    lib = _lib()
    n = len(frames)
    arr = (abi.flam3_frame * n)(*[F.f for F in frames])
    r = lib.flam3gpu_autotune(arr, n, quality_scale)
    if r < 0:
        raise render.Flam3GpuError("autotune failed: " + lib.flam3gpu_last_error().decode())
    return r


def autotune_save(path):
    return _lib().flam3gpu_autotune_save(path.encode())


def autotune_load(path):
    return _lib().flam3gpu_autotune_load(path.encode())


def autotune_clear():
    _lib().flam3gpu_autotune_clear()

