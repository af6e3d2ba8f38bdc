"""Temporal samples planned on the device (f3g_plan.cu) against the host
planner (host/interp.c + host/prep.c, itself pinned to the reference's
flam3_interpolate): the same passes for every frame of the interpolation
cases -- padding rules, palette modes, matrix modes, chaos, final xforms,
four-key Catmull-Rom -- and the same images for an animation frame.

Bars: integer fields, choice rows, variation lists and the colour map
(no libm in their arithmetic) exactly equal; coefficients, parameters and
precalc values within 1e-12 relative (CUDA's and glibc's atan2, exp, log,
sin, cos and pow may differ in the last bit); the camera is planned by the
host in both paths and equal exactly."""
import ctypes as C

import numpy as np
import pytest

from flam3_gb300 import genome as gm, render
import interp_cases

pytestmark = pytest.mark.gpu

NV, NX, NVAR, PRM = 99, 32, 384, 128


class F3GXform(C.Structure):
    _fields_ = [("c", C.c_double * 6), ("post", C.c_double * 6), ("color", C.c_double), ("color_speed", C.c_double),
                ("vis_adjusted", C.c_double), ("opacity", C.c_double), ("preblur", C.c_double), ("flags", C.c_int),
                ("var_off", C.c_int), ("nvars", C.c_int), ("pad", C.c_int), ("prm", C.c_double * PRM)]


class F3GPass(C.Structure):
    """Mirror of F3GPass (flam3_gb300/csrc/f3g_common.h), checked by size."""
    _fields_ = [("samples", C.c_int64), ("chunk_begin", C.c_int64), ("nchunks", C.c_int64), ("key", C.c_uint32 * 2),
                ("fuse", C.c_int), ("iter_mode", C.c_int), ("num_xforms", C.c_int), ("num_std", C.c_int),
                ("final_index", C.c_int), ("final_enable", C.c_int), ("chaos_enable", C.c_int),
                ("full_variations", C.c_int), ("nbrk", C.c_uint16 * (NX + 1)), ("brk", (C.c_uint16 * NX) * (NX + 1)),
                ("var_id", C.c_uint8 * NVAR), ("var_w", C.c_double * NVAR), ("dmap", (C.c_float * 4) * 256),
                ("cmap_size", C.c_int), ("palette_mode", C.c_int), ("trunc_hits", C.c_int),
                ("bounds", C.c_double * 4), ("rot", (C.c_double * 2) * 2), ("rot_center", C.c_double * 2),
                ("rotate", C.c_int), ("width", C.c_int), ("height", C.c_int), ("ws0", C.c_double),
                ("wb0s0", C.c_double), ("hs1", C.c_double), ("hb1s1", C.c_double), ("buckets", C.c_void_p),
                ("count", C.c_void_p), ("bucket_kind", C.c_int), ("S", C.c_int), ("S_tail", C.c_int),
                ("chunk_tail", C.c_int64), ("counters", C.c_void_p),
                ("xf", F3GXform * NX)]


def passes(frame, on_device):
    raw = render.plan_passes(frame, on_device, max_passes=64)
    return [F3GPass.from_buffer_copy(raw[i].tobytes()) for i in range(raw.shape[0])]


def close(a, b, rtol=1e-12, atol=1e-14):
    a, b = np.asarray(a, float), np.asarray(b, float)
    ok = np.abs(a - b) <= atol + rtol * np.maximum(np.abs(a), np.abs(b))
    return np.all(ok | (np.isnan(a) & np.isnan(b)))


def compare(h, d, what):
    for f in ("samples", "fuse", "iter_mode", "num_xforms", "num_std", "final_index", "final_enable", "chaos_enable",
              "full_variations", "cmap_size", "palette_mode", "rotate", "width", "height"):
        assert getattr(h, f) == getattr(d, f), (what, f, getattr(h, f), getattr(d, f))
    assert list(h.key) == list(d.key), what
    for f in ("bounds", "rot_center", "ws0", "wb0s0", "hs1", "hb1s1"):
        assert np.array_equal(np.ctypeslib.as_array(getattr(h, f)) if not isinstance(getattr(h, f), float)
                              else getattr(h, f),
                              np.ctypeslib.as_array(getattr(d, f)) if not isinstance(getattr(d, f), float)
                              else getattr(d, f)), (what, f)
    rows = 1 + (h.num_std if h.chaos_enable else 0)
    for r in range(rows):
        assert h.nbrk[r] == d.nbrk[r], (what, "nbrk", r)
        assert list(h.brk[r])[:h.nbrk[r]] == list(d.brk[r])[:d.nbrk[r]], (what, "brk", r)
    nv = sum(h.xf[i].nvars for i in range(h.num_xforms))
    assert list(h.var_id)[:nv] == list(d.var_id)[:nv], (what, "var_id")
    assert close(list(h.var_w)[:nv], list(d.var_w)[:nv]), (what, "var_w")
    hd = np.ctypeslib.as_array(h.dmap).reshape(256, 4)
    dd = np.ctypeslib.as_array(d.dmap).reshape(256, 4)
    assert np.array_equal(hd, dd), (what, "dmap", float(np.max(np.abs(hd - dd))))
    for i in range(h.num_xforms):
        a, b = h.xf[i], d.xf[i]
        for f in ("flags", "var_off", "nvars"):
            assert getattr(a, f) == getattr(b, f), (what, i, f)
        for f in ("c", "post", "prm"):
            assert close(list(getattr(a, f)), list(getattr(b, f))), (what, i, f)
        for f in ("color", "color_speed", "vis_adjusted", "opacity", "preblur"):
            assert close(getattr(a, f), getattr(b, f)), (what, i, f, getattr(a, f), getattr(b, f))


def test_pass_record_mirror_matches_library(gpulib):
    assert C.sizeof(F3GPass) == render.load().flam3gpu_pass_bytes()


@pytest.mark.parametrize("ci", range(len(interp_cases.cases())), ids=[c[0] for c in interp_cases.cases()])
def test_device_plan_equals_host_plan(gpulib, ci):
    name, gs, queries = interp_cases.cases()[ci]
    # the cases vary every genome scalar to test interpolation; a render also
    # needs valid frame settings, the same in every key (so that blends and
    # extrapolations stay valid): the xforms, palettes and matrices stay as
    # the cases make them
    for G in gs:
        g = G.g
        g.ntemporal_samples = 5
        g.temporal_filter_width = 0.8
        g.sample_density = 10.0
        g.width, g.height = 64, 48
        g.spatial_oversample = 1
        g.nbatches = 1
        g.estimator, g.estimator_minimum, g.estimator_curve = 0.0, 0.0, 0.4
        g.spatial_filter_radius = 0.5
        g.zoom = 0.0
        g.pixels_per_unit = 20.0
    checked = 0
    for qi, (t, stagger) in enumerate(queries):
        if stagger:
            continue  # flam3_render interpolates without stagger
        hp = passes(gm.Frame(gs, bits=33, seed="plan-%d" % qi, time=t), False)
        dp = passes(gm.Frame(gs, bits=33, seed="plan-%d" % qi, time=t), True)
        assert len(hp) == len(dp) == 5
        for k in range(5):
            compare(hp[k], dp[k], "%s t=%g sample %d" % (name, t, k))
        checked += 1
    assert checked > 0


def test_device_planned_animation_renders_like_host_planned(gpulib):
    """The animation workload's keys at a frame with motion blur: the same
    passes and random streams, so the two images agree to the FP32 noise of
    chains that start from coefficients a last bit apart."""
    gs = gm.animation_keys(2, width=320, height=180, quality=200.0, temporal_samples=20, estimator=3.0)
    outs = []
    for host in (1, 0):
        render.set_options(host_plan=host)
        try:
            img, st = render.render(gm.Frame(gs, bits=33, seed="anim-plan", time=37.5))
        finally:
            render.reset_options()
        outs.append((img, st.num_iters))
    assert outs[0][1] == outs[1][1]
    d = np.abs(outs[0][0].astype(np.int64) - outs[1][0].astype(np.int64))
    assert float(np.mean(d <= 1)) >= 0.99 and float(d.mean()) < 0.2, (float(np.mean(d <= 1)), float(d.mean()))
    assert outs[0][0].mean() > 1.0
