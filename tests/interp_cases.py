"""Seeded genome-interpolation cases shared by tests/golden/make_golden.py
(which runs them through the reference's flam3_interpolate, flam3.c:717-802)
and tests/test_interp_pin.py (which runs them through flam3gpu_interpolate).

Each case is a list of control points and a list of (time, stagger) queries.
The cases cover the branches of flam3_align (interpolation.c:768-1033):
unequal xform counts, a final xform on one side only, parametric variations
present on one side only, and every padding substitution (rotated linear -1
for spherical/ngon/julian/juliascope/polar/wedge_sph/wedge_julia,
rectangles/rings2/fan2/blob/perspective/curl/super_shape, fan/rings with
swapped coefficients, plain linear); and of flam3_interpolate_n
(interpolation.c:373-709): every palette interpolation mode, non-unity
palette alpha, log/linear/compat/older matrix interpolation, `wind`, zero and
tiny matrix rows, non-identity post matrices, chaos, stagger, extrapolation
outside the key times, and Catmull-Rom over four control points.
"""
import ctypes as C

import numpy as np

from flam3_gb300 import abi, genome as gm

VARIATIONS = list(range(0, 20)) + [21, 22, 23, 25, 26, 30, 32, 33, 38, 39, 40, 50, 78, 79]

# fields of a result genome that flam3_interpolate defines
GENOME_FIELDS = (
    "time interpolation interpolation_type palette_interpolation hsv_rgb_palette_blend num_xforms "
    "final_xform_index final_xform_enable symmetry palette_index brightness contrast gamma "
    "highlight_power width height spatial_oversample rotate vibrancy hue_rotation zoom "
    "pixels_per_unit spatial_filter_radius spatial_filter_select sample_density nbatches "
    "ntemporal_samples estimator estimator_curve estimator_minimum gam_lin_thresh "
    "temporal_filter_type temporal_filter_width temporal_filter_exp palette_mode"
).split()
GENOME_ARRAYS = (("center", 2), ("rot_center", 2), ("background", 3))

# xform fields left undefined by flam3_add_xforms (recomputed before a render)
XFORM_SKIP = {"vis_adjusted", "precalc_angles_flag", "precalc_atan_xy_flag", "precalc_atan_yx_flag",
              "has_preblur", "has_post", "waves_dx2", "waves_dy2", "super_shape_pm_4",
              "super_shape_pneg1_n1", "num_active_vars", "active_var_weights", "varFunc", "motion_freq",
              "motion_func", "motion", "num_motion"}


def _xform_vector(x):
    out = []
    for name, typ in abi.flam3_xform._fields_:
        if name in XFORM_SKIP:
            continue
        v = getattr(x, name)
        if name in ("c", "post"):
            out.extend(v[a][b] for a in range(3) for b in range(2))
        elif hasattr(v, "__len__"):
            out.extend(v)
        else:
            out.append(float(v))
    return out


def xform_field_names():
    names = []
    for name, typ in abi.flam3_xform._fields_:
        if name in XFORM_SKIP:
            continue
        if name in ("c", "post"):
            names.extend("%s%d%d" % (name, a, b) for a in range(3) for b in range(2))
        elif name in ("var", "wind"):
            n = abi.NVARS if name == "var" else 2
            names.extend("%s%d" % (name, k) for k in range(n))
        else:
            names.append(name)
    return names


def flatten(g):
    """(scalars, xforms, chaos, palette) of a flam3_genome as float64 arrays."""
    sc = [float(getattr(g, f)) for f in GENOME_FIELDS]
    for f, n in GENOME_ARRAYS:
        sc.extend(getattr(g, f)[k] for k in range(n))
    xf = np.array([_xform_vector(g.xform[i]) for i in range(g.num_xforms)], dtype=np.float64)
    ns = g.num_xforms - (1 if g.final_xform_index >= 0 else 0)
    ch = np.array([[g.chaos[i][j] for j in range(ns)] for i in range(ns)], dtype=np.float64).reshape(ns, ns)
    pal = np.array([[g.palette[i].index] + [g.palette[i].color[k] for k in range(4)] for i in range(256)])
    return np.array(sc, dtype=np.float64), xf, ch, pal


def _genome(rng, nstd, final=False, variations=VARIATIONS, t=0.0):
    G = gm.random_genome(rng, nstd, final=final, variations=variations)
    G.g.time = t
    for i in range(G.g.num_xforms):
        x = G.xform(i)
        for name in ("julian_power", "juliascope_power"):
            setattr(x, name, float(rng.integers(2, 5)))
        x.julian_dist = x.juliascope_dist = float(rng.uniform(0.5, 1.5))
        x.blob_low, x.blob_high, x.blob_waves = (float(v) for v in rng.uniform(0.2, 3, 3))
        x.fan2_x, x.fan2_y, x.rings2_val = (float(v) for v in rng.uniform(-1, 1, 3))
        x.perspective_angle, x.perspective_dist = float(rng.uniform(0, 1)), float(rng.uniform(1.5, 3))
        x.ngon_sides, x.ngon_power = float(rng.integers(3, 8)), float(rng.uniform(1, 4))
        x.curl_c1, x.curl_c2 = (float(v) for v in rng.uniform(-1, 1, 2))
        x.rectangles_x, x.rectangles_y = (float(v) for v in rng.uniform(0.2, 1.5, 2))
        x.super_shape_m, x.super_shape_n1 = float(rng.uniform(0, 8)), float(rng.uniform(0.5, 3))
        x.wedge_julia_power, x.wedge_julia_count = float(rng.integers(2, 4)), float(rng.integers(1, 4))
        x.opacity = float(rng.uniform(0.3, 1.0))
        x.color_speed = float(rng.uniform(0, 1))
        x.animate = float(rng.integers(0, 2))
    g = G.g
    g.brightness = float(rng.uniform(2, 6))
    g.contrast = float(rng.uniform(0.8, 1.2))
    g.gamma = float(rng.uniform(2, 5))
    g.vibrancy = float(rng.uniform(0.5, 1))
    g.hue_rotation = float(rng.uniform(0, 1))
    g.width = int(rng.integers(80, 400))
    g.height = int(rng.integers(60, 300))
    g.spatial_oversample = int(rng.integers(1, 4))
    g.center[0], g.center[1] = (float(v) for v in rng.uniform(-1, 1, 2))
    g.rot_center[0], g.rot_center[1] = (float(v) for v in rng.uniform(-1, 1, 2))
    g.background[0], g.background[1], g.background[2] = (float(v) for v in rng.uniform(0, 1, 3))
    g.pixels_per_unit = float(rng.uniform(30, 120))
    g.spatial_filter_radius = float(rng.uniform(0.3, 1.5))
    g.sample_density = float(rng.uniform(5, 50))
    g.zoom = float(rng.uniform(-0.5, 0.5))
    g.rotate = float(rng.uniform(-90, 90))
    g.nbatches = int(rng.integers(1, 4))
    g.ntemporal_samples = int(rng.integers(1, 60))
    g.estimator = float(rng.uniform(0, 9))
    g.estimator_minimum = float(rng.uniform(0, 0.5))
    g.estimator_curve = float(rng.uniform(0.3, 0.7))
    g.gam_lin_thresh = float(rng.uniform(0, 0.05))
    g.highlight_power = float(rng.uniform(-1, 2))
    g.temporal_filter_width = float(rng.uniform(0.5, 1.5))
    g.temporal_filter_exp = float(rng.uniform(-1, 1))
    return G


def _var_only(G, xi, j, w=1.0):
    x = G.xform(xi)
    for k in range(abi.NVARS):
        x.var[k] = 0.0
    x.var[j] = w


def cases(seed=777):
    rng = np.random.default_rng(seed)
    out = []
    q2 = [(0.0, 0.0), (0.3, 0.0), (1.0, 0.0), (-0.4, 0.0), (1.7, 0.0), (0.6, 0.5)]

    def add(name, gs, queries=q2):
        out.append((name, gs, list(queries)))

    # equal xform counts, each palette mode and matrix mode
    for pi in range(4):
        for it in range(4):
            a, b = _genome(rng, 3, t=0.0), _genome(rng, 3, t=1.0)
            for G in (a, b):
                G.g.palette_interpolation = pi
                G.g.interpolation_type = it
                G.g.hsv_rgb_palette_blend = 0.3 if pi == 3 and it == 1 else 0.0
            add("pal%d_int%d" % (pi, it), [a, b])
    # palette alpha below one on one side
    a, b = _genome(rng, 2, t=0.0), _genome(rng, 2, t=1.0)
    pal = a.palette_array()
    pal[::3, 3] = 0.5
    a.set_palette(pal)
    add("alpha", [a, b])
    # unequal counts and final xforms, log and linear
    for it in (1, 0, 3):
        for fa, fb in ((False, True), (True, False), (True, True)):
            a, b = _genome(rng, 2, final=fa, t=0.0), _genome(rng, 4, final=fb, t=2.0)
            for G in (a, b):
                G.g.interpolation_type = it
            add("pad_int%d_f%d%d" % (it, fa, fb), [a, b], [(0.0, 0.0), (0.5, 0.0), (1.2, 0.0), (2.0, 0.3)])
    # every padding substitution: the longer genome's extra xform uses one variation
    for j in (2, 38, 32, 33, 5, 79, 78, 40, 26, 25, 23, 30, 39, 50, 22, 21, 9, 1):
        for it in (1, 0):
            a, b = _genome(rng, 1, t=0.0), _genome(rng, 2, t=1.0)
            _var_only(b, 1, j, float(rng.uniform(0.5, 1.5)))
            for G in (a, b):
                G.g.interpolation_type = it
            add("subst_v%d_int%d" % (j, it), [b, a] if j % 2 else [a, b], [(0.4, 0.0)])
    # parametric variation on one side only: its parameters are borrowed
    a, b = _genome(rng, 2, t=0.0), _genome(rng, 2, t=1.0)
    for j in (32, 23, 50, 78):
        a.xform(0).var[j] = 0.0
        b.xform(0).var[j] = 0.7
    add("borrow", [a, b])
    # wind, zero rows, tiny rows, post matrices, chaos
    a, b = _genome(rng, 3, t=0.0), _genome(rng, 3, t=1.0)
    b.xform(0).wind[0] = 2.0
    b.xform(1).wind[1] = 5.0
    a.xform(1).c[0][0] = a.xform(1).c[0][1] = 0.0
    b.xform(2).c[1][0], b.xform(2).c[1][1] = 1e-6, -1e-6
    for k in range(6):
        a.xform(2).post[k // 2][k % 2] = float(rng.uniform(-1, 1))
    a.set_chaos(0, 1, 0.0)
    a.set_chaos(2, 2, 2.5)
    b.set_chaos(1, 0, 0.25)
    add("wind_rows_post_chaos", [a, b])
    # three keys: segment selection
    gs = [_genome(rng, 3, t=float(t)) for t in (0.0, 1.0, 3.0)]
    add("three_keys", gs, [(0.5, 0.0), (1.0, 0.0), (2.0, 0.0), (3.5, 0.0)])
    # Catmull-Rom on the middle segment of four keys
    gs = [_genome(rng, 3, t=float(t)) for t in (0.0, 1.0, 2.0, 3.0)]
    for G in gs:
        G.g.interpolation = 1
    add("smooth", gs, [(1.25, 0.0), (1.5, 0.0), (1.9, 0.0)])
    gs = [_genome(rng, n, final=(n == 3), t=float(t)) for n, t in ((2, 0.0), (3, 1.0), (2, 2.0), (4, 3.0))]
    for G in gs:
        G.g.interpolation = 1
    add("smooth_pad", gs, [(1.5, 0.0)])
    return out


def genome_array(gs):
    """A contiguous flam3_genome array over Genome objects (pointers shared)."""
    arr = (abi.flam3_genome * len(gs))(*[G.g for G in gs])
    return arr
