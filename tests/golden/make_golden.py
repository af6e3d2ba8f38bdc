"""Generates the golden fixtures in tests/golden/ from the reference flam3
library, compiled unmodified from its sources by oracle/Makefile (`make -C
oracle ref`), so the tests can pin the oracle and the CUDA path on machines
where the reference tree does not exist.

  variations.npz  per-variation apply_xform vectors (variations.c:2129-2399):
                  random xform parameters, points and random words, and the
                  reference's outputs.
  renders.npz     small whole renders through the reference flam3_render
                  (strict IEEE build, nthreads=1) for a set of settings.
  isaac.npz       irand() words for seeded contexts (isaac.c).
  filters.npz     spatial / DE / temporal filter tables (filters.c).
  abi_offsets.txt struct layout of flam3.h as printed by oracle/abi_offsets.c.
  interp.npz      flam3_interpolate (flam3.c:717-802) results for the seeded
                  cases of tests/interp_cases.py, and small multi-genome
                  (animation / motion blur) renders through flam3_render.

Run from the repository root:  python tests/golden/make_golden.py [section ...]
(sections: variations renders isaac filters abi interp; default all)
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from flam3_gb300 import abi, genome as gm  # noqa: E402
import _oracle  # noqa: E402
import interp_cases  # noqa: E402

OUT = os.path.join(ROOT, "tests", "golden")

# parameter sampling: (low, high, integer, nonzero)
SPECIAL = {
    "julian_power": (-5, 6, True, True), "juliascope_power": (-5, 6, True, True),
    "wedge_julia_power": (-4, 5, True, True), "pie_slices": (1, 9, True, True),
    "ngon_sides": (2, 9, True, True), "cpow_power": (1, 6, True, True), "wedge_count": (1, 7, True, True),
    "wedge_sph_count": (1, 7, True, True), "wedge_julia_count": (1, 5, True, True),
    "cell_size": (0.2, 1.5, False, True), "super_shape_n1": (0.5, 3.0, False, True),
    "super_shape_m": (0.0, 8.0, False, False), "flower_petals": (0.0, 8.0, False, False),
    "conic_eccentricity": (0.05, 1.0, False, True), "curve_xlength": (0.3, 2.0, False, True),
    "curve_ylength": (0.3, 2.0, False, True), "ngon_power": (0.5, 4.0, False, False),
    "oscope_damping": (0.0, 1.0, False, False), "pie_thickness": (0.0, 1.0, False, False),
    "super_shape_rnd": (0.0, 1.0, False, False), "rectangles_x": (0.2, 1.5, False, True),
    "rectangles_y": (0.2, 1.5, False, True), "modulus_x": (0.2, 1.5, False, True),
    "modulus_y": (0.2, 1.5, False, True), "perspective_dist": (1.5, 3.0, False, True),
}


def sample_param(rng, name):
    lo, hi, integer, nonzero = SPECIAL.get(name, (-1.5, 1.5, False, False))
    while True:
        v = int(rng.integers(lo, hi)) if integer else float(rng.uniform(lo, hi))
        if not nonzero or v != 0:
            return float(v)


def variation_cases(seed=12345, npoints=32):
    rng = np.random.default_rng(seed)
    cases = []
    for v in range(abi.NVARS):
        for variant in range(2):
            extra = []
            if variant == 1:
                # a second variation and sometimes pre_blur, to exercise sums
                extra = [int(rng.integers(0, abi.NVARS))]
                if rng.uniform() < 0.3:
                    extra.append(67)
            case = {
                "coefs": rng.uniform(-1.2, 1.2, 6),
                "post": rng.uniform(-1, 1, 6) if rng.uniform() < 0.4 else np.array([1, 0, 0, 1, 0, 0.0]),
                "var": np.zeros(abi.NVARS),
                "params": np.array([sample_param(rng, n) for n in abi.XFORM_PARAMS]),
                "color": rng.uniform(0, 1), "color_speed": rng.uniform(0, 1), "opacity": rng.uniform(0.2, 1),
                "points": np.stack([rng.uniform(-2, 2, npoints), rng.uniform(-2, 2, npoints),
                                    rng.uniform(0, 1, npoints), rng.uniform(0, 1, npoints)], 1),
                "words": rng.integers(0, 2 ** 32, size=(npoints, 16), dtype=np.uint64).astype(np.uint32),
            }
            for vv in [v] + extra:
                case["var"][vv] = rng.uniform(0.3, 1.2) * (1 if rng.uniform() < 0.8 else -1)
            cases.append(case)
    return cases


def genome_from_case(case):
    G = gm.Genome(1)
    x = G.xform(0)
    for k in range(6):
        x.c[k // 2][k % 2] = case["coefs"][k]
        x.post[k // 2][k % 2] = case["post"][k]
    for j in range(abi.NVARS):
        x.var[j] = case["var"][j]
    for name, val in zip(abi.XFORM_PARAMS, case["params"]):
        setattr(x, name, float(val))
    x.color = float(case["color"])
    x.color_speed = float(case["color_speed"])
    x.opacity = float(case["opacity"])
    x.density = 1.0
    return G


RENDER_SETTINGS = [
    # name, genome seed, bits, est, oversample, earlyclip, nchan, transp, bpc, field, nthreads
    ("c0_b33", 0, 33, 0.0, 1, 0, 3, 0, 1, 0, 1),
    ("c0_b64", 1, 64, 0.0, 1, 0, 3, 0, 1, 0, 1),
    ("c0_b32", 2, 32, 0.0, 1, 0, 3, 0, 1, 0, 1),
    ("c0_de3_b64", 0, 64, 3.0, 1, 0, 3, 0, 1, 0, 1),
    ("c0_de2_ss2_b33", 1, 33, 2.0, 2, 0, 3, 0, 1, 0, 1),
    ("c0_early_rgba_transp", 2, 64, 0.0, 1, 1, 4, 1, 1, 0, 1),
    ("c0_bpc16_rgba", 0, 33, 0.0, 1, 0, 4, 0, 2, 0, 1),
    ("c0_field_odd", 1, 33, 0.0, 1, 0, 3, 0, 1, 2, 1),
    ("c0_nt3_b33", 2, 33, 0.0, 1, 0, 3, 0, 1, 0, 3),
    ("c1_final_b64_de", 5, 64, 4.0, 1, 0, 3, 0, 1, 0, 1),
]


def render_genome(seed):
    if seed >= 5:
        G = gm.still_genome(seed, width=96, height=72, quality=30.0, oversample=1, estimator=4.0)
    else:
        G = gm.small_genome(seed)
        gm.resize(G, 96, 72)
        G.g.sample_density = 30.0
    return G


def make_render_frame(setting):
    name, seed, bits, est, ss, early, nchan, transp, bpc, field, nt = setting
    G = render_genome(seed)
    G.g.estimator = est
    G.g.spatial_oversample = ss
    return gm.Frame(G, bits=bits, nthreads=nt, seed="golden-%s" % name, earlyclip=early, bytes_per_channel=bpc), \
        nchan, transp, field


# multi-genome renders: name, genome seed, bits, estimator, time, temporal samples, nbatches
ANIM_SETTINGS = [
    ("anim_b64_de", 2, 64, 3.0, 40.0, 6, 1),
    ("anim_b33_t2", 3, 33, 0.0, 85.0, 5, 2),
    ("anim_b64_edge", 4, 64, 0.0, 0.0, 4, 1),
]


def make_anim_frame(setting):
    name, seed, bits, est, t, nts, nb = setting
    gs = gm.animation_keys(seed, width=96, height=72, quality=20.0, temporal_samples=nts, estimator=est)
    for G in gs:
        G.g.nbatches = nb
    return gm.Frame(gs, bits=bits, nthreads=1, seed="golden-%s" % name, time=t)


def make_interp(ref):
    ref.flam3_interpolate.argtypes = [C.POINTER(abi.flam3_genome), C.c_int, C.c_double, C.c_double,
                                      C.POINTER(abi.flam3_genome)]
    ref.flam3_interpolate.restype = None
    res = {}
    for ci, (name, gs, queries) in enumerate(interp_cases.cases()):
        arr = interp_cases.genome_array(gs)
        for qi, (t, stagger) in enumerate(queries):
            out = abi.flam3_genome()
            ref.flam3_interpolate(arr, len(gs), t, stagger, C.byref(out))
            sc, xf, ch, pal = interp_cases.flatten(out)
            key = "%s_q%d" % (name, qi)
            res[key + "_scalars"], res[key + "_xforms"] = sc, xf
            res[key + "_chaos"], res[key + "_palette"] = ch, pal
    for s in ANIM_SETTINGS:
        F = make_anim_frame(s)
        out = F.out_buffer(3)
        st = abi.stat_struct()
        r = ref.flam3_render(C.byref(F.f), out.ctypes.data, 0, 3, 0, C.byref(st))
        assert r == 0, s
        res[s[0]] = out
        res[s[0] + "__iters"] = np.array([st.num_iters, st.badvals])
    np.savez_compressed(os.path.join(OUT, "interp.npz"), **res)


def main():
    ref = _oracle.reference(True)
    if ref is None:
        sys.exit("build the reference first: make -C oracle ref REF=<reference source tree>")
    os.makedirs(OUT, exist_ok=True)
    sections = set(sys.argv[1:]) or {"variations", "renders", "isaac", "filters", "abi", "interp"}
    if "interp" in sections:
        make_interp(ref)

    # --- variations
    if "variations" in sections:
        cases = variation_cases()
        arrays = {k: [] for k in ("coefs", "post", "var", "params", "color", "color_speed", "opacity", "points",
                                  "words", "q", "bad")}
        for case in cases:
            G = genome_from_case(case)
            q, bad = _oracle.ref_apply_xform(G, 0, case["points"], case["words"])
            for k in ("coefs", "post", "var", "params", "color", "color_speed", "opacity", "points", "words"):
                arrays[k].append(case[k])
            arrays["q"].append(q)
            arrays["bad"].append(bad)
        np.savez_compressed(os.path.join(OUT, "variations.npz"), **{k: np.array(v) for k, v in arrays.items()},
                            param_names=np.array(abi.XFORM_PARAMS))

    # --- renders
    if "renders" in sections:
        imgs = {}
        for s in RENDER_SETTINGS:
            F, nchan, transp, field = make_render_frame(s)
            out = F.out_buffer(nchan)
            st = abi.stat_struct()
            r = ref.flam3_render(C.byref(F.f), out.ctypes.data, field, nchan, transp, C.byref(st))
            assert r == 0, s
            imgs[s[0]] = out
            imgs[s[0] + "__iters"] = np.array([st.num_iters, st.badvals])
            imgs[s[0] + "__rc"] = np.array([F.f.rc.randrsl[i] for i in range(16)] + [F.f.rc.randcnt], dtype=np.uint64)
        np.savez_compressed(os.path.join(OUT, "renders.npz"), **imgs)

    # --- isaac
    if "isaac" in sections:
        lib = _oracle.oracle()
        rows = []
        for seed in (b"", b"abc", b"flam3-gb300", b"x" * 200):
            rc = abi.randctx()
            lib.f3o_init_rc(C.byref(rc), seed)
            rows.append([lib.f3o_irand(C.byref(rc)) for _ in range(100)])
        # the reference's own seeding: flam3_init_frame reads isaac_seed from env
        ref_rows = []
        for seed in ("", "abc", "flam3-gb300", "x" * 200):
            env = dict(os.environ, isaac_seed=seed)
            code = ("import ctypes as C,sys;sys.path.insert(0,%r);from flam3_gb300 import abi;"
                    "L=C.CDLL(%r);f=abi.flam3_frame();L.flam3_init_frame(C.byref(f));"
                    "L.irandinit;print(' '.join(str(f.rc.randrsl[i]) for i in range(16)), f.rc.randcnt)"
                    % (ROOT, os.path.join(_oracle.REF_DIR, "libflam3ref_strict.so")))
            r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, check=True)
            ref_rows.append([int(t) for t in r.stdout.split()])
        np.savez_compressed(os.path.join(OUT, "isaac.npz"), oracle_words=np.array(rows, dtype=np.uint64),
                            ref_init=np.array(ref_rows, dtype=np.uint64))

    # --- filters (reference functions)
    if "filters" in sections:
        ref.flam3_create_temporal_filter.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double,
                                                     C.POINTER(C.POINTER(C.c_double)), C.POINTER(C.POINTER(C.c_double))]
        ref.flam3_create_temporal_filter.restype = C.c_double

        class DEHelper(C.Structure):
            _fields_ = [("max_filtered_counts", C.c_int), ("max_filter_index", C.c_int), ("kernel_size", C.c_int),
                        ("filter_widths", C.POINTER(C.c_double)), ("filter_coefs", C.POINTER(C.c_double))]

        ref.flam3_create_de_filters.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int]
        ref.flam3_create_de_filters.restype = DEHelper
        ref.flam3_create_spatial_filter.argtypes = [C.POINTER(abi.flam3_frame), C.c_int, C.POINTER(C.POINTER(C.c_double))]
        fil = {}
        for (rad, mn, curve, ss) in [(9, 0, 0.4, 2), (7, 0, 0.4, 1), (11, 0, 0.4, 2), (3, 0.5, 0.6, 1), (2, 0, 0.4, 3)]:
            d = ref.flam3_create_de_filters(rad, mn, curve, ss)
            n = d.max_filter_index + 1
            key = "de_%g_%g_%g_%d" % (rad, mn, curve, ss)
            fil[key + "_meta"] = np.array([d.max_filtered_counts, d.max_filter_index, d.kernel_size])
            fil[key + "_widths"] = np.array([d.filter_widths[i] for i in range(n)])
            fil[key + "_coefs"] = np.array([d.filter_coefs[i] for i in range(n * d.kernel_size)])
        for (n, typ, fexp, width) in [(1, 0, 0, 1), (100, 0, 0, 1), (50, 1, 0, 1.5), (40, 2, 1.5, 1), (40, 2, -2, 1)]:
            tf, td = C.POINTER(C.c_double)(), C.POINTER(C.c_double)()
            s = ref.flam3_create_temporal_filter(n, typ, fexp, width, C.byref(tf), C.byref(td))
            key = "tf_%d_%d_%g_%g" % (n, typ, fexp, width)
            fil[key] = np.array([tf[i] for i in range(n)] + [td[i] for i in range(n)] + [s])
        for knum in range(14):
            for (ss, rad, field, aspect) in [(1, 0.5, 0, 1.0), (2, 1.0, 0, 1.0), (3, 0.7, 1, 1.3)]:
                G = gm.small_genome(0)
                G.g.spatial_filter_select = knum
                G.g.spatial_oversample = ss
                G.g.spatial_filter_radius = rad
                F = gm.Frame(G, pixel_aspect_ratio=aspect)
                fp = C.POINTER(C.c_double)()
                w = ref.flam3_create_spatial_filter(C.byref(F.f), field, C.byref(fp))
                fil["sf_%d_%d_%g_%d_%g" % (knum, ss, rad, field, aspect)] = np.array([w] + [fp[i] for i in range(w * w)])
        np.savez_compressed(os.path.join(OUT, "filters.npz"), **fil)

    # --- ABI
    if "abi" in sections:
        r = subprocess.run([os.path.join(_oracle.REF_DIR, "abi_offsets")], capture_output=True, text=True, check=True)
        with open(os.path.join(OUT, "abi_offsets.txt"), "w") as f:
            f.write(r.stdout)

    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    main()
