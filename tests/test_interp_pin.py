"""Pins libflam3gpu's genome interpolation (flam3gpu_interpolate, host FP64)
to the reference's flam3_interpolate (flam3.c:717-802): field for field
against the golden results of tests/golden/interp.npz on any machine, bit for
bit against the reference library itself where it was built here
(oracle/_ref).  Then pins the oracle's multi-genome renders (which take the
interpolator from the caller) against the reference's own flam3_render of
the same animation frames.

On x86-64 the strict builds agree bit for bit; elsewhere libm may round the
last bit of atan2/exp/log/sin/cos differently, so floating-point fields are
held to 1e-12 relative there and whole renders to a small mean error."""
import ctypes as C
import os
import platform

import numpy as np
import pytest

from flam3_gb300 import abi, render
import _oracle
import interp_cases
from golden import make_golden as mg

GOLD = os.path.join(os.path.dirname(__file__), "golden")
X86 = platform.machine() in ("x86_64", "AMD64")
INT_SCALARS = {"interpolation", "interpolation_type", "palette_interpolation", "num_xforms", "final_xform_index",
               "final_xform_enable", "symmetry", "palette_index", "width", "height", "spatial_oversample",
               "spatial_filter_select", "nbatches", "ntemporal_samples", "temporal_filter_type", "palette_mode"}

CASES = interp_cases.cases()


def _close(a, b, exact):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.shape != b.shape:
        return False
    if exact:
        return np.array_equal(a, b)
    return bool(np.all(np.abs(a - b) <= 1e-12 + 1e-12 * np.maximum(np.abs(a), np.abs(b))))


def _check(got, want, exact, what):
    sc, xf, ch, pal = got
    wsc, wxf, wch, wpal = want
    names = interp_cases.GENOME_FIELDS + ["center0", "center1", "rot_center0", "rot_center1", "bg0", "bg1", "bg2"]
    for k, n in enumerate(names):
        if n in INT_SCALARS:
            assert sc[k] == wsc[k], (what, n, sc[k], wsc[k])
        else:
            assert _close(sc[k], wsc[k], exact), (what, n, sc[k], wsc[k])
    assert xf.shape == wxf.shape, (what, xf.shape, wxf.shape)
    xnames = interp_cases.xform_field_names()
    for i in range(xf.shape[0]):
        for k, n in enumerate(xnames):
            if n == "padding":
                assert xf[i, k] == wxf[i, k], (what, i, n)
            else:
                assert _close(xf[i, k], wxf[i, k], exact), (what, "xform", i, n, xf[i, k], wxf[i, k])
    assert _close(ch, wch, exact), (what, "chaos")
    assert _close(pal, wpal, exact), (what, "palette", np.max(np.abs(pal - wpal)) if pal.shape == wpal.shape else -1)


def _product(gs, t, stagger):
    r = render.interpolate(gs, t, stagger)
    return interp_cases.flatten(r.g)


def test_case_inventory():
    names = [c[0] for c in CASES]
    assert len(names) == len(set(names))
    assert sum(len(c[2]) for c in CASES) >= 150


@pytest.mark.parametrize("ci", range(len(CASES)), ids=[c[0] for c in CASES])
def test_interpolate_matches_reference_goldens(ci):
    d = np.load(os.path.join(GOLD, "interp.npz"))
    name, gs, queries = CASES[ci]
    for qi, (t, stagger) in enumerate(queries):
        key = "%s_q%d" % (name, qi)
        want = tuple(d[key + s] for s in ("_scalars", "_xforms", "_chaos", "_palette"))
        _check(_product(gs, t, stagger), want, X86, key)


@pytest.mark.skipif(_oracle.reference(True) is None, reason="reference not built on this machine")
def test_interpolate_matches_reference_directly():
    ref = _oracle.reference(True)
    ref.flam3_interpolate.argtypes = [C.POINTER(abi.flam3_genome), C.c_int, C.c_double, C.c_double,
                                      C.POINTER(abi.flam3_genome)]
    ref.flam3_interpolate.restype = None
    rng = np.random.default_rng(99)
    n = 0
    for name, gs, queries in CASES:
        arr = interp_cases.genome_array(gs)
        extra = [(float(rng.uniform(gs[0].g.time - 0.5, gs[-1].g.time + 0.5)), float(rng.choice([0.0, 0.7])))
                 for _ in range(3)]
        for t, stagger in list(queries) + extra:
            if any(G.g.interpolation == 1 for G in gs) and len(gs) == 4 and not (1.0 < t < 2.0):
                continue  # smooth outside the middle segment reads past the keys in the reference
            out = abi.flam3_genome()
            ref.flam3_interpolate(arr, len(gs), t, stagger, C.byref(out))
            _check(_product(gs, t, stagger), interp_cases.flatten(out), X86, "%s t=%g s=%g" % (name, t, stagger))
            n += 1
    assert n > 200


def test_interpolate_single_genome_is_a_copy():
    gs = CASES[0][1][:1]
    r = render.interpolate(gs, 0.7)
    assert r.g.num_xforms == gs[0].g.num_xforms
    for i in range(r.g.num_xforms):
        assert list(r.g.xform[i].var) == list(gs[0].g.xform[i].var)


def test_interpolate_rejects_empty():
    lib = render.load()
    out = abi.flam3_genome()
    assert lib.flam3gpu_interpolate(None, 0, 0.0, 0.0, C.byref(out)) == 1
    assert b"no genomes" in lib.flam3gpu_last_error()


@pytest.mark.parametrize("setting", mg.ANIM_SETTINGS, ids=[s[0] for s in mg.ANIM_SETTINGS])
def test_oracle_animation_renders_match_reference_goldens(setting):
    d = np.load(os.path.join(GOLD, "interp.npz"))
    F = mg.make_anim_frame(setting)
    _oracle.set_interpolator("product")
    out, st, _ = _oracle.oracle_render(F)
    ref = d[setting[0]]
    assert [st.num_iters, st.badvals] == list(d[setting[0] + "__iters"])
    if X86:
        np.testing.assert_array_equal(out, ref)
    else:
        mae = np.mean(np.abs(out.astype(float) - ref.astype(float)))
        assert mae < 1.5, mae


@pytest.mark.skipif(_oracle.reference(True) is None, reason="reference not built on this machine")
def test_oracle_animation_with_reference_interpolator():
    """The same frame rendered by the oracle with the reference's own
    flam3_interpolate installed: identical to the golden render."""
    d = np.load(os.path.join(GOLD, "interp.npz"))
    s = mg.ANIM_SETTINGS[0]
    F = mg.make_anim_frame(s)
    _oracle.set_interpolator("reference")
    try:
        out, st, _ = _oracle.oracle_render(F)
    finally:
        _oracle.set_interpolator("product")
    np.testing.assert_array_equal(out, d[s[0]])
