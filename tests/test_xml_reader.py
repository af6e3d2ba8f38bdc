"""The flame genome XML reader (flam3gpu_parse_xml2) against the reference's
flam3_parse_xml2 built from its sources (where the reference tree was
available at build time): every scalar field of every parsed genome, every
xform (and motion element) field, the chaos rows and the palette are equal.
The documents below exercise the format's features; a small palette library
written here stands in for the reference's ($flam3_palettes, honoured by
both).  Host code only: no GPU."""
import ctypes as C
import os

import numpy as np
import pytest

from flam3_gb300 import abi, genome as gm, render
import _oracle

LIBC = C.CDLL(None)


def _hex(n, chan, seed):
    rng = np.random.default_rng(seed)
    cols = rng.integers(0, 256, (n, 4))
    if chan == 3:
        return "\n".join("".join("%02X%02X%02X" % tuple(c[:3]) for c in cols[i:i + 8]) for i in range(0, n, 8))
    if chan == 4:
        return "".join("%02X%02X%02X%02X" % tuple(c) for c in cols)
    return "".join("00%02X%02X%02X" % tuple(c[:3]) for c in cols)


@pytest.fixture(scope="module")
def palette_library(tmp_path_factory):
    p = tmp_path_factory.mktemp("pal") / "palettes.xml"
    body = "".join('<palette number="%d" name="p%d" data="%s"/>\n' % (k, k, _hex(256, -4, 100 + k)) for k in range(5))
    p.write_text("<palettes>\n" + body + "</palettes>\n")
    os.environ["flam3_palettes"] = str(p)
    return p


DOCS = {
    "basic": """<flames><flame name="two words" time="3" size="320 240" center="0.25 -0.5" scale="80"
      rotate="12.5" zoom="0.5" oversample="2" filter="0.75" filter_shape="mitchell" quality="50" passes="2"
      temporal_samples="10" temporal_filter_type="gaussian" temporal_filter_width="1.5" temporal_filter_exp="0.3"
      background="0.1 0.2 0.3" brightness="3.5" gamma="2.2" highlight_power="1.25" vibrancy="0.8"
      estimator_radius="7" estimator_minimum="1" estimator_curve="0.6" gamma_threshold="0.02"
      palette_mode="linear" interpolation="smooth" interpolation_type="linear" palette_interpolation="rgb"
      hsv_rgb_palette_blend="0.25" contrast="9">
      <xform weight="0.5" color="0" color_speed="0.3" spherical="1" coefs="0.5 0 0 0.5 0 0" opacity="0.75"/>
      <xform weight="0.25" color="1 0" symmetry="0.4" linear="0.7" julian="0.3" julian_power="3"
        julian_dist="-1" coefs="0.5 0.1 -0.1 0.5 0.5 0" post="1 0.2 0 1 0.1 0.1"/>
      <xform weight="0.25" color="0.5" animate="0" rings2="1" rings2_val="0.4" blob="0.2" blob_low="0.3"
        super_shape="0.5" super_shape_rnd="1.7" super_shape_m="5" Re_A="0.3" mobius_im_b="0.2" mobius="0.1"
        oscilloscope_frequency="2" oscope_damping="0.1" coefs="-0.5 0 0 0.5 0 0.5"/>
      <color index="0" rgb="255 0 0"/><color index="100" rgba="0 255 0 128"/><color index="255" a="64" rgb="0 0 255"/>
    </flame></flames>""",
    "final_first_chaos_solo": """<flame size="64 64" soloxform="1">
      <finalxform color="0.5" swirl="1" coefs="1 0 0 1 0 0"/>
      <xform weight="1" color="0" linear="1" chaos="1 0.5 2" coefs="0.5 0 0 0.5 0 0"/>
      <xform weight="1" color="1" sinusoidal="1" chaos="0 1" coefs="0.5 0 0 0.5 0.5 0"/>
      <xform weight="2" color="0.3" polar="1" plotmode="off" coefs="0.5 0 0 0.5 0 0.5"/>
      <palette count="256" format="RGB">
      %s
      </palette>
    </flame>""" % _hex(256, 3, 1),
    # flames as siblings: the reference's scan reallocates its array through a
    # stale pointer when flames sit at different depths (undefined behaviour)
    "many_flames_time_carry_defaults": """<doc><flame name="first" time="7" size="10 10">
      <xform weight="1" linear="1" coefs="1 0 0 1 0 0"/></flame>
      <flame name="second"><xform weight="1" var1="13" coefs="1 0 0 1 0 0"/></flame>
      <flame name="third" time="2" supersample="3"><xform weight="1" var="%s" coefs="1 0 0 1 0 0"/></flame></doc>"""
    % " ".join("%g" % (0.01 * (i % 7)) for i in range(99)),
    "colors_old_hex_missing": """<flame size="32 32"><xform weight="1" linear="1" coefs="1 0 0 1 0 0"/>
      <colors count="64" data="%s"/><color index="200" rgb="10 20 30"/></flame>""" % _hex(64, -4, 2),
    "rgba_palette": """<flame size="32 32"><xform weight="1" linear="1" coefs="1 0 0 1 0 0"/>
      <palette count="256" format="RGBA">%s</palette></flame>""" % _hex(256, 4, 3),
    "symmetry_motion": """<flame size="32 32"><xform weight="1" linear="1" coefs="0.4 0 0 0.4 0.3 0">
      <motion motion_frequency="2" motion_function="triangle" linear="0.5" coefs="0.1 0 0 0.1 0 0"/>
      <motion motion_frequency="1" motion_function="sin" julian_power="1"/></xform>
      <symmetry kind="3"/><symmetry kind="-2"/>
      <xform weight="1" ex="1" coefs="0.3 0 0 0.3 0 0"/></flame>""",
    "symmetry_random": """<flame size="32 32"><xform weight="1" linear="1" coefs="0.4 0 0 0.4 0.3 0"/>
      <symmetry kind="0"/></flame>""",
    "library_palette_hue": """<flames><flame size="16 16" palette="3" hue="1.25"><xform weight="1" linear="1"
      coefs="1 0 0 1 0 0"/></flame><flame size="16 16"><xform weight="1" linear="1" coefs="1 0 0 1 0 0"/>
      <palette index0="1" index1="4" hue0="0.1" hue1="0.7" blend="0.3"/></flame>
      <flame size="16 16" palette="99"><xform weight="1" linear="1" coefs="1 0 0 1 0 0"/></flame></flames>""",
    "entities_comments": """<?xml version="1.0"?><!DOCTYPE flames><!-- a comment -->
      <flames><flame name="a&amp;b &#65;" size="8 8"><![CDATA[ignored]]><edit date="x"><edit/></edit>
      <xform weight="1" linear="1" coefs="1 0 0 1 0 0"/></flame></flames>""",
    "no_colors": """<flame size="8 8"><xform weight="1" linear="1" coefs="1 0 0 1 0 0"/></flame>""",
}

BAD_DOCS = {
    "trailing_chars": '<flame size="8 8" quality="1.5x"><xform weight="1" linear="1"/></flame>',
    "bad_size": '<flame size="8"><xform weight="1" linear="1"/></flame>',
    "two_finals": '<flame size="8 8"><finalxform linear="1"/><finalxform linear="1"/></flame>',
    "final_with_weight": '<flame size="8 8"><finalxform weight="1" linear="1"/></flame>',
    "bad_color_index": '<flame size="8 8"><xform weight="1" linear="1"/><color index="300" rgb="1 2 3"/></flame>',
}
# malformed XML (libxml2 rejects it; the reference as built here parses with a
# lenient stand-in for libxml2, so only the reader itself is checked)
UNCLOSED = '<flame size="8 8"><xform weight="1" linear="1"></flame>'



def _ref():
    ref = _oracle.reference(strict=True)
    if ref is None:
        pytest.skip("the reference was not built here")
    ref.flam3_parse_xml2.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.POINTER(C.c_int)]
    ref.flam3_parse_xml2.restype = C.POINTER(abi.flam3_genome)
    return ref


def _parse(fn, text, default_flag):
    LIBC.srandom(12345)
    n = C.c_int(0)
    buf = C.create_string_buffer(text.encode())
    p = fn(buf, C.c_char_p(b"some/dir/doc.flam3"), default_flag, C.byref(n))
    return p, n.value


SKIP_G = {"xform", "chaos", "edits"}
# xform fields the reference leaves as they were in reallocated memory; they
# are derived from the others by prepare_precalc_flags / xform_precalc
# before any render (variations.c:1942-2126)
SKIP_X = {"motion", "vis_adjusted", "precalc_angles_flag", "precalc_atan_xy_flag", "precalc_atan_yx_flag",
          "has_preblur", "has_post", "waves_dx2", "waves_dy2", "super_shape_pm_4", "super_shape_pneg1_n1",
          "num_active_vars", "active_var_weights", "varFunc", "persp_vsin", "persp_vfcos", "julian_rN",
          "julian_cn", "juliascope_rN", "juliascope_cn", "wedgeJulia_rN", "wedgeJulia_cn", "wedgeJulia_cf",
          "radialBlur_spinvar", "radialBlur_zoomvar", "disc2_sinadd", "disc2_cosadd", "disc2_timespi"}


def _cmp_struct(a, b, skip, where):
    for name, _ in type(a)._fields_:
        if name in skip:
            continue
        va, vb = getattr(a, name), getattr(b, name)
        if hasattr(va, "__len__") and not isinstance(va, (bytes, str)):
            va = np.array(np.ctypeslib.as_array(va) if not isinstance(va, C.Array) or not isinstance(
                va[0], C.Structure) else [[e.index, *e.color] for e in va], dtype=float)
            vb = np.array(np.ctypeslib.as_array(vb) if not isinstance(vb, C.Array) or not isinstance(
                vb[0], C.Structure) else [[e.index, *e.color] for e in vb], dtype=float)
            assert np.array_equal(va, vb, equal_nan=True), (where, name)
        else:
            assert va == vb or (va != va and vb != vb), (where, name, va, vb)


def _cmp_genome(ga, gb, where):
    _cmp_struct(ga, gb, SKIP_G, where)
    assert ga.num_xforms == gb.num_xforms
    ns = ga.num_xforms - (ga.final_xform_index >= 0)
    for i in range(ga.num_xforms):
        xa, xb = ga.xform[i], gb.xform[i]
        _cmp_struct(xa, xb, SKIP_X, "%s xform %d" % (where, i))
        assert xa.num_motion == xb.num_motion
        for m in range(xa.num_motion):
            _cmp_struct(xa.motion[m], xb.motion[m], SKIP_X, "%s xform %d motion %d" % (where, i, m))
    for i in range(ns):
        assert [ga.chaos[i][j] for j in range(ns)] == [gb.chaos[i][j] for j in range(ns)], (where, "chaos", i)


@pytest.mark.parametrize("default_flag", [1, 0])
@pytest.mark.parametrize("name", sorted(DOCS))
def test_reader_equals_reference(palette_library, name, default_flag):
    ref = _ref()
    ours = render.load()
    pr, nr = _parse(ref.flam3_parse_xml2, DOCS[name], default_flag)
    po, no = _parse(ours.flam3gpu_parse_xml2, DOCS[name], default_flag)
    assert bool(pr) and bool(po) and nr == no and nr > 0, (name, nr, no)
    for k in range(nr):
        _cmp_genome(pr[k], po[k], "%s[%d]" % (name, k))
    for k in range(no):
        ours.flam3gpu_free_genome(C.byref(po[k]))
    LIBC.free(C.cast(po, C.c_void_p))


@pytest.mark.parametrize("name", sorted(BAD_DOCS))
def test_reader_rejects_what_the_reference_rejects(name):
    ref = _ref()
    ours = render.load()
    pr, nr = _parse(ref.flam3_parse_xml2, BAD_DOCS[name], 1)
    po, no = _parse(ours.flam3gpu_parse_xml2, BAD_DOCS[name], 1)
    assert no == 0 and not po
    assert nr == 0 or not pr, name


def test_reader_without_reference():
    """host-only checks that need no reference build"""
    gs = gm.parse_flam3(DOCS["basic"], "x/y.flam3")
    g = gs[0].g
    assert (g.width, g.height, g.spatial_oversample, g.num_xforms) == (320, 240, 2, 3)
    assert g.flame_name == b"two_words" and g.parent_fname == b"y.flam3"
    assert abs(g.palette[100].color[1] - 128 / 255.0) < 1e-12  # premultiplied by alpha 128/255
    assert g.xform[2].super_shape_rnd == 1.0  # clamped to [0, 1]
    assert g.xform[1].color_speed == pytest.approx(0.3)  # (1 - symmetry) / 2
    with pytest.raises(render.Flam3GpuError):
        gm.parse_flam3(UNCLOSED)
