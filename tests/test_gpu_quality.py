"""Whole renders of the workloads' requests against 16x-quality reference
renders, and the statistical checks of the GPU's sampling choices.

Matched image error (tests/golden/quality_refs.npz, made by
tests/golden/make_quality_refs.py): for each request window -- the config-1
still, draws of the mixed-size batch including bits 64, supersample 2, no DE
and DE radius 11, and the serving trace's 3840x2160 DE-11 still -- the
fixture holds the oracle's FP64-bucket render at 16x the request's quality
and the oracle's own error at q/16, q/4 and q.  The GPU renders the window
through the drop-in at those qualities with the request's bits.  Error is
the per-channel mean absolute difference from the 16x render in 8-bit
levels.  Bars:
  * at every quality the GPU's error is at most the oracle's error at the
    same quality and bits plus the 0.5/255 budget (0.5 levels), and at most
    10% (+0.05 levels) above it;
  * the error falls with quality like the reference's: the GPU's ratio per 4x
    of quality is at most the oracle's + 0.05.  The reference's own ratio is
    0.53-0.81 in these windows, slower than the 0.5 of 1/sqrt(q): density
    estimation kernels narrow only as density^-0.4 (filters.c:272-407), so the
    low-quality blur is a bias that shrinks slowly, and the tonemap is
    nonlinear.
At the requests' own qualities the reference's arithmetic is at 1.5-12
levels from its 16x render, so neither it nor the GPU is within 0.5/255
there; the bench's error leg reports the quality each would need.

Sampling: the warp-coherent xform choice (mode 1, one draw per warp per
step) picks each xform with the genome's probabilities, as the per-thread
choice (mode 0) does: a genome whose xforms map the plane into disjoint
discs counts every choice in the real iterate kernel's histogram, and a
chi-square test with the warp's 32-fold correlation holds both modes to the
weights.  The two modes' images sit at the same error against the 16x
render.

bits=32 (u32 buckets and accumulator in the reference, density estimation
off, flam3.c:3642-3647, 3771-3790) renders like the oracle's bits=32; the
strip loop of flam3-render (flam3-render.c:311-345) on the GPU matches the
same loop over the oracle."""
import math

import numpy as np
import pytest

from flam3_gb300 import abi, genome as gm, render
import _oracle
from golden import make_quality_refs as qr

pytestmark = pytest.mark.gpu

REFS = qr.load()


def mae(a, b):
    return qr.mae(a, b)


@pytest.mark.parametrize("name", sorted(REFS))
def test_request_error_matches_reference_arithmetic(gpulib, name):
    m = REFS[name]
    ref = m["ref"]
    errs = {}
    for div in (16, 4, 1):
        G, bits = qr.build(name, m, quality=m["q"] / div)
        out, st = render.render(gm.Frame(G, bits=bits, seed="quality-%s-%d" % (name, div)))
        errs[div] = mae(out, ref)
        o = m["oracle_mae"]["b%d_q/%d" % (bits, div)][0]
        assert errs[div] <= min(1.10 * o + 0.05, o + 0.5), (name, div, errs[div], o)
    bits = m["bits"]
    o16, o4, o1 = (m["oracle_mae"]["b%d_q/%d" % (bits, d)][0] for d in (16, 4, 1))
    assert errs[4] / errs[16] <= o4 / o16 + 0.05, (name, errs, (o16, o4, o1))
    assert errs[1] / errs[4] <= o1 / o4 + 0.05, (name, errs, (o16, o4, o1))
    assert errs[1] / errs[16] < 0.6, (name, errs)


def disc_genome(weights, scale=0.2, radius=1.0, size=256, quality=200.0):
    """xform i: p -> scale*p + radius*(cos, sin)(2 pi i / n), linear only: the
    attractor lies in n disjoint discs, the point plotted after xform i in
    disc i, so the histogram's hit count per disc counts the choices of i."""
    n = len(weights)
    G = gm.Genome(n)
    for i, w in enumerate(weights):
        x = G.xform(i)
        a = 2.0 * math.pi * i / n
        x.c[0][0] = scale
        x.c[1][1] = scale
        x.c[0][1] = x.c[1][0] = 0.0
        x.c[2][0] = radius * math.cos(a)
        x.c[2][1] = radius * math.sin(a)
        x.density = float(w)
        x.color = i / max(n - 1, 1)
    G.set_palette(np.ones((256, 3)))
    g = G.g
    g.width = g.height = size
    g.center[0] = g.center[1] = 0.0
    g.pixels_per_unit = size / (2.0 * (radius + 0.5))
    g.sample_density = quality
    g.estimator = 0.0
    g.spatial_oversample = 1
    return G


def disc_counts(hist, G, n, radius=1.0):
    h, w = hist.shape[:2]
    g = G.g
    ys, xs = np.mgrid[0:h, 0:w]
    # bucket centres in world units (the histogram includes the gutter)
    gut_x = (w - g.width) / 2.0
    gut_y = (h - g.height) / 2.0
    wx = (xs + 0.5 - gut_x - g.width / 2.0) / g.pixels_per_unit + g.center[0]
    wy = (ys + 0.5 - gut_y - g.height / 2.0) / g.pixels_per_unit + g.center[1]
    ang = 2.0 * math.pi * np.arange(n) / n
    d2 = (wx[..., None] - radius * np.cos(ang)) ** 2 + (wy[..., None] - radius * np.sin(ang)) ** 2
    which = np.argmin(d2, axis=2)
    hits = hist[..., 4] / 255.0
    assert np.all(np.min(d2, axis=2)[hits > 0] < 0.3 ** 2)  # every hit inside a disc
    return np.bincount(which.ravel(), weights=hits.ravel(), minlength=n)


@pytest.mark.parametrize("mode", [0, 1])
def test_xform_choice_frequencies_chi_square(gpulib, mode):
    weights = np.array([0.05, 0.3, 0.1, 0.2, 0.02, 0.18, 0.15])
    p = weights / weights.sum()
    n = len(p)
    render.set_options(iter_mode=mode)
    try:
        G = disc_genome(weights)
        # FP64 buckets count every hit exactly (an FP32 count channel rounds
        # once a bucket passes 2^24)
        _, st, ex = render.render(gm.Frame(G, bits=64, seed="discs-%d" % mode), want_hist=True)
    finally:
        render.reset_options()
    counts = disc_counts(ex["hist"], G, n)
    N = counts.sum()
    assert abs(N - st.num_iters) < 1e-6 * N
    # mode 1: the 32 lanes of a warp share each step's draw, so the count of
    # an xform varies 32x more than with independent draws
    corr = 32.0 if mode == 1 else 1.0
    chi2 = float(np.sum((counts - N * p) ** 2 / (N * p)) / corr)
    # chi-square, 6 degrees of freedom: P(chi2 > 22.46) = 0.001
    assert chi2 < 22.46, (mode, chi2, counts / N, p)
    np.testing.assert_allclose(counts / N, p, atol=5 * np.sqrt(corr * p * (1 - p) / N).max())


def test_warp_coherent_choice_image_error_equals_per_thread(gpulib):
    name = "still_crop"
    m = REFS[name]
    errs = {}
    for mode in (0, 1):
        render.set_options(iter_mode=mode)
        try:
            e = []
            for s in range(2):
                G, bits = qr.build(name, m)
                out, _ = render.render(gm.Frame(G, bits=bits, seed="mode-%d-%d" % (mode, s)))
                e.append(mae(out, m["ref"]))
            errs[mode] = float(np.mean(e))
        finally:
            render.reset_options()
    assert errs[1] <= 1.03 * errs[0] + 0.02, errs
    assert errs[0] <= 1.03 * errs[1] + 0.02, errs


def test_bits32_matches_oracle_bits32(gpulib):
    """bits 32: DE requested by the genome is switched off, as the reference
    does; the GPU image sits at the oracle's error against the oracle's
    16x bits-32 render."""
    def mk(q):
        G = gm.small_genome(2, width=200, height=150, quality=q)
        G.g.estimator = 4.0
        return G

    q = 100.0
    ref, _, _ = _oracle.oracle_render(gm.Frame(mk(16 * q), bits=32, nthreads=8, seed="b32-ref"), fast=True)
    o, so, _ = _oracle.oracle_render(gm.Frame(mk(q), bits=32, nthreads=8, seed="b32-o"), fast=True)
    g, sg = render.render(gm.Frame(mk(q), bits=32, seed="b32-g"))
    assert sg.num_iters == so.num_iters
    e_o, e_g = mae(o, ref), mae(g, ref)
    assert e_g <= min(1.1 * e_o + 0.05, e_o + 0.5), (e_g, e_o)
    # the reference's integer accumulator drops log-scaled values below one
    # unit (the dim parts of the image); exact FP32 sums keep them and so sit
    # far from the reference's picture
    render.set_options(float_buckets=1)
    try:
        gf, _ = render.render(gm.Frame(mk(q), bits=32, seed="b32-g"))
    finally:
        render.reset_options()
    assert mae(gf, ref) > e_g + 0.5, (mae(gf, ref), e_g)
    assert ref.mean() > 5.0


def oracle_render_strips(F, nstrips):
    """flam3-render's strip loop (flam3-render.c:311-345) over the oracle:
    sample density times nstrips, strip height ceil(H/nstrips), centres from
    center_base, a shorter last strip re-centred, the same ISAAC context for
    every strip, one temporal sample."""
    g = F.genomes[0].g
    W, H = g.width, g.height
    saved = (g.sample_density, g.height, g.center[1], g.ntemporal_samples)
    sh = int(math.ceil(H / float(nstrips)))
    zs = 2.0 ** g.zoom
    base = g.center[1] - ((nstrips - 1) * sh) / (2 * g.pixels_per_unit * zs)
    rc = abi.randctx()
    C_memmove(rc, F.f.rc)
    out = np.zeros((H, W, 3), np.uint8)
    iters = 0.0
    g.sample_density = saved[0] * nstrips
    for s in range(nstrips):
        g.height = sh
        g.center[1] = base + sh * float(s) / (g.pixels_per_unit * zs)
        if sh * (s + 1) > H:
            g.height = H - sh * s
            g.center[1] -= (sh - g.height) * 0.5 / (g.pixels_per_unit * zs)
        g.ntemporal_samples = 1
        F.sync()
        C_memmove(F.f.rc, rc)
        img, st, _ = _oracle.oracle_render(F, fast=True)
        out.reshape(-1)[sh * s * W * 3: sh * s * W * 3 + img.size] = img.reshape(-1)
        iters += st.num_iters
    g.sample_density, g.height, g.center[1], g.ntemporal_samples = saved
    F.sync()
    return out, iters


def C_memmove(dst, src):
    import ctypes

    ctypes.memmove(ctypes.addressof(dst), ctypes.addressof(src), ctypes.sizeof(src))


def test_render_strips_match_oracle_strip_loop(gpulib):
    def mk(q):
        return gm.small_genome(4, width=200, height=250, quality=q)

    q = 200.0
    ref, _ = oracle_render_strips(gm.Frame(mk(16 * q), bits=33, nthreads=8, seed="strips-ref"), 3)
    o, it_o = oracle_render_strips(gm.Frame(mk(q), bits=33, nthreads=8, seed="strips-o"), 3)
    g, st = render.render_strips(gm.Frame(mk(q), bits=33, nthreads=8, seed="strips-g"), 3)
    assert st.num_iters == it_o
    e_o, e_g = mae(o, ref), mae(g, ref)
    assert e_g <= min(1.1 * e_o + 0.05, e_o + 0.5), (e_g, e_o)
    # strip by strip (the last one is shorter): no band is off
    for r0, r1 in ((0, 84), (84, 168), (168, 250)):
        eo, eg = mae(o[r0:r1], ref[r0:r1]), mae(g[r0:r1], ref[r0:r1])
        assert eg <= min(1.15 * eo + 0.1, eo + 0.5), (r0, eg, eo)
    assert ref.mean() > 2.0
