"""GPU chaos game against the oracle: chains driven by the same Philox words
(same xform choices and random parameters) agree step by step in FP64 until
chaotic divergence amplifies the last-ulp libm differences; the bucket
accumulation of a given point stream matches the oracle's to FP64 rounding;
the xform-choice breakpoints reproduce the reference's 16384-entry table."""
import numpy as np
import pytest

from flam3_gb300 import genome as gm, render
import _oracle

pytestmark = pytest.mark.gpu


def test_chains_fp64_track_oracle(gpulib):
    G = gm.small_genome(3)
    rng = np.random.default_rng(1)
    starts = np.stack([rng.uniform(-1, 1, 256), rng.uniform(-1, 1, 256), rng.uniform(0, 1, 256),
                       rng.uniform(0, 1, 256)], 1)
    seed = 0x1234_5678_9ABC_DEF0
    go, bo = _oracle.oracle_iterate_chains(G, starts, 40, 0, seed)
    gg, bg = render.iterate_chains(G, starts, 40, 0, seed, precision=64)
    # the first 8 steps of every chain agree tightly
    err = np.abs(gg[:, :8] - go[:, :8]) / (1e-12 + np.abs(go[:, :8]))
    assert np.max(err) < 1e-9, np.max(err)
    # colour coordinates depend only on the xform sequence: identical choices
    np.testing.assert_allclose(gg[:, :, 2], go[:, :, 2], rtol=1e-12, atol=1e-12)
    assert bg == bo


def test_chains_with_final_xform_and_xaos(gpulib):
    rng = np.random.default_rng(5)
    G = gm.random_genome(rng, 4, final=True)
    for i in range(4):
        for j in range(4):
            G.set_chaos(i, j, float(rng.uniform(0.0, 2.0)))
    starts = np.stack([rng.uniform(-1, 1, 128), rng.uniform(-1, 1, 128), rng.uniform(0, 1, 128),
                       rng.uniform(0, 1, 128)], 1)
    go, bo = _oracle.oracle_iterate_chains(G, starts, 24, 3, 77)
    G2 = gm.random_genome(np.random.default_rng(5), 4, final=True)
    for i in range(4):
        for j in range(4):
            G2.set_chaos(i, j, G._chaos_rows[i][j])
    gg, bg = render.iterate_chains(G2, starts, 24, 3, 77, precision=64)
    np.testing.assert_allclose(gg[:, :, 2], go[:, :, 2], rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(gg[:, :4, :2], go[:, :4, :2], rtol=1e-7, atol=1e-9)


def test_xform_choice_equals_reference_table(gpulib):
    """Every 14-bit value of every choice row picks the xform the oracle's
    16384-entry table holds (flam3.c:76-111, 165-224), with and without
    xaos, final xforms, and weights that put breakpoints mid-bucket."""
    import ctypes as C

    lib = _oracle.oracle()
    rng = np.random.default_rng(11)
    for trial in range(12):
        n = int(rng.integers(1, 13))
        G = gm.random_genome(rng, n, final=bool(trial % 2))
        if trial % 3 == 0 and n > 1:
            for i in range(n):
                for j in range(n):
                    G.set_chaos(i, j, float(rng.choice([0.0, rng.uniform(0, 2)])))
                G.set_chaos(i, int(rng.integers(0, n)), 1.0)
        gpu = render.xform_choice_table(G)
        ref = lib.f3o_create_xform_distrib(C.byref(G.g))
        rows = gpu.shape[0]
        assert rows == 1 + (n if G.g.chaos_enable else 0)
        want = np.ctypeslib.as_array(ref, shape=(rows * 16384,)).reshape(rows, 16384)
        np.testing.assert_array_equal(gpu, want)


@pytest.mark.parametrize("palette_mode", [0, 1])
def test_accumulate_matches_oracle(gpulib, palette_mode):
    G = gm.small_genome(1)
    gm.resize(G, 64, 48)
    G.g.palette_mode = palette_mode
    G.g.rotate = 17.0 if palette_mode else 0.0
    F = gm.Frame(G)
    rng = np.random.default_rng(3)
    n = 200000
    pts = np.stack([rng.normal(G.g.center[0], 1.0, n), rng.normal(G.g.center[1], 1.0, n), rng.uniform(-0.1, 1.1, n),
                    rng.choice([1.0, 0.5, 0.0], n)], 1)
    ho = _oracle.oracle_accumulate(F, pts)
    hg = render.accumulate_points(F, pts)
    assert ho.shape == hg.shape
    # colours are staged as FP32 on the device: equal to FP32 rounding
    np.testing.assert_allclose(hg, ho, rtol=2e-6, atol=1e-3)
    assert ho[..., 4].sum() > 0


def test_accumulate_concentrated_points_match_oracle(gpulib):
    """Most points of a warp land in a handful of buckets: the warp-aggregated
    sums (shuffle reductions, one atomic per bucket) equal the oracle's
    one-by-one adds to FP32 rounding."""
    G = gm.small_genome(2)
    gm.resize(G, 32, 24)
    F = gm.Frame(G)
    rng = np.random.default_rng(5)
    n = 100000
    centers = rng.normal(0.0, 0.3, (5, 2)) + np.array([G.g.center[0], G.g.center[1]])
    pick = rng.integers(0, 5, n)
    pts = np.stack([centers[pick, 0] + rng.normal(0, 1e-4, n), centers[pick, 1] + rng.normal(0, 1e-4, n),
                    rng.uniform(0, 1, n), rng.choice([1.0, 0.5], n)], 1)
    ho = _oracle.oracle_accumulate(F, pts)
    hg = render.accumulate_points(F, pts)
    np.testing.assert_allclose(hg, ho, rtol=2e-6, atol=1e-3)
    assert (ho[..., 4] > 0).sum() <= 20



def _rc_chain_inputs(seed, nchains):
    """The start points and stream key flam3gpu_colorhist / _bounding_box
    draw from a caller's ISAAC context (flam3.c:2523-2525 for the starts)."""
    from flam3_gb300 import abi as _abi
    from flam3_gb300.isaac import init_rc, irand

    rc = _abi.randctx()
    init_rc(rc, seed)
    u = lambda: (((irand(rc) & 0xfffffff) - 0x7ffffff) / float(0x7ffffff))
    starts = np.array([[u(), u(), 0.0, 0.0] for _ in range(nchains)])
    key = irand(rc) & 0xffffffff
    key |= (irand(rc) & 0xffffffff) << 32
    return starts, key


def test_bounding_box_matches_oracle_chains(gpulib):
    from flam3_gb300 import abi as _abi
    from flam3_gb300.isaac import init_rc

    G = gm.still_genome(1, width=320, height=180, quality=10.0)
    nsamples, per = 200 * 1024, 1024
    rc = _abi.randctx()
    init_rc(rc, b"bb")
    bmin, bmax, bv = render.estimate_bounding_box(G, 0.01, nsamples, rc)
    starts, key = _rc_chain_inputs(b"bb", nsamples // per)
    pts = _oracle.oracle_iterate_chains(G, starts, per, 20, key)[0].reshape(-1, 4)
    lo = np.quantile(pts[:, :2], 0.01, axis=0)
    hi = np.quantile(pts[:, :2], 0.99, axis=0)
    span = hi - lo
    # FP32 chains decorrelate from the FP64 oracle's after tens of steps:
    # the same distribution, so the quantiles agree to sampling noise
    assert np.all(np.abs(bmin - lo) < 0.03 * span), (bmin, lo)
    assert np.all(np.abs(bmax - hi) < 0.03 * span), (bmax, hi)
    assert bv == 0


def test_colorhist_matches_oracle_chains(gpulib):
    from flam3_gb300 import abi as _abi
    from flam3_gb300.isaac import init_rc

    G = gm.still_genome(2, width=320, height=180, quality=10.0)
    rc = _abi.randctx()
    init_rc(rc, b"ch")
    h = render.colorhist(G, 20, rc)
    starts, key = _rc_chain_inputs(b"ch", 20)
    pts = _oracle.oracle_iterate_chains(G, starts, 10000, 20, key)[0].reshape(-1, 4)
    ho = np.bincount(np.clip((pts[:, 2] * 256).astype(int), 0, 255), minlength=256) / len(pts)
    assert abs(h.sum() - 1.0) < 1e-6
    assert np.abs(h - ho).sum() < 0.08, np.abs(h - ho).sum()


def _sierpinski(width=512, height=512):
    """three linear xforms of scale 1/2: the gasket on [0,1]^2, correlation
    dimension log 3 / log 2"""
    from flam3_gb300 import abi
    G = gm.Genome(3)
    for i, (tx, ty) in enumerate(((0.0, 0.0), (0.5, 0.0), (0.25, 0.5))):
        x = G.xform(i)
        x.c[0][0], x.c[0][1], x.c[1][0], x.c[1][1], x.c[2][0], x.c[2][1] = 0.5, 0.0, 0.0, 0.5, tx, ty
        x.density = 1.0 / 3
        x.color = i / 2.0
        for j in range(abi.NVARS):
            x.var[j] = 0.0
        x.var[0] = 1.0
    gm.resize(G, width, height)
    G.g.center[0], G.g.center[1] = 0.5, 0.5
    G.g.pixels_per_unit = width / 1.25  # the camera covers the gasket with a margin
    G.g.zoom = 0.0
    return G


def _oracle_dimension(G, ntries, seed):
    """flam3.c:3949-4052 restated on oracle chains (camera clip, no points
    outside it for this genome)"""
    rng = np.random.default_rng(seed)
    nchains = (ntries + 9999) // 10000
    starts = np.stack([rng.uniform(-1, 1, nchains), rng.uniform(-1, 1, nchains), np.zeros(nchains),
                       np.zeros(nchains)], 1)
    pts = _oracle.oracle_iterate_chains(G, starts, 10000, 20, int(rng.integers(1 << 62)))[0].reshape(-1, 4)
    pts = pts[:ntries, :2]
    span = G.g.width / G.g.pixels_per_unit, G.g.height / G.g.pixels_per_unit
    d2max = span[0] ** 2 + span[1] ** 2
    k = rng.integers(0, ntries, ntries)
    d2 = np.sum((pts[k] - pts) ** 2, axis=1)
    n2, n1 = np.sum(d2 < 0.004 * d2max), np.sum(d2 < 0.00004 * d2max)
    return 0.434294 * np.log(n2 / (n1 - 0.5))


def test_dimension_matches_oracle_and_theory(gpulib):
    G = _sierpinski()
    d = render.dimension(G, ntries=400000, clip_to_camera=True)
    do = _oracle_dimension(G, 400000, 7)
    assert abs(d - do) < 0.08, (d, do)
    assert abs(d - np.log(3) / np.log(2)) < 0.15, d
    # without the camera: the box comes from flam3_estimate_bounding_box
    d2 = render.dimension(G, ntries=400000, clip_to_camera=False)
    assert abs(d2 - np.log(3) / np.log(2)) < 0.2, d2


def _oracle_lyapunov(G, ntries, seed):
    """flam3.c:4054-4150 restated on oracle chains in FP64"""
    rng = np.random.default_rng(seed)
    st = np.stack([rng.uniform(-1, 1, ntries), rng.uniform(-1, 1, ntries), np.zeros(ntries), np.zeros(ntries)], 1)
    on = _oracle.oracle_iterate_chains(G, st, 1, 25, int(rng.integers(1 << 62)))[0][:, 0]
    s1 = _oracle.oracle_iterate_chains(G, on, 1, 0, int(rng.integers(1 << 62)))[0][:, 0]
    ang = rng.uniform(0, 2 * np.pi, ntries)
    pert = on.copy()
    pert[:, 0] += 1e-5 * np.cos(ang)
    pert[:, 1] += 1e-5 * np.sin(ang)
    pert[:, 2] = 0.0
    s2 = _oracle.oracle_iterate_chains(G, pert, 1, 0, int(rng.integers(1 << 62)))[0][:, 0]
    r = np.hypot(s1[:, 0] - s2[:, 0], s1[:, 1] - s2[:, 1])
    return np.sum(np.log(r / 1e-5)) / (np.log(2.0) * ntries)


def test_lyapunov_matches_oracle(gpulib):
    G = _sierpinski()
    v = render.lyapunov(G, ntries=20000)
    vo = _oracle_lyapunov(G, 20000, 3)
    # the two steps draw independent xforms (as in the reference): 2/3 of the
    # tries land a translation apart, 1/3 contract by 1/2
    expect = ((2 / 3) * np.mean(np.log(np.array([0.5, 0.5590169943749475, 0.5590169943749475]) / 1e-5)) +
              (1 / 3) * np.log(0.5))
    assert abs(v - vo) < 0.3, (v, vo)
    assert abs(v - expect / np.log(2.0)) < 0.5, (v, expect / np.log(2.0))


def test_atomic_rate_probe(gpulib):
    """the roofline probe runs and reports a plausible L2 float4-atomic rate"""
    r = render.measure_atomic_rate(1 << 20, 1 << 26)
    assert 1e9 < r < 1e13, r
