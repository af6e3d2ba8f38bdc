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
    G = gm.config0_genome(3)
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


@pytest.mark.parametrize("palette_mode", [0, 1])
def test_accumulate_matches_oracle(gpulib, palette_mode):
    G = gm.config0_genome(1)
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
    G = gm.config0_genome(2)
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

    G = gm.config1_genome(1, width=320, height=180, quality=10.0)
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

    G = gm.config1_genome(2, width=320, height=180, quality=10.0)
    rc = _abi.randctx()
    init_rc(rc, b"ch")
    h = render.colorhist(G, 20, rc)
    starts, key = _rc_chain_inputs(b"ch", 20)
    pts = _oracle.oracle_iterate_chains(G, starts, 10000, 20, key)[0].reshape(-1, 4)
    ho = np.bincount(np.clip((pts[:, 2] * 256).astype(int), 0, 255), minlength=256) / len(pts)
    assert abs(h.sum() - 1.0) < 1e-6
    assert np.abs(h - ho).sum() < 0.08, np.abs(h - ho).sum()
