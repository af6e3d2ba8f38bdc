"""Whole renders through flam3gpu_render (the drop-in) against the oracle.

The GPU draws its random numbers from a counter-based stream instead of
ISAAC, so images are compared statistically: per-channel mean absolute error
against an oracle render at 16x the quality, which must fall as
1/sqrt(quality); the warp-coherent mode is checked against the per-thread
mode the same way.  Also: stats and the caller's ISAAC context advance as in
the reference, error returns, progress-callback abort."""
import ctypes as C

import numpy as np
import pytest

from flam3_gb300 import abi, genome as gm, render
import _oracle

pytestmark = pytest.mark.gpu


def cfg0(seed=0, w=256, h=192, q=50.0, bits=33, est=0.0):
    G = gm.small_genome(seed)
    gm.resize(G, w, h)
    G.g.sample_density = q
    G.g.estimator = est
    return G


def mae(a, b):
    return float(np.mean(np.abs(a.astype(np.float64) - b.astype(np.float64))))


@pytest.fixture(scope="module")
def hq_reference():
    """Oracle render at 16x quality (and 8 worker threads)."""
    G = cfg0(q=50.0 * 16)
    F = gm.Frame(G, bits=64, nthreads=8, seed="hq")
    out, st, _ = _oracle.oracle_render(F)
    return out


@pytest.mark.parametrize("mode", [0, 1])
def test_render_matches_hq_reference_and_converges(gpulib, hq_reference, mode):
    render.set_options(iter_mode=mode)
    try:
        errs = []
        for q in (12.5, 50.0, 200.0):
            F = gm.Frame(cfg0(q=q), bits=33, seed="gpu-%g" % q)
            out, st = render.render(F)
            errs.append(mae(out, hq_reference))
        # error falls roughly as 1/sqrt(quality): 4x quality -> about half
        assert errs[1] < 0.8 * errs[0] and errs[2] < 0.8 * errs[1], errs
        assert errs[2] < 2.0, errs
    finally:
        render.reset_options()


def test_gpu_error_comparable_to_oracle_error(gpulib, hq_reference):
    F = gm.Frame(cfg0(q=50.0), bits=33, seed="o")
    o, _, _ = _oracle.oracle_render(F)
    F = gm.Frame(cfg0(q=50.0), bits=33, seed="g")
    g, _ = render.render(F)
    e_o, e_g = mae(o, hq_reference), mae(g, hq_reference)
    assert e_g < 1.5 * e_o + 0.1, (e_g, e_o)


def test_stats_and_isaac_consumption_match_reference(gpulib):
    Fo = gm.Frame(cfg0(q=20.0), bits=33, nthreads=3, seed="rc")
    _, so, _ = _oracle.oracle_render(Fo)
    Fg = gm.Frame(cfg0(q=20.0), bits=33, nthreads=3, seed="rc")
    _, sg = render.render(Fg)
    assert sg.num_iters == so.num_iters
    assert [Fg.f.rc.randrsl[i] for i in range(16)] == [Fo.f.rc.randrsl[i] for i in range(16)]
    assert Fg.f.rc.randcnt == Fo.f.rc.randcnt


def test_bad_bits_and_bad_oversample_return_1(gpulib):
    F = gm.Frame(cfg0(q=5.0), bits=48)
    out = F.out_buffer(3)
    st = abi.stat_struct()
    assert gpulib.flam3gpu_render(C.byref(F.f), out.ctypes.data, 0, 3, 0, C.byref(st)) == 1
    G = cfg0(q=5.0)
    G.g.spatial_oversample = 0
    F = gm.Frame(G, bits=33)
    assert gpulib.flam3gpu_render(C.byref(F.f), out.ctypes.data, 0, 3, 0, C.byref(st)) == 1
    G = cfg0(q=5.0)
    G.xform(0).density = -1.0
    F = gm.Frame(G, bits=33)
    assert gpulib.flam3gpu_render(C.byref(F.f), out.ctypes.data, 0, 3, 0, C.byref(st)) == 1


def test_progress_abort_returns_0(gpulib):
    calls = []

    @abi.PROGRESS_FN
    def prog(param, pct, stage, eta):
        calls.append(pct)
        return 1

    F = gm.Frame(cfg0(q=20.0), bits=33)
    F.f.progress = prog
    out = F.out_buffer(3)
    st = abi.stat_struct()
    assert gpulib.flam3gpu_render(C.byref(F.f), out.ctypes.data, 0, 3, 0, C.byref(st)) == 0
    assert len(calls) == 1


def test_de_render_close_to_oracle(gpulib):
    Fo = gm.Frame(cfg0(q=400.0, est=4.0, w=160, h=120), bits=33, nthreads=8, seed="de")
    o, _, _ = _oracle.oracle_render(Fo)
    Fg = gm.Frame(cfg0(q=400.0, est=4.0, w=160, h=120), bits=33, seed="de-g")
    g, _ = render.render(Fg)
    assert mae(o, g) < 2.5


def test_bits64_render_close_to_bits33(gpulib):
    a, _ = render.render(gm.Frame(cfg0(q=100.0), bits=33, seed="x"))
    b, _ = render.render(gm.Frame(cfg0(q=100.0), bits=64, seed="x"))
    assert mae(a, b) < 0.5


def anim_frame(t, nts, est, q=400.0, bits=33, nthreads=8, rc_seed="anim", w=160, h=120):
    gs = gm.animation_keys(2, width=w, height=h, quality=q, temporal_samples=nts, estimator=est)
    return gm.Frame(gs, bits=bits, nthreads=nthreads, seed=rc_seed, time=t)


@pytest.mark.parametrize("t,nts,est,bits", [(40.0, 8, 3.0, 33), (119.8, 4, 0.0, 64), (0.0, 3, 0.0, 33)])
def test_animation_render_close_to_oracle(gpulib, t, nts, est, bits):
    """Two key genomes, a frame between them with temporal samples (motion
    blur): every temporal sample interpolates its own genome."""
    Fo = anim_frame(t, nts, est, bits=bits)
    o, so, _ = _oracle.oracle_render(Fo)
    Fg = anim_frame(t, nts, est, bits=bits, rc_seed="anim-g")
    g, sg = render.render(Fg)
    assert sg.num_iters == so.num_iters
    assert mae(o, g) < 2.5, mae(o, g)


def test_calc_nstrips_against_budget(gpulib):
    F = gm.Frame(gm.small_genome(3), bits=33, seed="ns")
    need = render.memory_required(F)
    assert render.calc_nstrips(F, need * 10) == 1
    assert render.calc_nstrips(F, need / 2.5) == 3
    assert render.calc_nstrips(F) == 1  # a 512x512 still fits 80 % of free HBM


def test_render_strips_matches_full_render(gpulib):
    """flam3-render's strip loop: one strip is the plain render; three strips
    (the last one shorter) carry the same image up to sampling noise, and the
    caller's genome is unchanged."""
    G = gm.small_genome(4, width=200, height=250, quality=200.0)
    F = gm.Frame(G, bits=33, seed="strips")
    full, st_full = render.render(F)
    F1 = gm.Frame(G, bits=33, seed="strips")
    one, st_one = render.render_strips(F1, 1)
    assert mae(full, one) < 0.02 and st_one.num_iters == st_full.num_iters
    dens, cy, h = G.g.sample_density, G.g.center[1], G.g.height
    F3 = gm.Frame(G, bits=33, seed="strips")
    three, st3 = render.render_strips(F3, 3)
    assert (G.g.sample_density, G.g.center[1], G.g.height) == (dens, cy, h)
    # each strip iterates sample_density * 3 over a third of the rows: the
    # full frame's samples per strip, three times in all (as flam3-render)
    assert abs(st3.num_iters - 3 * st_full.num_iters) < 0.02 * 3 * st_full.num_iters
    other, _ = render.render(gm.Frame(G, bits=33, seed="strips-other"))
    noise = mae(full, other)
    # flam3-render lays the strips out for 3 * 84 = 252 rows around the centre,
    # which moves the 250-row image down by one row
    assert mae(full[:-1], three[1:]) < 1.5 * noise + 0.05, (mae(full[:-1], three[1:]), noise)
    # every strip is populated (no empty band at a seam)
    for r0 in (0, 84, 168):
        assert three[r0 + 1:r0 + 82].mean() > 0.5 * full[r0:r0 + 81].mean()
    with pytest.raises(render.Flam3GpuError):
        render.render_strips(gm.Frame(G, bits=33, seed="x"), 251)


FLAME_XML = """<flames><flame name="xml test" size="160 120" center="0 0" scale="40" quality="400"
  oversample="1" filter="0.5" estimator_radius="4" brightness="4" gamma="4">
  <xform weight="0.4" color="0" linear="0.6" spherical="0.4" coefs="0.5 0.3 -0.3 0.5 0.4 0.1"/>
  <xform weight="0.3" color="0.5" sinusoidal="1" coefs="0.6 0 0 0.6 -0.4 0.2"/>
  <xform weight="0.3" color="1" julia="0.7" swirl="0.3" coefs="0.4 -0.2 0.2 0.4 0 -0.5"/>
  <finalxform color="0.5" color_speed="0" linear="0.8" polar="0.2" coefs="1 0 0 1 0 0"/>
  <color index="0" rgb="255 40 0"/><color index="128" rgb="40 255 80"/><color index="255" rgb="20 60 255"/>
</flame></flames>"""


def test_render_of_parsed_genome_close_to_oracle(gpulib):
    """a genome read from flam3's XML format renders on the GPU like the
    oracle renders the same genome"""
    G = gm.parse_flam3(FLAME_XML, "test.flam3")[0]
    o, _, _ = _oracle.oracle_render(gm.Frame(G, bits=33, nthreads=8, seed="xml"))
    g, _ = render.render(gm.Frame(G, bits=33, seed="xml-g"))
    assert o.mean() > 5.0
    assert mae(o, g) < 2.5


@pytest.mark.parametrize("threads", [32, 64, 128])
@pytest.mark.parametrize("mode", [0, 1])
def test_block_sizes_render_like_the_default(gpulib, hq_reference, threads, mode):
    """Blocks of 32, 64 or 128 threads (the point exchange between warps, its
    buffers and barrier counts all depend on the block): the same samples
    counted, the same error against the 16x render as 256-thread blocks."""
    errs, iters = {}, {}
    for t in (256, threads):
        render.set_options(iter_mode=mode, threads_per_block=t)
        try:
            F = gm.Frame(cfg0(q=200.0), bits=33, seed="blk-%d" % t)
            out, st = render.render(F)
        finally:
            render.reset_options()
        errs[t] = mae(out, hq_reference)
        iters[t] = st.num_iters
    assert iters[threads] == iters[256]
    assert errs[threads] <= 1.05 * errs[256] + 0.03, errs


def test_exchange_wait_runs_out_and_the_context_stays_usable(gpulib):
    """Failure detection of the iterate kernel's point exchange, without a GPU
    fault: with the test option one block withholds an mbarrier arrival, its
    warps' bounded waits run out after 2 s, the kernel sets its error flag
    and the render fails with that error; the next render on the same context
    succeeds."""
    render.set_options(test_exchange_stall=1)
    try:
        with pytest.raises(render.Flam3GpuError, match="exchange wait timed out"):
            render.render(gm.Frame(cfg0(q=50.0), bits=33, seed="stall"))
    finally:
        render.reset_options()
    out, st = render.render(gm.Frame(cfg0(q=50.0), bits=33, seed="after-stall"))
    assert out.mean() > 1.0 and st.num_iters > 0
