"""The batched / served path (include/flam3_gpu_service.h) against the plain
drop-in.

A job's chunking and random streams are fixed when it is planned, so a
served or batched render equals flam3gpu_render of the same frame up to the
order of floating-point atomic additions into the histogram.  The stated
tolerance: at least 99.9% of channel values within one 8-bit level and none
more than 8 levels apart; sample counts, bad-value counts and the caller's
ISAAC context identical."""
import threading

import numpy as np
import pytest

from flam3_gb300 import abi, genome as gm, render, service

pytestmark = pytest.mark.gpu


def close_images(a, b, frac=0.999, worst=8):
    d = np.abs(a.astype(np.int64) - b.astype(np.int64))
    scale = 256 if a.dtype == np.uint16 else 1
    return float(np.mean(d <= scale)) >= frac and int(d.max()) <= worst * scale, (float(np.mean(d <= scale)),
                                                                                 int(d.max()))


def frame(kind, seed=0):
    """Small frames covering the tail shapes: fused log, fused DE, several
    batches, temporal samples, FP64 buckets, fields, earlyclip, RGBA16."""
    if kind == "plain":
        G = gm.small_genome(seed)
        gm.resize(G, 200, 150)
        G.g.sample_density = 40.0
        return gm.Frame(G, bits=33, seed="svc-%s-%d" % (kind, seed))
    if kind == "de":
        G = gm.small_genome(seed)
        gm.resize(G, 160, 120)
        G.g.sample_density = 60.0
        G.g.estimator = 4.0
        return gm.Frame(G, bits=33, seed="svc-%s-%d" % (kind, seed))
    if kind == "b64_ss2_de":
        G = gm.still_genome(seed + 5, width=128, height=96, quality=30.0, oversample=2, estimator=5.0)
        return gm.Frame(G, bits=64, seed="svc-%s-%d" % (kind, seed))
    if kind == "batches":
        G = gm.small_genome(seed)
        gm.resize(G, 120, 90)
        G.g.sample_density = 40.0
        G.g.nbatches = 3
        G.g.ntemporal_samples = 2
        G.g.estimator = 3.0
        return gm.Frame(G, bits=33, seed="svc-%s-%d" % (kind, seed))
    if kind == "anim":
        gs = gm.animation_keys(seed + 2, width=144, height=96, quality=40.0, temporal_samples=6, estimator=3.0)
        return gm.Frame(gs, bits=33, seed="svc-%s-%d" % (kind, seed), time=30.0 + seed)
    if kind == "early":
        G = gm.small_genome(seed)
        gm.resize(G, 100, 80)
        G.g.sample_density = 30.0
        return gm.Frame(G, bits=64, seed="svc-%s-%d" % (kind, seed), earlyclip=1)
    if kind == "rgba16":
        G = gm.small_genome(seed)
        gm.resize(G, 96, 64)
        G.g.sample_density = 30.0
        return gm.Frame(G, bits=33, seed="svc-%s-%d" % (kind, seed), bytes_per_channel=2)
    raise ValueError(kind)


KINDS = ["plain", "de", "b64_ss2_de", "batches", "anim", "early", "rgba16"]
NCHAN = {"rgba16": 4}


def plain(kind, seed=0, field=0):
    F = frame(kind, seed)
    nchan = NCHAN.get(kind, 3)
    out, st = render.render(F, field=field, nchan=nchan)
    return out, st, F


@pytest.mark.parametrize("kind", KINDS)
def test_served_equals_plain(gpulib, kind):
    ref, st_ref, F_ref = plain(kind)
    F = frame(kind)
    with service.Service() as svc:
        t = svc.submit(F, nchan=NCHAN.get(kind, 3))
        out, st, times = svc.wait(t)
        cnt = svc.counters()
    ok, info = close_images(out, ref)
    assert ok, info
    assert st.num_iters == st_ref.num_iters
    assert st.badvals == st_ref.badvals
    assert [F.f.rc.randrsl[i] for i in range(16)] == [F_ref.f.rc.randrsl[i] for i in range(16)]
    assert cnt["jobs_done"] == 1 and cnt["rounds"] >= 1 and times[2] > 0


def test_field_render_served(gpulib):
    ref, _, _ = plain("plain", field=2)
    F = frame("plain")
    with service.Service() as svc:
        out, _, _ = svc.wait(svc.submit(F, field=2))
    ok, info = close_images(out, ref)
    assert ok, info


def test_alone_equals_in_mix(gpulib):
    """The same request alone and among 24 others of other sizes, through
    rounds small enough that every job is split over several launches."""
    target = ("de", 3)
    with service.Service(round_samples=1 << 20) as svc:
        alone, st_a, _ = svc.wait(svc.submit(frame(*target)))
    mix = [(k, s) for s in range(4) for k in ("plain", "de", "anim", "batches", "b64_ss2_de", "early")]
    with service.Service(round_samples=1 << 20) as svc:
        tickets = []
        for i, (k, s) in enumerate(mix):
            if i == 7:
                tickets.append(("target", svc.submit(frame(*target))))
            tickets.append(((k, s), svc.submit(frame(k, s), nchan=NCHAN.get(k, 3))))
        res = {}
        for key, t in tickets:
            res[key] = svc.wait(t)
        cnt = svc.counters()
    out, st, times = res["target"]
    ok, info = close_images(out, alone)
    assert ok, info
    assert st.num_iters == st_a.num_iters and st.badvals == st_a.badvals
    assert times[3] >= 2  # split over several rounds
    assert cnt["jobs_done"] == len(mix) + 1 and cnt["jobs_failed"] == 0


def test_render_batch_equals_plain(gpulib):
    kinds = [("plain", 1), ("anim", 0), ("anim", 1), ("de", 2), ("b64_ss2_de", 1)]
    frames = [frame(k, s) for k, s in kinds]
    res = service.render_batch(frames)
    for (k, s), (out, st) in zip(kinds, res):
        ref, st_ref, _ = plain(k, s)
        ok, info = close_images(out, ref)
        assert ok, (k, s, info)
        assert st.num_iters == st_ref.num_iters


def test_tail_graphs_and_direct_tails_agree(gpulib):
    outs = []
    for graphs, branches in ((1, 1), (2, 3), (0, 1)):
        with service.Service(tail_graphs=graphs, tail_branches=branches) as svc:
            ts = [svc.submit(frame(k, 0), nchan=NCHAN.get(k, 3)) for k in KINDS + KINDS]
            outs.append([svc.wait(t)[0] for t in ts])
            cnt = svc.counters()
        if graphs:
            assert cnt["tail_graphs"] >= 1
        else:
            assert cnt["tail_graphs"] == 0
        if graphs == 1:
            # one executable graph per tail shape, reused for the repeats
            assert cnt["graphs_instantiated"] < len(KINDS) * 2
    for other in outs[1:]:
        for a, b in zip(outs[0], other):
            ok, info = close_images(a, b)
            assert ok, info


def test_admission_by_budget(gpulib):
    """A budget that holds about two jobs: the rest queue and run later."""
    F0 = frame("de", 0)
    with service.Service() as probe:
        probe.wait(probe.submit(F0))
        need = probe.counters()["peak_device_bytes"]
    with service.Service(hbm_budget_bytes=2.5 * need) as svc:
        ts = [svc.submit(frame("de", s)) for s in range(8)]
        for t in ts:
            svc.wait(t)
        cnt = svc.counters()
    assert cnt["jobs_done"] == 8
    assert cnt["peak_device_bytes"] <= 2.5 * need


def test_oversize_job_fails_cleanly(gpulib):
    with service.Service(hbm_budget_bytes=1e5) as svc:
        t = svc.submit(frame("plain"))
        with pytest.raises(render.Flam3GpuError, match="service budget"):
            svc.wait(t)
        assert svc.counters()["jobs_failed"] == 1


def test_concurrent_submitters(gpulib):
    results = {}
    with service.Service() as svc:
        def worker(k):
            for s in range(3):
                t = svc.submit(frame(k, s), nchan=NCHAN.get(k, 3))
                results[(k, s)] = svc.wait(t)[0]

        th = [threading.Thread(target=worker, args=(k,)) for k in ("plain", "de", "anim", "rgba16")]
        for x in th:
            x.start()
        for x in th:
            x.join()
    assert len(results) == 12
    ref, _, _ = plain("anim", 1)
    ok, info = close_images(results[("anim", 1)], ref)
    assert ok, info


def test_autotune_table_roundtrip(gpulib, tmp_path):
    frames = [frame("de", 0), frame("plain", 0)]
    n = service.autotune(frames, quality_scale=0.5)
    assert n == 2
    p = str(tmp_path / "tune.txt")
    assert service.autotune_save(p) == 0
    lines = open(p).read().split("\n")
    assert sum(1 for ln in lines if ln.strip()) >= 2
    assert service.autotune_load(p) == 0
    # tuned jobs draw other chunkings: same picture statistically
    ref, _, _ = plain("de", 0)
    try:
        with service.Service(use_tuning=1) as svc:
            out, st, _ = svc.wait(svc.submit(frame("de", 0)))
    finally:
        service.autotune_clear()
    assert float(np.mean(np.abs(out.astype(float) - ref.astype(float)))) < 3.0


def test_progress_callback_abort_pause_and_batch(gpulib):
    """Requests with a progress callback (the contract of rect.c:324-391):
    one that aborts at its first call completes with its output untouched
    while the requests beside it render; one that pauses for its first three
    calls renders after it resumes, like the plain render; the batch API calls
    the callbacks too."""
    calls = {"abort": [], "pause": [], "batch": []}

    def callback(name, answer):
        @abi.PROGRESS_FN
        def f(param, pct, stage, eta):
            calls[name].append(pct)
            return answer(len(calls[name]))
        return f

    abort_cb = callback("abort", lambda n: 1)
    pause_cb = callback("pause", lambda n: 2 if n <= 3 else 0)
    Fa, Fp, Fo = frame("de", 1), frame("de", 2), frame("plain", 3)
    Fa.f.progress = abort_cb
    Fp.f.progress = pause_cb
    with service.Service(round_samples=1 << 20) as svc:
        ta, tp, to = svc.submit(Fa), svc.submit(Fp), svc.submit(Fo)
        out_a, _, _ = svc.wait(ta)
        out_p, st_p, _ = svc.wait(tp)
        out_o, _, _ = svc.wait(to)
        cnt = svc.counters()
    assert len(calls["abort"]) == 1 and not out_a.any()
    assert len(calls["pause"]) >= 4 and all(0.0 <= c <= 100.0 for c in calls["pause"])
    ref_p, st_ref, _ = plain("de", 2)
    ok, info = close_images(out_p, ref_p)
    assert ok, info
    assert st_p.num_iters == st_ref.num_iters
    ref_o, _, _ = plain("plain", 3)
    ok, info = close_images(out_o, ref_o)
    assert ok, info
    assert cnt["jobs_done"] == 3 and cnt["jobs_failed"] == 0
    batch_cb = callback("batch", lambda n: 0)
    Fb = frame("de", 0)
    Fb.f.progress = batch_cb
    (out_b, _), = service.render_batch([Fb])
    assert len(calls["batch"]) >= 1 and out_b.mean() > 1.0


@pytest.mark.parametrize("order", [0, 1, 2])
def test_round_order_policies(gpulib, order):
    """A long job submitted just before short ones: shortest-remaining (0)
    and response-ratio (1) ordering let the short jobs pass it, arrival
    order (2) finishes it first; every image still equals the plain render."""
    import time

    def mk(size, q, seed):
        G = gm.small_genome(seed)
        gm.resize(G, size, size)
        G.g.sample_density = q
        return gm.Frame(G, bits=33, seed="order-%d-%d" % (order, seed))

    frames = [mk(512, 300.0, 0)] + [mk(64, 20.0, k) for k in range(1, 5)]
    done = []
    with service.Service(order=order, round_samples=1 << 22) as svc:
        # both arms warm (allocations, graphs) before the timed submissions
        svc.wait(svc.submit(mk(64, 5.0, 9)))
        subs = []
        for F in frames:
            t0 = time.perf_counter()
            subs.append((t0, svc.submit(F)))
        for t0, tk in subs:
            img, st, times = svc.wait(tk)
            done.append((t0 + times[2] * 1e-3, img))
    big = done[0][0]
    small = [d for d, _ in done[1:]]
    if order == 2:
        assert big < min(small), (big, small)
    else:
        assert max(small) < big, (big, small)
    for (_, img), F in zip(done, [mk(512, 300.0, 0)] + [mk(64, 20.0, k) for k in range(1, 5)]):
        ref, _ = render.render(F)
        ok, info = close_images(img, ref)
        assert ok, info
