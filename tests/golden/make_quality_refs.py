"""Reference renders for the matched-image-error measurement.

Each case is one request of the synthetic workloads (the config-1 still,
draws of the mixed-size batch, the serving trace's 3840x2160 still), cut to
a window of at most 480x270 output pixels at the request's own pixels per
unit, so its samples per pixel, oversample, DE radius and filter are the
request's.  The reference is the oracle (the plain-C restatement of the
reference path, pinned to the reference) rendering that window in FP64
buckets (bits 64) at 16x the request's quality; the error of any render of
the window at quality q is its per-channel mean absolute difference from
that reference in 8-bit levels, and its PSNR.

The fixture also records the oracle's own error at q/16, q/4 and q (its own
bits and bits 64), so a GPU render can be held to the error the reference's
arithmetic makes at the same quality.

Run from the repository root (minutes: about 8 G oracle iterations):
    python tests/golden/make_quality_refs.py
writes tests/golden/quality_refs.npz.
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from flam3_gb300 import genome as gm  # noqa: E402

PATH = os.path.join(HERE, "quality_refs.npz")
REF_FACTOR = 16

# name -> (workload, index in it, window width, window height)
CASES = {
    "still_crop": ("still", 0, 480, 270),               # 1920x1080 q2000 ss2 DE9, 6 xforms + final
    "mixed83_b64_ss2_de3": ("mixed", 83, 256, 256),     # bits 64
    "mixed17_ss2_de9": ("mixed", 17, 256, 256),
    "mixed6_ss1_node": ("mixed", 6, 256, 256),
    "mixed15_ss2_de6": ("mixed", 15, 256, 192),          # 1024x768 q899
    "mixed14_ss1_de11": ("mixed", 14, 256, 192),         # 1024x768 q58: wide kernels on a sparse histogram
    "trace57_big_de11": ("trace", 57, 384, 216),         # 3840x2160 q1000 ss2 DE11
}


def request(name):
    """The full-frame request of a case: (Genome, bits)."""
    src, idx, _, _ = CASES[name]
    if src == "still":
        return gm.still_genome(1), 33
    if src == "mixed":
        return gm.mixed_jobs(seed=3, njobs=idx + 1)[idx]
    _, G, bits = gm.serving_trace(seed=4, nrequests=64)[idx]
    return G, bits


def build(name, meta, quality=None):
    """The case's window as a Genome at `quality` (default: the request's),
    camera taken from the fixture so every platform frames it identically."""
    G, bits = request(name)
    g = G.g
    g.width, g.height = int(meta["w"]), int(meta["h"])
    g.center[0], g.center[1] = float(meta["cx"]), float(meta["cy"])
    g.pixels_per_unit = float(meta["ppu"])
    g.sample_density = float(meta["q"] if quality is None else quality)
    return G, bits


def mae(a, b):
    return float(np.mean(np.abs(a.astype(np.float64) - b.astype(np.float64))))


def psnr(a, b):
    mse = float(np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2))
    return float("inf") if mse == 0 else 10.0 * np.log10(255.0 ** 2 / mse)


def load():
    """name -> dict(meta..., ref=uint8 image, oracle_mae={...})."""
    d = np.load(PATH)
    meta = json.loads(str(d["meta"]))
    out = {}
    for name, m in meta.items():
        m = dict(m)
        m["ref"] = d["ref_" + name]
        out[name] = m
    return out


def _window(G, w, h):
    """Offset (dx, dy) of the w x h window with the most pixels that are
    neither black nor saturated, from a quality-10 preview of the full frame."""
    import _oracle

    g = G.g
    W, H = g.width, g.height
    if W <= w and H <= h:
        return 0.0, 0.0
    q0 = g.sample_density
    g.sample_density = 10.0
    img, _, _ = _oracle.oracle_render(gm.Frame(G, bits=64, nthreads=os.cpu_count(), seed="preview"), fast=True)
    g.sample_density = q0
    m = img.astype(np.float64).mean(2)
    score = ((m > 0) & (m < 250)).astype(np.float64)
    S = np.pad(score.cumsum(0).cumsum(1), ((1, 0), (1, 0)))
    best = None
    for y in range(0, H - h + 1, 8):
        for x in range(0, W - w + 1, 8):
            v = S[y + h, x + w] - S[y, x + w] - S[y + h, x] + S[y, x]
            if best is None or v > best[0]:
                best = (v, x, y)
    _, x, y = best
    return (x + w / 2.0) - W / 2.0, (y + h / 2.0) - H / 2.0


def main():
    import _oracle

    meta, arrays = {}, {}
    nt = os.cpu_count()
    for name, (src, idx, w, h) in CASES.items():
        t0 = time.time()
        G, bits = request(name)
        dx, dy = _window(G, w, h)
        gm.crop(G, w, h, dx, dy)
        g = G.g
        m = dict(src=src, index=idx, w=w, h=h, dx=dx, dy=dy, cx=g.center[0], cy=g.center[1], ppu=g.pixels_per_unit,
                 q=g.sample_density, bits=bits, oversample=g.spatial_oversample, estimator=g.estimator,
                 ref_quality=g.sample_density * REF_FACTOR, ref_bits=64)
        G, _ = build(name, m, quality=m["ref_quality"])
        ref, st, _ = _oracle.oracle_render(gm.Frame(G, bits=64, nthreads=nt, seed="reference-16x"), fast=True)
        arrays["ref_" + name] = ref
        errs = {}
        for b in sorted({bits, 64}):
            for div in (16, 4, 1):
                G, _ = build(name, m, quality=m["q"] / div)
                img, _, _ = _oracle.oracle_render(gm.Frame(G, bits=b, nthreads=nt, seed="oracle-q"), fast=True)
                errs["b%d_q/%d" % (b, div)] = [mae(img, ref), psnr(img, ref)]
        m["oracle_mae"] = errs
        m["ref_mean"] = float(ref.mean())
        meta[name] = m
        print("%-22s %4dx%-4d q=%7.1f ref mean %.2f  oracle MAE %s  (%.0f s)" % (
            name, w, h, m["q"], ref.mean(), {k: round(v[0], 3) for k, v in errs.items()}, time.time() - t0),
            flush=True)
    np.savez_compressed(PATH, meta=json.dumps(meta), **arrays)
    print("wrote", PATH, os.path.getsize(PATH), "bytes")


if __name__ == "__main__":
    main()
