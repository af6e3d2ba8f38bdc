"""GPU apply_xform (all 99 variations) against the reference's own vectors
(tests/golden/variations.npz) and the oracle, given identical points and
random words.

Tolerances: FP64 iteration matches to 1e-12 relative (CUDA's and glibc's
libm differ by an ulp or two); FP32 iteration is held to 2e-4 relative +
2e-5 absolute on at least 99% of outputs (points next to a pole or a branch
cut of atan2/fmod/floor may land on the other side in FP32)."""
import os

import numpy as np
import pytest

from flam3_gb300 import abi, render
import _oracle
from golden import make_golden as mg

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def cases():
    d = np.load(os.path.join(GOLD, "variations.npz"))
    for k in range(d["q"].shape[0]):
        yield k, {n: d[n][k] for n in ("coefs", "post", "var", "params", "color", "color_speed", "opacity",
                                       "points", "words", "q", "bad")}


def close(a, b, rtol, atol):
    return np.abs(a - b) <= atol + rtol * np.maximum(np.abs(a), np.abs(b))


def test_fp64_apply_xform_matches_reference_vectors(gpulib):
    fails = []
    for k, c in cases():
        G = mg.genome_from_case(c)
        q, bad = render.apply_xform(G, 0, c["points"], c["words"], precision=64)
        ok = close(q, c["q"], 1e-12, 1e-12)
        # a bad value is replaced by random words on both sides; compare flags
        if not np.all(ok) or not np.array_equal(bad, c["bad"]):
            vars_ = [abi.VARIATION_NAMES[j] for j in np.nonzero(c["var"])[0]]
            fails.append((k, vars_, float(np.max(np.abs(q - c["q"])))))
    assert not fails, fails[:10]


def test_fp32_apply_xform_within_bound(gpulib):
    total, good = 0, 0
    worst = []
    for k, c in cases():
        G = mg.genome_from_case(c)
        q, bad = render.apply_xform(G, 0, c["points"], c["words"], precision=32)
        ok = close(q, c["q"], 2e-4, 2e-5)
        total += ok.size
        good += int(ok.sum())
        if ok.mean() < 0.9:
            worst.append((k, [abi.VARIATION_NAMES[j] for j in np.nonzero(c["var"])[0]], float(ok.mean())))
    assert good / total >= 0.99, (good / total, worst[:10])


def test_gpu_matches_oracle_on_fresh_vectors(gpulib):
    rng = np.random.default_rng(99)
    for k, c in list(cases())[::7]:
        c = dict(c)
        c["points"] = np.stack([rng.uniform(-3, 3, 64), rng.uniform(-3, 3, 64), rng.uniform(0, 1, 64),
                                rng.uniform(0, 1, 64)], 1)
        c["words"] = rng.integers(0, 2 ** 32, size=(64, 24), dtype=np.uint64).astype(np.uint32)
        G = mg.genome_from_case(c)
        qo, bo = _oracle.oracle_apply_xform(G, 0, c["points"], c["words"])
        G = mg.genome_from_case(c)
        qg, bg = render.apply_xform(G, 0, c["points"], c["words"], precision=64)
        assert np.all(close(qg, qo, 1e-12, 1e-12)), k
        assert np.array_equal(bg, bo)
