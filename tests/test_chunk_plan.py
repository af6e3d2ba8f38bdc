"""The iterate launch's chunking (f3g_chunk_passes, host/render.c), through
the host probe flam3gpu_chunk_plan: every pass's samples covered exactly by
its chunks, full-length chunks first and quarter-length chunks over the
launch's last samples (half a wave of full chunks, a whole wave for 2048-sample
chains), and the chain length rule (1024, or 2048 for launches of 8 or more
waves of 2048, never above the sub-batch size)."""
import numpy as np
import pytest

from flam3_gb300 import render

T, B = 256, 608


def check_plan(samples, sub=10000):
    S, St, ct, nc = render.chunk_plan(samples, T, B, sub)
    total = sum(samples)
    per = total // (T * B)
    cap = min(2048 if per >= 8 * 2048 else 1024, sub)
    assert S == min(max(min(per, cap), 64), cap), (S, per, cap)
    assert St == (S // 4 if S >= 512 and S // 4 >= 64 else S)
    big, small = T * S, T * St
    short_region = 0
    first_short = None
    for i, (n, c0, c) in enumerate(zip(samples, ct, nc)):
        assert 0 <= c0 <= c
        if St == S or c0 == c:
            # every chunk full length (the last may be shorter)
            assert c == -(-n // big), (i, n, c0, c)
            assert c0 == c
        else:
            # whole full-length chunks, then short ones to the end
            assert c0 * big <= n, (i, n, c0)
            rest = n - c0 * big
            assert c == c0 + -(-rest // small), (i, n, c0, c)
            short_region += rest
            if first_short is None:
                first_short = i
    if first_short is not None:
        # the short chunks sit at the end of the launch: every later pass is all short
        for i in range(first_short + 1, len(samples)):
            assert ct[i] == 0 or samples[i] == 0
        waves = 1.0 if S >= 2048 else 0.5
        want = int(waves * B * big)
        assert short_region >= min(want, total) and short_region < want + big, (short_region, want)
    return S, St, ct, nc


def test_single_pass_still():
    # the 1920x1080 q2000 still: 4.147 G samples, 26 waves of 1024 -> 2048-sample chains
    S, St, ct, nc = check_plan([4147200000])
    assert (S, St) == (2048, 512)
    assert nc[0] - ct[0] > 0


def test_animation_frame():
    # 100 temporal samples of a 1280x720 q500 frame: 3 waves of 1024
    S, St, ct, nc = check_plan([4608000] * 100)
    assert (S, St) == (1024, 256)
    assert ct[0] == nc[0] and ct[-1] < nc[-1]


def test_small_and_empty():
    check_plan([1000])
    check_plan([0, 0, 5, 0])
    S, St, _, _ = check_plan([3 * 256 * 64])
    assert S == 64 and St == 64  # no short chunks below 512-sample chains
    check_plan([123456789], sub=300)  # the sub-batch size caps the chains


@pytest.mark.parametrize("seed", range(6))
def test_random_pass_lists(seed):
    rng = np.random.default_rng(seed)
    for _ in range(25):
        n = int(rng.integers(1, 120))
        scale = 10 ** rng.uniform(3, 9.5)
        samples = [int(x) for x in rng.uniform(0, 1, n) * scale]
        a = check_plan(samples)
        assert a == render.chunk_plan(samples, T, B, 10000)  # the same plan every time
