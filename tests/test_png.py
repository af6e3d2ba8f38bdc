"""PNG output on the device (write_png, png.c:36-116) against the oracle.

Bar: every chunk's CRC-32 is right, IHDR carries write_png's parameters
(png.c:93-98), the IDAT chunks inflate (zlib checks the Adler-32) to exactly
the oracle's filtered stream (per-row filter choice included), which
reconstructs exactly the input pixels; the text chunks are write_png's, in
its order.  The CPU tests check the oracle's filter restatement and the
argument checks that need no device."""
import ctypes as C
import os
import struct
import zlib

import numpy as np
import pytest

import _oracle
from flam3_gb300 import genome as gm, render

SIG = b"\x89PNG\r\n\x1a\n"


def chunks(png):
    assert png[:8] == SIG
    out, p = [], 8
    while p < len(png):
        n, = struct.unpack(">I", png[p:p + 4])
        t, d = png[p + 4:p + 8], png[p + 8:p + 8 + n]
        crc, = struct.unpack(">I", png[p + 8 + n:p + 12 + n])
        assert zlib.crc32(t + d) == crc, (t, p)
        out.append((t.decode("latin-1"), d))
        p += 12 + n
    assert p == len(png)
    return out


def decode(png, shape, dtype):
    """(pixels, filtered stream, IHDR tuple, text chunks) of a PNG."""
    cs = chunks(png)
    assert cs[0][0] == "IHDR" and cs[-1] == ("IEND", b"")
    ihdr = struct.unpack(">IIBBBBB", cs[0][1])
    names = [t for t, _ in cs]
    first = names.index("IDAT")
    last = len(names) - 1 - names[::-1].index("IDAT")
    assert all(t == "IDAT" for t in names[first:last + 1])
    F = np.frombuffer(zlib.decompress(b"".join(d for t, d in cs if t == "IDAT")), np.uint8)
    texts = [(t, d) for t, d in cs[1:first]]
    return _oracle.png_unfilter(F, shape, dtype), F, ihdr, texts


def text_items(texts):
    out = []
    for t, d in texts:
        k, rest = d.split(b"\0", 1)
        if t == "zTXt":
            assert rest[0] == 0
            rest = zlib.decompress(rest[1:])
        out.append((t, k.decode(), rest.decode("latin-1")))
    return out


def render_like(h, w, nchan=4, dtype=np.uint8, seed=0):
    """black background, a noisy bright blob, alpha 255 (as a flame render)"""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w]
    v = np.exp(-((xx - w * .45) ** 2 + (yy - h * .5) ** 2) / (0.05 * w * h)) + rng.normal(0, .03, (h, w))
    top = 65535 if dtype == np.uint16 else 255
    img = np.zeros((h, w, nchan), np.float64)
    for k, s in enumerate((1.0, .6, .25)):
        img[..., k] = v * s
    img = np.clip(img * top, 0, top)
    img[v < .08] = 0
    if nchan == 4:
        img[..., 3] = top
    return img.astype(dtype)


# ---- CPU: the oracle restatement ----

def test_oracle_filter_reconstructs_and_picks_cheapest():
    rng = np.random.default_rng(3)
    for shape, dt in [((7, 9, 4), np.uint8), ((5, 6, 3), np.uint16), ((1, 1, 4), np.uint8)]:
        img = rng.integers(0, np.iinfo(dt).max + 1, shape, dtype=dt)
        F = _oracle.png_filter(img)
        assert np.array_equal(_oracle.png_unfilter(F, shape, dt), img)
    # a horizontal ramp: Sub makes every byte after the first pixel 1 -> type 1
    ramp = np.tile(np.arange(16, dtype=np.uint8)[None, :, None], (3, 1, 4))
    F = _oracle.png_filter(ramp).reshape(3, -1)
    assert list(F[:, 0]) == [1, 2, 2]  # row 0 Sub; later rows Up (all zero)


def test_encode_argument_checks_without_gpu():
    lib = render.load()
    out = C.POINTER(C.c_ubyte)()
    n = C.c_size_t()
    buf = (C.c_ubyte * 64)()
    for w, h, nchan, bpc in [(0, 4, 4, 1), (4, 4, 5, 1), (4, 4, 4, 3), (4, -1, 3, 2)]:
        assert lib.flam3gpu_encode_png(buf, 0, w, h, nchan, bpc, None, 0, C.byref(out), C.byref(n)) == 1
    assert lib.flam3gpu_encode_png(None, 0, 4, 4, 4, 1, None, 0, C.byref(out), C.byref(n)) == 1
    # text chunk keywords: 1-79 bytes (checked before any device work)
    bad = (render.PngText * 2)(render.PngText(b"ok", b"x", 0), render.PngText(b"k" * 80, b"x", 0))
    assert lib.flam3gpu_encode_png(buf, 0, 4, 4, 4, 1, bad, 2, C.byref(out), C.byref(n)) == 1
    assert b"keyword" in lib.flam3gpu_last_error()
    assert lib.flam3gpu_encode_png(buf, 0, 4, 4, 4, 1, None, 1, C.byref(out), C.byref(n)) == 1


# ---- GPU ----

IMAGES = [
    # id, h, w, nchan, dtype, kind
    ("rgba8_render", 181, 243, 4, np.uint8, "render"),
    ("rgb8_render", 120, 333, 3, np.uint8, "render"),
    ("rgba16_render", 97, 150, 4, np.uint16, "render"),
    ("rgb16_noise", 31, 77, 3, np.uint16, "noise"),
    ("rgba8_noise", 64, 300, 4, np.uint8, "noise"),
    ("black", 300, 411, 4, np.uint8, "zero"),
    ("one_pixel", 1, 1, 4, np.uint8, "noise"),
    ("one_row", 1, 5000, 4, np.uint8, "render"),
    ("one_column", 3000, 1, 3, np.uint8, "render"),
    ("wide_rows", 12, 9001, 4, np.uint8, "render"),      # rows longer than the 32 KB window
    ("segment_edge", 64, 128, 4, np.uint8, "noise"),     # stream of 64 * 513 bytes
    ("uhd_rgba16", 2160, 3840, 4, np.uint16, "render"),  # 66 MB raw, about 4050 segments
]


def make(h, w, nchan, dt, kind, seed):
    rng = np.random.default_rng(seed)
    if kind == "noise":
        return rng.integers(0, np.iinfo(dt).max + 1, (h, w, nchan), dtype=dt)
    if kind == "zero":
        return np.zeros((h, w, nchan), dt)
    return render_like(h, w, nchan, dt, seed)


@pytest.mark.gpu
@pytest.mark.parametrize("case", IMAGES, ids=[c[0] for c in IMAGES])
def test_encode_png_round_trip(gpulib, case):
    cid, h, w, nchan, dt, kind = case
    img = make(h, w, nchan, dt, kind, 11)
    png = render.encode_png(img)
    pix, F, ihdr, texts = decode(png, img.shape, dt)
    assert ihdr == (w, h, 8 * img.dtype.itemsize, 6 if nchan == 4 else 2, 0, 0, 0)
    assert texts == []
    assert np.array_equal(F, _oracle.png_filter(img)), cid
    assert np.array_equal(pix, img), cid
    if kind == "render" and h * w >= 10000:
        # the segment coder against zlib's default level on the same stream
        # (a sanity bound: matches stop at each thread's 64-byte share, which
        # costs most on long black runs)
        assert len(png) < 2.0 * len(zlib.compress(F.tobytes(), 6)) + 200, (len(png), len(zlib.compress(F.tobytes(), 6)))


@pytest.mark.gpu
def test_encode_png_from_device_memory(gpulib):
    import torch

    img = render_like(200, 260, 4, np.uint8, 5)
    d = torch.from_numpy(img).cuda()
    torch.cuda.synchronize()
    png = render.encode_png(img, on_device_ptr=d.data_ptr())
    pix, _, _, _ = decode(png, img.shape, np.uint8)
    assert np.array_equal(pix, img)


@pytest.mark.gpu
def test_write_png_text_chunks(gpulib, tmp_path, monkeypatch):
    monkeypatch.setenv("nick", "someone")
    monkeypatch.delenv("url", raising=False)
    monkeypatch.setenv("id", "42")
    monkeypatch.delenv("enable_png_comments", raising=False)
    img = render_like(90, 120, 4, np.uint16, 2)
    genome = '<flame name="t" size="120 90">' + "x" * 70000 + "</flame>"
    path = str(tmp_path / "a.png")
    render.write_png(path, img, genome=genome, badvals="0.001", numiters="1e+06", rtime="3")
    png = open(path, "rb").read()
    pix, _, _, texts = decode(png, img.shape, np.uint16)
    assert np.array_equal(pix, img)
    items = text_items(texts)
    assert [(t, k) for t, k, _ in items] == [("tEXt", "flam3_version"), ("tEXt", "flam3_nickname"),
                                             ("tEXt", "flam3_url"), ("tEXt", "flam3_id"),
                                             ("tEXt", "flam3_error_rate"), ("tEXt", "flam3_samples"),
                                             ("tEXt", "flam3_time"), ("zTXt", "flam3_genome")]
    vals = {k: v for _, k, v in items}
    assert vals["flam3_nickname"] == "someone" and vals["flam3_url"] == "" and vals["flam3_id"] == "42"
    assert vals["flam3_error_rate"] == "0.001" and vals["flam3_samples"] == "1e+06" and vals["flam3_time"] == "3"
    assert vals["flam3_genome"] == genome
    monkeypatch.setenv("enable_png_comments", "0")
    render.write_png(path, img)
    _, _, _, texts = decode(open(path, "rb").read(), img.shape, np.uint16)
    assert texts == []


@pytest.mark.gpu
@pytest.mark.parametrize("bpc,transp", [(1, 0), (2, 1)])
def test_render_png_matches_render(gpulib, bpc, transp):
    def mk():
        G = gm.small_genome(4, 256, 192, 40.0)
        return gm.Frame(G, bits=33, seed="png-%d" % bpc, bytes_per_channel=bpc)

    png, st = render.render_png(mk(), transp=transp, genome_xml="<flame/>")
    ref, st2 = render.render(mk(), nchan=4, transp=transp)
    dt = np.uint8 if bpc == 1 else np.uint16
    pix, F, ihdr, texts = decode(png, ref.shape, dt)
    assert ihdr[:4] == (256, 192, 8 * bpc, 6)
    assert np.array_equal(F, _oracle.png_filter(pix))
    d = np.abs(pix.astype(np.int64) - ref.astype(np.int64))
    if bpc == 2:
        d //= 256
    assert float(np.mean(d <= 1)) >= 0.999
    assert st.num_iters == st2.num_iters
    vals = {k: v for _, k, v in text_items(texts)}
    assert vals["flam3_samples"] == "%g" % st.num_iters
    assert vals["flam3_genome"] == "<flame/>"
    assert render.png_last_ms() > 0


@pytest.mark.gpu
def test_render_batch_png_matches_render_batch(gpulib):
    from flam3_gb300 import service

    def frames(tag):
        gs = gm.animation_keys(2, width=192, height=108, quality=30.0, temporal_samples=10)
        # 35 frames: two chunks of the batch pipeline
        return [gm.Frame(gs, bits=33, seed="bpng-%d" % i, time=float(i)) for i in range(35)]

    got = service.render_batch_png(frames("a"))
    ref = service.render_batch(frames("a"), nchan=4)
    for (png, st), (img, st2) in zip(got, ref):
        pix, F, ihdr, texts = decode(png, img.shape, np.uint8)
        assert ihdr[:4] == (192, 108, 8, 6)
        assert np.array_equal(F, _oracle.png_filter(pix))
        assert float(np.mean(np.abs(pix.astype(np.int64) - img.astype(np.int64)) <= 1)) >= 0.999
        assert st.num_iters == st2.num_iters
        vals = {k: v for _, k, v in text_items(texts)}
        assert vals["flam3_samples"] == "%g" % st.num_iters and vals["flam3_genome"] == ""
