"""ISAAC seeding of a flam3_frame's random context (isaac.c:25-110,
flam3.c:2494-2516), so callers can set up `frame.rc` exactly as
flam3_init_frame does for a given isaac_seed string.  `ub4` is unsigned long
(64-bit), and the arithmetic is masked exactly where the reference masks it.
"""
M64 = (1 << 64) - 1
M32 = 0xFFFFFFFF
RANDSIZL = 4
RANDSIZ = 1 << RANDSIZL


def _mix(a, b, c, d, e, f, g, h):
    a ^= (b << 11) & M64; d = (d + a) & M64; b = (b + c) & M64
    b ^= c >> 2;          e = (e + b) & M64; c = (c + d) & M64
    c ^= (d << 8) & M64;  f = (f + c) & M64; d = (d + e) & M64
    d ^= e >> 16;         g = (g + d) & M64; e = (e + f) & M64
    e ^= (f << 10) & M64; h = (h + e) & M64; f = (f + g) & M64
    f ^= g >> 4;          a = (a + f) & M64; g = (g + h) & M64
    g ^= (h << 8) & M64;  b = (b + g) & M64; h = (h + a) & M64
    h ^= a >> 9;          c = (c + h) & M64; a = (a + b) & M64
    return a, b, c, d, e, f, g, h


def isaac(rc):
    mm = rc.randmem
    r = rc.randrsl
    a = rc.randa
    rc.randc = (rc.randc + 1) & M64
    b = (rc.randb + rc.randc) & M32
    half = RANDSIZ // 2
    order = [(i, i + half) for i in range(half)] + [(i + half, i) for i in range(half)]
    for k, (mi, m2i) in enumerate(order):
        s = k & 3
        if s == 0:
            mix = (a << 13) & M64
        elif s == 1:
            mix = a >> 6
        elif s == 2:
            mix = (a << 2) & M64
        else:
            mix = a >> 16
        x = mm[mi]
        a = ((a ^ mix) + mm[m2i]) & M32
        y = (mm[(x >> 2) & (RANDSIZ - 1)] + a + b) & M32
        mm[mi] = y
        b = (mm[(y >> RANDSIZL >> 2) & (RANDSIZ - 1)] + x) & M32
        r[k] = b
    rc.randb = b
    rc.randa = a


def irandinit(rc, flag=True):
    rc.randa = rc.randb = rc.randc = 0
    m = rc.randmem
    r = rc.randrsl
    v = [0x9E3779B9] * 8
    for _ in range(4):
        v = list(_mix(*v))
    if flag:
        for src in (r, m):
            for i in range(0, RANDSIZ, 8):
                v = [(v[k] + src[i + k]) & M64 for k in range(8)]
                v = list(_mix(*v))
                for k in range(8):
                    m[i + k] = v[k]
    else:
        for i in range(0, RANDSIZ, 8):
            v = list(_mix(*v))
            for k in range(8):
                m[i + k] = v[k]
    isaac(rc)
    rc.randcnt = RANDSIZ


def irand(rc):
    if rc.randcnt == 0:
        isaac(rc)
        rc.randcnt = RANDSIZ - 1
    else:
        rc.randcnt -= 1
    return rc.randrsl[rc.randcnt]


def init_rc(rc, seed):
    """flam3_init_frame with isaac_seed=`seed` (bytes/str, up to 128 bytes)."""
    if isinstance(seed, str):
        seed = seed.encode()
    buf = bytearray(8 * RANDSIZ)
    buf[: min(len(seed), len(buf))] = seed[: len(buf)]
    for i in range(RANDSIZ):
        rc.randrsl[i] = int.from_bytes(buf[8 * i: 8 * i + 8], "little")
    irandinit(rc, True)
