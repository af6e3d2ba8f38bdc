"""Genome and frame construction on the flam3 ABI (flam3_gb300.abi).

`Genome` owns the ctypes memory of one flam3_genome (its xform array and
chaos rows) and starts from the reference defaults: clear_cp with
flam3_defaults_on (flam3.c:1270-1370) and initialize_xforms
(variations.c:2401-2563).  `Frame` wraps a flam3_frame over a list of
genomes with the ISAAC context seeded as flam3_init_frame does.

The seeded generators `small_genome` ... `serving_trace` build the
synthetic workloads (3 xforms linear/sinusoidal/spherical; 6+final xforms
drawn from variations 0-19; interpolated animations; mixed-size batches).
Their camera rule: center on the bounding box of a short chaos game
(quantiles eps=0.01 as flam3_estimate_bounding_box, flam3.c:3574) and scale
so that box fills 90% of the frame.
"""
import ctypes as C
import math

import numpy as np

from . import abi
from .isaac import init_rc

# defaults of initialize_xforms (variations.c:2432-2561); unlisted params are 0
_XFORM_PARAM_DEFAULTS = {
    "blob_high": 1.0, "blob_waves": 1.0, "bent2_x": 1.0, "bent2_y": 1.0, "cell_size": 1.0,
    "cpow_r": 1.0, "cpow_power": 1.0, "curve_xlength": 1.0, "curve_ylength": 1.0,
    "oscope_separation": 1.0, "oscope_frequency": math.pi, "oscope_amplitude": 1.0,
    "wedge_count": 1.0, "wedge_sph_count": 1.0, "wedge_julia_power": 1.0, "wedge_julia_count": 1.0,
    "wedgeJulia_cn": 0.5, "wedgeJulia_rN": 1.0, "auger_freq": 1.0, "auger_weight": 0.5,
    "auger_scale": 1.0, "julian_power": 1.0, "julian_dist": 1.0, "julian_rN": 1.0, "julian_cn": 0.5,
    "juliascope_power": 1.0, "juliascope_dist": 1.0, "juliascope_rN": 1.0, "juliascope_cn": 0.5,
    "radialBlur_zoomvar": 1.0, "pie_slices": 6.0, "pie_thickness": 0.5, "ngon_sides": 5.0,
    "ngon_power": 3.0, "ngon_circle": 1.0, "ngon_corners": 2.0, "curl_c1": 1.0,
    "rectangles_x": 1.0, "rectangles_y": 1.0, "amw_amp": 1.0, "super_shape_n1": 1.0,
    "super_shape_n2": 1.0, "super_shape_n3": 1.0, "conic_eccentricity": 1.0,
}


def init_xform(x, index):
    """initialize_xforms (variations.c:2401-2563) for one xform."""
    C.memset(C.addressof(x), 0, C.sizeof(x))
    x.color_speed = 0.5
    x.animate = 1.0
    x.color = float(index & 1)
    x.opacity = 1.0
    x.var[0] = 1.0
    x.c[0][0] = 1.0
    x.c[1][1] = 1.0
    x.post[0][0] = 1.0
    x.post[1][1] = 1.0
    for k, v in _XFORM_PARAM_DEFAULTS.items():
        setattr(x, k, v)


def clear_genome_defaults(g):
    """clear_cp(cp, flam3_defaults_on) (flam3.c:1270-1330) on a zeroed genome."""
    g.palette_index = -1
    g.gamma = 4.0
    g.vibrancy = 1.0
    g.contrast = 1.0
    g.brightness = 4.0
    g.pixels_per_unit = 50
    g.palette_interpolation = 3  # hsv_circular
    g.highlight_power = -1.0
    g.width = 100
    g.height = 100
    g.spatial_oversample = 1
    g.spatial_filter_radius = 0.5
    g.sample_density = 1
    g.estimator = 9.0
    g.estimator_curve = 0.4
    g.gam_lin_thresh = 0.01
    g.nbatches = 1
    g.ntemporal_samples = 1000
    g.spatial_filter_select = 0
    g.interpolation_type = 1  # log
    g.temporal_filter_type = 0
    g.temporal_filter_width = 1.0
    g.palette_mode = 0
    g.final_xform_index = -1
    g.final_xform_enable = 0


class Genome:
    """One flam3_genome with Python-owned xform and chaos storage."""

    def __init__(self, num_std, final=False):
        self.g = abi.flam3_genome()
        clear_genome_defaults(self.g)
        self.num_std = num_std
        n = num_std + (1 if final else 0)
        self._xforms = (abi.flam3_xform * max(n, 1))()
        for i in range(n):
            init_xform(self._xforms[i], i)
        self.g.xform = C.cast(self._xforms, C.POINTER(abi.flam3_xform))
        self.g.num_xforms = n
        if final:
            self.g.final_xform_index = num_std
            self.g.final_xform_enable = 1
        self._chaos_rows = [(C.c_double * max(num_std, 1))(*([1.0] * num_std)) for _ in range(num_std)]
        self._chaos = (C.POINTER(C.c_double) * max(num_std, 1))(
            *[C.cast(r, C.POINTER(C.c_double)) for r in self._chaos_rows])
        self.g.chaos = C.cast(self._chaos, C.POINTER(C.POINTER(C.c_double)))
        for i in range(256):
            self.g.palette[i].index = float(i)
            self.g.palette[i].color[3] = 1.0

    def xform(self, i):
        return self._xforms[i]

    @property
    def final(self):
        return self._xforms[self.num_std] if self.g.final_xform_index >= 0 else None

    def set_chaos(self, i, j, v):
        self._chaos_rows[i][j] = v

    def set_palette(self, rgb):
        rgb = np.asarray(rgb, dtype=np.float64)
        for i in range(256):
            e = self.g.palette[i]
            e.index = float(i)
            e.color[0], e.color[1], e.color[2] = (float(v) for v in rgb[i, :3])
            e.color[3] = float(rgb[i, 3]) if rgb.shape[1] > 3 else 1.0

    def palette_array(self):
        return np.array([[self.g.palette[i].color[k] for k in range(4)] for i in range(256)])


class Frame:
    """A flam3_frame over Genome objects (kept alive here)."""

    def __init__(self, genomes, bits=33, nthreads=1, seed="flam3-gb300", time=0.0, earlyclip=0,
                 bytes_per_channel=1, sub_batch_size=10000, pixel_aspect_ratio=1.0):
        if isinstance(genomes, Genome):
            genomes = [genomes]
        self.genomes = list(genomes)
        self._garr = (abi.flam3_genome * len(self.genomes))(*[g.g for g in self.genomes])
        # the array holds copies of the genome structs; xform/chaos pointers are shared
        self.f = abi.flam3_frame()
        self.f.pixel_aspect_ratio = pixel_aspect_ratio
        self.f.genomes = C.cast(self._garr, C.POINTER(abi.flam3_genome))
        self.f.ngenomes = len(self.genomes)
        self.f.verbose = 0
        self.f.bits = bits
        self.f.bytes_per_channel = bytes_per_channel
        self.f.earlyclip = earlyclip
        self.f.time = time
        self.f.nthreads = nthreads
        self.f.sub_batch_size = sub_batch_size
        init_rc(self.f.rc, seed)

    def sync(self):
        """Copy edited Genome structs into the frame's genome array."""
        for i, g in enumerate(self.genomes):
            self._garr[i] = g.g

    def genome(self, i=0):
        return self._garr[i]

    @property
    def width(self):
        return self._garr[0].width

    @property
    def height(self):
        return self._garr[0].height

    def out_buffer(self, nchan=3):
        bpc = self.f.bytes_per_channel
        dt = np.uint8 if bpc == 1 else np.uint16
        return np.zeros((self.height, self.width, nchan), dtype=dt)


# ---------------------------------------------------------------------------
# seeded synthetic workloads
# ---------------------------------------------------------------------------

def genome_from_struct(src):
    """A Genome holding a copy of a C flam3_genome (xforms, chaos rows;
    motion elements and edits are not carried)."""
    nx = src.num_xforms
    final = src.final_xform_index >= 0
    num_std = nx - (1 if final else 0)
    G = Genome(num_std, final=final)
    C.memmove(C.addressof(G.g), C.addressof(src), C.sizeof(abi.flam3_genome))
    # the pointers back to this Genome's own storage
    G.g.xform = C.cast(G._xforms, C.POINTER(abi.flam3_xform))
    G.g.chaos = C.cast(G._chaos, C.POINTER(C.POINTER(C.c_double)))
    G.g.edits = None
    for i in range(nx):
        C.memmove(C.addressof(G._xforms[i]), C.addressof(src.xform[i]), C.sizeof(abi.flam3_xform))
        G._xforms[i].motion = None
        G._xforms[i].num_motion = 0
    for i in range(num_std):
        for j in range(num_std):
            G._chaos_rows[i][j] = src.chaos[i][j]
    return G


def parse_flam3(xml, filename="", default_flag=1):
    """flam3_parse_xml2 through the library's reader: the <flame> elements of
    an XML text (str or bytes) as Genomes."""
    from . import render
    lib = render.load()
    data = xml.encode() if isinstance(xml, str) else bytes(xml)
    n = C.c_int(0)
    p = lib.flam3gpu_parse_xml2(C.c_char_p(data), C.c_char_p(filename.encode()), default_flag, C.byref(n))
    if not p:
        raise render.Flam3GpuError("flam3gpu_parse_xml2 failed: " + lib.flam3gpu_last_error().decode())
    try:
        return [genome_from_struct(p[i]) for i in range(n.value)]
    finally:
        for i in range(n.value):
            lib.flam3gpu_free_genome(C.byref(p[i]))
        C.CDLL(None).free(C.cast(p, C.c_void_p))


def random_palette(rng, ncontrol=8):
    """256-entry RGB gradient through `ncontrol` U(0,1) control colours."""
    ctl = rng.uniform(0.0, 1.0, size=(ncontrol, 3))
    xs = np.linspace(0.0, 255.0, ncontrol)
    idx = np.arange(256, dtype=np.float64)
    rgb = np.stack([np.interp(idx, xs, ctl[:, k]) for k in range(3)], axis=1)
    return np.concatenate([rgb, np.ones((256, 1))], axis=1)


def _np_variations(tx, ty, var, xf, rng):
    """Vectorised variations 0-19 (variations.c:142-487) for camera framing."""
    eps = 1e-10
    sumsq = tx * tx + ty * ty
    sq = np.sqrt(sumsq)
    with np.errstate(all="ignore"):
        atan = np.arctan2(tx, ty)
        sina = tx / sq
        cosa = ty / sq
        p0 = np.zeros_like(tx)
        p1 = np.zeros_like(ty)
        for v, w in var:
            if v == 0:
                p0 += w * tx; p1 += w * ty
            elif v == 1:
                p0 += w * np.sin(tx); p1 += w * np.sin(ty)
            elif v == 2:
                r2 = w / (sumsq + eps); p0 += r2 * tx; p1 += r2 * ty
            elif v == 3:
                c1, c2 = np.sin(sumsq), np.cos(sumsq)
                p0 += w * (c1 * tx - c2 * ty); p1 += w * (c2 * tx + c1 * ty)
            elif v == 4:
                r = w / (sq + eps); p0 += (tx - ty) * (tx + ty) * r; p1 += 2.0 * tx * ty * r
            elif v == 5:
                p0 += w * atan / math.pi; p1 += w * (sq - 1.0)
            elif v == 6:
                p0 += w * sq * np.sin(atan + sq); p1 += w * sq * np.cos(atan - sq)
            elif v == 7:
                a = sq * atan; r = w * sq; p0 += r * np.sin(a); p1 -= r * np.cos(a)
            elif v == 8:
                a = atan / math.pi; r = math.pi * sq
                p0 += w * np.sin(r) * a; p1 += w * np.cos(r) * a
            elif v == 9:
                r = sq + eps; r1 = w / r
                p0 += r1 * (cosa + np.sin(r)); p1 += r1 * (sina - np.cos(r))
            elif v == 10:
                r = sq + eps; p0 += w * sina / r; p1 += w * cosa * r
            elif v == 11:
                p0 += w * sina * np.cos(sq); p1 += w * cosa * np.sin(sq)
            elif v == 12:
                n0 = np.sin(atan + sq); n1 = np.cos(atan - sq)
                m0 = n0 ** 3 * sq; m1 = n1 ** 3 * sq
                p0 += w * (m0 + m1); p1 += w * (m0 - m1)
            elif v == 13:
                a = 0.5 * atan + math.pi * rng.integers(0, 2, size=tx.shape)
                r = w * np.sqrt(sq); p0 += r * np.cos(a); p1 += r * np.sin(a)
            elif v == 14:
                nx = np.where(tx < 0, tx * 2.0, tx); ny = np.where(ty < 0, ty / 2.0, ty)
                p0 += w * nx; p1 += w * ny
            elif v == 15:
                dx2 = 1.0 / (xf.c[2][0] ** 2 + eps); dy2 = 1.0 / (xf.c[2][1] ** 2 + eps)
                p0 += w * (tx + xf.c[1][0] * np.sin(ty * dx2)); p1 += w * (ty + xf.c[1][1] * np.sin(tx * dy2))
            elif v == 16:
                r = 2 * w / (sq + 1); p0 += r * ty; p1 += r * tx
            elif v == 17:
                p0 += w * (tx + xf.c[2][0] * np.sin(np.tan(3 * ty)))
                p1 += w * (ty + xf.c[2][1] * np.sin(np.tan(3 * tx)))
            elif v == 18:
                dx = w * np.exp(tx - 1.0); dy = math.pi * ty
                p0 += dx * np.cos(dy); p1 += dx * np.sin(dy)
            elif v == 19:
                r = w * np.power(sq, sina); p0 += r * cosa; p1 += r * sina
            else:
                raise ValueError("camera framing supports variations 0-19")
    return p0, p1


def estimate_bbox(genome, eps=0.01, nchains=2048, steps=40, fuse=20, seed=1):
    """Bounding box holding all but `eps` of the attractor in each direction.
    A short vectorised chaos game used only to frame synthetic genomes."""
    rng = np.random.default_rng(seed)
    g = genome.g
    nstd = genome.num_std
    dens = np.array([genome.xform(i).density for i in range(nstd)])
    prob = dens / dens.sum()
    xs = rng.uniform(-1, 1, nchains)
    ys = rng.uniform(-1, 1, nchains)
    pts = []

    def apply(xf, x, y):
        c = xf.c
        tx = c[0][0] * x + c[1][0] * y + c[2][0]
        ty = c[0][1] * x + c[1][1] * y + c[2][1]
        var = [(j, xf.var[j]) for j in range(abi.NVARS) if xf.var[j] != 0]
        p0, p1 = _np_variations(tx, ty, var, xf, rng)
        pp = xf.post
        if not (pp[0][0] == 1 and pp[0][1] == 0 and pp[1][0] == 0 and pp[1][1] == 1 and pp[2][0] == 0 and pp[2][1] == 0):
            p0, p1 = pp[0][0] * p0 + pp[1][0] * p1 + pp[2][0], pp[0][1] * p0 + pp[1][1] * p1 + pp[2][1]
        return p0, p1

    for s in range(fuse + steps):
        choice = rng.choice(nstd, size=nchains, p=prob)
        nx = np.empty_like(xs)
        ny = np.empty_like(ys)
        for i in range(nstd):
            m = choice == i
            if m.any():
                nx[m], ny[m] = apply(genome.xform(i), xs[m], ys[m])
        bad = ~np.isfinite(nx) | ~np.isfinite(ny) | (np.abs(nx) > 1e10) | (np.abs(ny) > 1e10)
        nx[bad] = rng.uniform(-1, 1, bad.sum())
        ny[bad] = rng.uniform(-1, 1, bad.sum())
        xs, ys = nx, ny
        if s >= fuse:
            if g.final_xform_index >= 0:
                fx, fy = apply(genome.final, xs, ys)
                ok = np.isfinite(fx) & np.isfinite(fy)
                pts.append(np.stack([fx[ok], fy[ok]], 1))
            else:
                pts.append(np.stack([xs, ys], 1))
    p = np.concatenate(pts, 0)
    lo = np.quantile(p, eps, axis=0)
    hi = np.quantile(p, 1 - eps, axis=0)
    return lo, hi


def frame_camera(genome, width, height, fill=0.9, seed=1):
    lo, hi = estimate_bbox(genome, seed=seed)
    cx, cy = (lo + hi) / 2
    span_x = max(hi[0] - lo[0], 1e-6)
    span_y = max(hi[1] - lo[1], 1e-6)
    ppu = fill * min(width / span_x, height / span_y)
    g = genome.g
    g.center[0] = float(cx)
    g.center[1] = float(cy)
    g.pixels_per_unit = float(ppu)


def resize(genome, width, height):
    """Change the output size keeping the framing (pixels_per_unit scales
    with the width, as flam3-render's ss= option does)."""
    g = genome.g
    g.pixels_per_unit *= width / float(g.width)
    g.width = width
    g.height = height


def crop(genome, width, height, dx=0.0, dy=0.0):
    """A width x height window of the genome's frame at the same
    pixels_per_unit (and so the same samples per pixel at a given quality),
    its centre moved by (dx, dy) output pixels from the frame's centre
    (rows grow with y, rect.c:785-827)."""
    g = genome.g
    g.center[0] += dx / g.pixels_per_unit
    g.center[1] += dy / g.pixels_per_unit
    g.width = width
    g.height = height


VARIATIONS_0_19 = list(range(20))


def _render_params(g, width, height, quality, oversample, estimator, filter_radius):
    g.width = width
    g.height = height
    g.sample_density = quality
    g.spatial_oversample = oversample
    g.estimator = estimator
    g.estimator_minimum = 0.0
    g.estimator_curve = 0.4
    g.spatial_filter_radius = filter_radius
    g.spatial_filter_select = 0
    g.gamma = 4.0
    g.brightness = 4.0
    g.vibrancy = 1.0
    g.ntemporal_samples = 1
    g.nbatches = 1


def small_genome(seed=0, width=512, height=512, quality=50.0):
    """3 xforms, coefs U(-1,1), weights U(.2,1) normalised, color U(0,1),
    color_speed .5, linear .5 / sinusoidal .3 / spherical .2, 8-colour
    gradient palette; 512x512 q50 ss1, no DE, gaussian r=0.5, gamma 4,
    brightness 4, vibrancy 1, one temporal sample."""
    rng = np.random.default_rng(seed)
    G = Genome(3)
    w = rng.uniform(0.2, 1.0, 3)
    w /= w.sum()
    for i in range(3):
        x = G.xform(i)
        coefs = rng.uniform(-1, 1, 6)
        for k in range(6):
            x.c[k // 2][k % 2] = coefs[k]
        x.density = w[i]
        x.color = rng.uniform(0, 1)
        x.color_speed = 0.5
        for j in range(abi.NVARS):
            x.var[j] = 0.0
        x.var[0], x.var[1], x.var[2] = 0.5, 0.3, 0.2
    G.set_palette(random_palette(rng))
    _render_params(G.g, width, height, quality, 1, 0.0, 0.5)
    frame_camera(G, width, height, seed=seed + 1)
    return G


def random_genome(rng, nxforms, final=False, variations=VARIATIONS_0_19, coef_sigma=0.6):
    """Xforms with 2-4 variations drawn from `variations`, Dirichlet(1) weights,
    affine entries N(0, sigma^2), weights U(.2,1) normalised."""
    G = Genome(nxforms, final=final)
    w = rng.uniform(0.2, 1.0, nxforms)
    w /= w.sum()
    n = nxforms + (1 if final else 0)
    for i in range(n):
        x = G.xform(i)
        coefs = rng.normal(0.0, coef_sigma, 6)
        for k in range(6):
            x.c[k // 2][k % 2] = coefs[k]
        x.density = w[i] if i < nxforms else 0.0
        x.color = rng.uniform(0, 1)
        x.color_speed = 0.5
        for j in range(abi.NVARS):
            x.var[j] = 0.0
        k = int(rng.integers(2, 5))
        chosen = rng.choice(variations, size=k, replace=False)
        vw = rng.dirichlet(np.ones(k))
        for v, ww in zip(chosen, vw):
            x.var[int(v)] = float(ww)
    G.set_palette(random_palette(rng))
    return G


def still_genome(seed=1, width=1920, height=1080, quality=2000.0, oversample=2, estimator=9.0):
    """6 xforms + final, variations from 0-19, DE radius 9, gaussian r=1."""
    rng = np.random.default_rng(seed)
    G = random_genome(rng, 6, final=True)
    _render_params(G.g, width, height, quality, oversample, estimator, 1.0)
    frame_camera(G, width, height, seed=seed + 1)
    return G


def animation_keys(seed=2, width=1280, height=720, quality=500.0, temporal_samples=100, estimator=7.0):
    """Two 5-xform genomes at times 0 and 120 for an interpolated animation."""
    rng = np.random.default_rng(seed)
    out = []
    for t in (0.0, 120.0):
        G = random_genome(rng, 5)
        _render_params(G.g, width, height, quality, 1, estimator, 1.0)
        G.g.ntemporal_samples = temporal_samples
        G.g.time = t
        G.g.interpolation = 0
        G.g.interpolation_type = 1
        frame_camera(G, width, height, seed=int(seed + t))
        out.append(G)
    return out


MIXED_SIZES = [(256, 256), (512, 512), (1024, 768), (1920, 1080)]


def mixed_jobs(seed=3, njobs=256, quality_scale=1.0):
    """Mixed-size batch: 2-12 xforms, size from 4 choices, quality
    log-uniform [50,1000], supersample 1|2, DE radius 0-11, bits 33 (90%)
    or 64 (10%).  Returns a list of (Genome, bits)."""
    rng = np.random.default_rng(seed)
    jobs = []
    for _ in range(njobs):
        nx = int(rng.integers(2, 13))
        G = random_genome(rng, nx)
        w, h = MIXED_SIZES[int(rng.integers(0, 4))]
        q = float(math.exp(rng.uniform(math.log(50), math.log(1000)))) * quality_scale
        ss = int(rng.integers(1, 3))
        est = float(rng.integers(0, 12))
        _render_params(G.g, w, h, q, ss, est, 1.0)
        frame_camera(G, w, h, seed=int(rng.integers(0, 1 << 30)))
        bits = 64 if rng.uniform() < 0.1 else 33
        jobs.append((G, bits))
    return jobs


def serving_trace(seed=4, nrequests=64, rate_hz=4.0, quality_scale=1.0):
    """Poisson arrivals: 95% mixed-size jobs (as mixed_jobs), 5% 3840x2160 q1000 ss2 DE 11.
    Returns a list of (arrival_s, Genome, bits)."""
    rng = np.random.default_rng(seed)
    small = mixed_jobs(seed=seed + 100, njobs=nrequests, quality_scale=quality_scale)
    t = 0.0
    out = []
    for i in range(nrequests):
        t += float(rng.exponential(1.0 / rate_hz))
        if rng.uniform() < 0.05:
            G = random_genome(rng, int(rng.integers(2, 13)))
            _render_params(G.g, 3840, 2160, 1000.0 * quality_scale, 2, 11.0, 1.0)
            frame_camera(G, 3840, 2160, seed=i + 7)
            out.append((t, G, 33))
        else:
            G, bits = small[i]
            out.append((t, G, bits))
    return out
