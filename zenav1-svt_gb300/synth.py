"""Seeded synthetic inputs for the filter stage.

The reference measures the encoder on image corpora that are not available
here; these generators stand in for them with the shapes, sizes and value
distributions of the benchmark workloads (source planes), plus the stage
inputs the encoder's mode decision would have produced upstream of the
filters: a per-4x4 block/transform geometry (the DeblockGeom the entropy walk
records, svtav1-encoder/src/deblock.rs:532-679) and a pre-deblock recon.

The geometry is a random AV1 partition of each 64x64 superblock: NONE /
HORZ / VERT / SPLIT down to 4x4, blocks that cross the canvas edge are split
(as AV1 forces), so every block and transform is aligned to its own
dimensions. The recon is source + a constant per-transform offset
U[-q/8, q/8] + Gaussian noise sigma q/16 (q = the AC quantizer step at the
frame's qindex, on the 8-bit scale), clamped; skipped blocks get the offset
only.
"""
import math

import numpy as np

SEED_BASE = 0xF117E5


def frame_seed(cfg, idx):
    return (SEED_BASE ^ (cfg << 32) ^ idx) & ((1 << 63) - 1)


def align8(v):
    return (v + 7) & ~7


# --------------------------------------------------------------------------
# Source content
# --------------------------------------------------------------------------

def _cosines(rng, h, w, n, amp, pmin=16.0, pmax=256.0):
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    out = np.zeros((h, w))
    for _ in range(n):
        period = rng.uniform(pmin, pmax)
        theta = rng.uniform(0, 2 * math.pi)
        phase = rng.uniform(0, 2 * math.pi)
        kx, ky = math.cos(theta) / period, math.sin(theta) / period
        out += amp * np.cos(2 * math.pi * (kx * xx + ky * yy) + phase)
    return out


def _rects(rng, img, n, offset, ellipses=False):
    h, w = img.shape
    for i in range(n):
        rw = int(rng.integers(4, max(5, w // 4)))
        rh = int(rng.integers(4, max(5, h // 4)))
        x0 = int(rng.integers(0, max(1, w - rw)))
        y0 = int(rng.integers(0, max(1, h - rh)))
        d = rng.uniform(-offset, offset)
        if ellipses and i % 2 == 1:
            yy, xx = np.mgrid[0:rh, 0:rw]
            m = ((xx - rw / 2 + 0.5) / (rw / 2)) ** 2 + ((yy - rh / 2 + 0.5) / (rh / 2)) ** 2 <= 1.0
            img[y0:y0 + rh, x0:x0 + rw][m] += d
        else:
            img[y0:y0 + rh, x0:x0 + rw] += d


def _power_field(rng, h, w, beta, sigma):
    """Gaussian field with a 1/f^beta power spectrum, scaled to sigma."""
    noise = rng.standard_normal((h, w))
    f = np.fft.rfft2(noise)
    fy = np.fft.fftfreq(h)[:, None]
    fx = np.fft.rfftfreq(w)[None, :]
    r = np.sqrt(fx * fx + fy * fy)
    r[0, 0] = 1.0
    f *= r ** (-beta / 2.0)
    f[0, 0] = 0.0
    field = np.fft.irfft2(f, s=(h, w))
    field *= sigma / max(field.std(), 1e-9)
    return field


def content_cosine_rects(rng, w, h, bd):
    """Cosines + rectangles + noise (the 512x512 plain drop-in content)."""
    s = 1 << (bd - 8)
    y = 128.0 * s + _cosines(rng, h, w, 3, 40.0 * s)
    _rects(rng, y, 12, 60.0 * s)
    y += rng.normal(0, 4.0 * s, size=y.shape)
    cw, ch = w // 2, h // 2
    u = 128.0 * s + _cosines(rng, ch, cw, 2, 20.0 * s, 8.0, 128.0)
    v = 128.0 * s + _cosines(rng, ch, cw, 2, 20.0 * s, 8.0, 128.0)
    return y, u, v


def content_power(rng, w, h, bd, beta_y=2.0, sig_y=35.0, mean_y=120.0, shapes=200, noise=3.0,
                  sig_c=12.0, mean_c=128.0):
    """1/f^beta field + shapes + noise (the 4K and 10-bit content)."""
    y = mean_y + _power_field(rng, h, w, beta_y, sig_y)
    if shapes:
        _rects(rng, y, shapes, 60.0 * (1 << (bd - 8)), ellipses=True)
    y += rng.normal(0, noise, size=y.shape)
    cw, ch = w // 2, h // 2
    u = mean_c + _power_field(rng, ch, cw, 2.0, sig_c)
    v = mean_c + _power_field(rng, ch, cw, 2.0, sig_c)
    return y, u, v


def _to_plane(a, bd):
    hi = (1 << bd) - 1
    a = np.clip(np.rint(a), 0, hi)
    return a.astype(np.uint8 if bd == 8 else np.uint16)


# --------------------------------------------------------------------------
# Geometry (DeblockGeom arrays) and recon
# --------------------------------------------------------------------------

class Geometry:
    """Explicit per-mi arrays in the reference's DeblockGeom layout."""

    def __init__(self, w, h):
        self.mi_cols, self.mi_rows = w // 4, h // 4
        n = (self.mi_rows, self.mi_cols)
        self.block_id = np.full(n, 0xFFFFFFFF, np.uint32)
        self.bw = np.zeros(n, np.uint8)
        self.bh = np.zeros(n, np.uint8)
        self.tw = np.zeros(n, np.uint8)
        self.th = np.zeros(n, np.uint8)
        self.skip = np.zeros(n, np.uint8)
        self.skip_inter = np.zeros(n, np.uint8)

    def record_block(self, x, y, bw, bh, skip, tx_depth):
        mx0, my0 = x // 4, y // 4
        mx1, my1 = min((x + bw) // 4, self.mi_cols), min((y + bh) // 4, self.mi_rows)
        sl = (slice(my0, my1), slice(mx0, mx1))
        self.block_id[sl] = my0 * self.mi_cols + mx0
        self.bw[sl] = bw
        self.bh[sl] = bh
        if tx_depth == 0:
            tw, th = bw, bh
        else:
            side = max(min(bw, bh) if bw != bh else bw // 2, 4)
            tw = th = side
        self.tw[sl] = min(tw, 64)
        self.th[sl] = min(th, 64)
        self.skip[sl] = 1 if skip else 0
        self.skip_inter[sl] = 0  # all-intra: skip_inter == skip && is_inter == false

    def arrays(self):
        return [np.ascontiguousarray(a.reshape(-1)) for a in
                (self.block_id, self.bw, self.bh, self.tw, self.th, self.skip, self.skip_inter)]


def random_geometry(rng, w, h, qp, sb=64, skip_prob=None):
    g = Geometry(w, h)
    t = min(max((qp - 20) / 40.0, 0.0), 1.0)
    p_skip = skip_prob if skip_prob is not None else min(max((qp - 20) / 40.0, 0.05), 0.8)
    p_split = {128: 0.95, 64: 0.85 - 0.3 * t, 32: 0.6 - 0.3 * t, 16: 0.45 - 0.25 * t, 8: 0.25 - 0.15 * t}

    def part(x, y, s):
        if x >= w or y >= h:
            return
        inside = x + s <= w and y + s <= h
        if s > 4 and (not inside or rng.random() < p_split.get(s, 0.0)):
            hs = s // 2
            for dy in (0, hs):
                for dx in (0, hs):
                    part(x + dx, y + dy, hs)
            return
        r = rng.random()
        depth = int(rng.random() < 0.35) if s > 4 else 0
        if s >= 8 and r < 0.15:  # HORZ
            for dy in (0, s // 2):
                g.record_block(x, y + dy, s, s // 2, rng.random() < p_skip, depth)
        elif s >= 8 and r < 0.30:  # VERT
            for dx in (0, s // 2):
                g.record_block(x + dx, y, s // 2, s, rng.random() < p_skip, depth)
        else:
            g.record_block(x, y, s, s, rng.random() < p_skip, depth)

    for y in range(0, h, sb):
        for x in range(0, w, sb):
            part(x, y, sb)
    assert (g.block_id != 0xFFFFFFFF).all()
    return g


def synth_recon(rng, src, geom, qindex, bd, plane):
    """src + per-TX offset + noise, clamped. plane 0 uses the luma TX grid,
    chroma planes the 4:2:0 chroma TX of each block."""
    from_tab = AC_QLOOKUP_8 if bd == 8 else AC_QLOOKUP_10
    q = from_tab[qindex] >> (bd - 8)
    scale = 1 << (bd - 8)
    h, w = src.shape
    mi_rows, mi_cols = geom.mi_rows, geom.mi_cols
    my, mx = np.mgrid[0:mi_rows, 0:mi_cols]
    if plane == 0:
        tw = (geom.tw.astype(np.int64) // 4)
        th = (geom.th.astype(np.int64) // 4)
        ox, oy = mx & ~(tw - 1), my & ~(th - 1)
    else:
        cw = np.maximum(geom.bw.astype(np.int64) // 8, 1) * 2
        chh = np.maximum(geom.bh.astype(np.int64) // 8, 1) * 2
        ox, oy = mx & ~(cw - 1), my & ~(chh - 1)
    tx_id = oy * mi_cols + ox
    off_tab = rng.integers(-(q // 8), q // 8 + 1, size=mi_rows * mi_cols) * scale
    off_mi = off_tab[tx_id]
    skip_mi = geom.skip.astype(bool)
    if plane == 0:
        off = np.repeat(np.repeat(off_mi, 4, 0), 4, 1)[:h, :w]
        skp = np.repeat(np.repeat(skip_mi, 4, 0), 4, 1)[:h, :w]
    else:
        off = np.repeat(np.repeat(off_mi, 2, 0), 2, 1)[:h, :w]
        skp = np.repeat(np.repeat(skip_mi, 2, 0), 2, 1)[:h, :w]
    noise = rng.normal(0, max(q / 16.0, 0.5) * scale, size=src.shape)
    noise[skp] = 0
    rec = src.astype(np.float64) + off + noise
    return _to_plane(rec, bd)


def _tx_blocks(geom, plane):
    """Transform blocks of a plane as (origin y, origin x, height, width)
    arrays in that plane's samples: the luma TX grid for plane 0, the 4:2:0
    chroma TX of each block (max(bw/2, 4) x max(bh/2, 4)) for planes 1, 2."""
    mi_rows, mi_cols = geom.mi_rows, geom.mi_cols
    my, mx = np.mgrid[0:mi_rows, 0:mi_cols]
    if plane == 0:
        tw = geom.tw.astype(np.int64) // 4
        th = geom.th.astype(np.int64) // 4
        px = 4
    else:
        tw = np.maximum(geom.bw.astype(np.int64) // 8, 1) * 2
        th = np.maximum(geom.bh.astype(np.int64) // 8, 1) * 2
        px = 2
    ox, oy = mx & ~(tw - 1), my & ~(th - 1)
    first = (mx == ox) & (my == oy)
    return oy[first] * px, ox[first] * px, th[first] * px, tw[first] * px, first


def synth_recon_quant(rng, src, geom, qindex, bd, plane):
    """Quantised-transform recon: every transform block of the plane is
    replaced by the inverse 2-D DCT of its quantised orthonormal DCT
    (step = AC quantiser / 8, on the plane's own bit-depth scale, rounding
    with a small dead zone). Skipped blocks keep only their quantised DC (a
    flat block, as an all-zero residual on a DC prediction gives). This is
    the blocky, band-limited recon the deblock level search and CDEF exist
    for: filtering it lowers the error against the source."""
    from scipy.fft import dctn, idctn
    tab = AC_QLOOKUP_8 if bd == 8 else AC_QLOOKUP_10
    step = max(tab[qindex] / 8.0, 1.0)
    h, w = src.shape
    base = src.astype(np.float64)
    out = base.copy()
    y0, x0, bh, bw, first = _tx_blocks(geom, plane)
    skip_first = geom.skip.astype(bool)[first]
    shapes = {}
    for i in range(len(y0)):
        shapes.setdefault((int(bh[i]), int(bw[i])), []).append(i)
    for (th, tw), idx in shapes.items():
        idx = np.asarray(idx)
        yy = y0[idx][:, None, None] + np.arange(th)[None, :, None]
        xx = x0[idx][:, None, None] + np.arange(tw)[None, None, :]
        yy, xx = np.broadcast_arrays(yy, xx)
        ok = (yy < h) & (xx < w)
        yy, xx = np.minimum(yy, h - 1), np.minimum(xx, w - 1)
        blk = base[yy, xx]
        c = dctn(blk, type=2, norm="ortho", axes=(1, 2))
        q = np.sign(c) * np.floor(np.abs(c) / step + 0.35)
        sk = skip_first[idx]
        q[sk, :, :] = np.where(np.arange(th)[:, None] + np.arange(tw)[None, :] == 0, q[sk, :, :], 0.0)
        rec = idctn(q * step, type=2, norm="ortho", axes=(1, 2))
        out[yy[ok], xx[ok]] = rec[ok]
    return _to_plane(out, bd)


AC_QLOOKUP_8 = None
AC_QLOOKUP_10 = None


def _load_tables():
    global AC_QLOOKUP_8, AC_QLOOKUP_10
    if AC_QLOOKUP_8 is not None:
        return
    import os
    import re
    here = os.path.dirname(os.path.abspath(__file__))
    hdr = open(os.path.join(here, "..", "include", "zf_av1_tables.h")).read()

    def tab(name):
        i = hdr.index(name)
        body = hdr[hdr.index("{", i) + 1:hdr.index("};", i)]
        return [int(x) for x in re.findall(r"-?\d+", body)]
    AC_QLOOKUP_8 = tab("zf_ac_qlookup_8")
    AC_QLOOKUP_10 = tab("zf_ac_qlookup_10")


class Frame:
    """One frame's stage inputs: planes (numpy), geometry and parameters."""

    def __init__(self, bd, true_w, true_h, src, rec, geom, qindex, preset, chroma=True,
                 sharpness=0, sc_class5=0, enable_restoration=1):
        self.bd = bd
        self.true_w, self.true_h = true_w, true_h
        self.w, self.h = src[0].shape[1], src[0].shape[0]
        self.src = src
        self.rec = rec
        self.geom = geom
        self.qindex = qindex
        self.preset = preset
        self.chroma = chroma
        self.sharpness = sharpness
        self.sc_class5 = sc_class5
        self.enable_restoration = enable_restoration

    @property
    def luma_px(self):
        return self.true_w * self.true_h

    def copy_rec(self):
        return [r.copy() for r in self.rec]


def qp_to_qindex(qp):
    """CLI qp (0..63) -> qindex (svtav1-encoder/src/rate_control.rs:129-141)."""
    qp = min(max(int(qp), 0), 63)
    if qp <= 61:
        return 4 * qp
    return 249 if qp == 62 else 255


def make_frame(seed, true_w, true_h, bd, qp, preset, content="cosine", chroma=True, skip_prob=None,
               recon="quant"):
    """One frame's stage inputs. recon: "quant" (quantised-transform recon,
    synth_recon_quant) or "offset" (source + per-TX offset + noise,
    synth_recon)."""
    _load_tables()
    rng = np.random.default_rng(seed)
    w, h = align8(true_w), align8(true_h)
    if content == "cosine":
        y, u, v = content_cosine_rects(rng, w, h, bd)
    elif content == "power":
        y, u, v = content_power(rng, w, h, bd)
    elif content == "power10":
        y, u, v = content_power(rng, w, h, bd, beta_y=1.8, sig_y=140.0, mean_y=512.0, shapes=0,
                                noise=8.0, sig_c=48.0, mean_c=512.0)
    elif content == "flat":
        y = np.full((h, w), 100.0 * (1 << (bd - 8)))
        u = np.full((h // 2, w // 2), 128.0 * (1 << (bd - 8)))
        v = u.copy()
    else:
        raise ValueError(content)
    src = [_to_plane(y, bd), _to_plane(u, bd), _to_plane(v, bd)]
    qindex = qp_to_qindex(qp)
    geom = random_geometry(rng, w, h, qp, skip_prob=skip_prob)
    if recon == "quant":
        rec = [synth_recon_quant(rng, src[p], geom, qindex, bd, p) for p in range(3)]
    elif recon == "offset":
        rec = [synth_recon(rng, src[p], geom, qindex, bd, p) for p in range(3)]
    else:
        raise ValueError(recon)
    if not chroma:
        src = [src[0], np.zeros((h // 2, w // 2), src[0].dtype), np.zeros((h // 2, w // 2), src[0].dtype)]
        rec = [rec[0], np.zeros_like(src[1]), np.zeros_like(src[2])]
    return Frame(bd, true_w, true_h, src, rec, geom, qindex, preset, chroma=chroma)


# --------------------------------------------------------------------------
# The benchmark workloads
# --------------------------------------------------------------------------

def workload_plain_512(idx=0):
    """512x512 8-bit 4:2:0, qp 32, preset 6."""
    return make_frame(frame_seed(1, idx), 512, 512, 8, 32, 6, "cosine")


def workload_4k(preset, qp, idx=0):
    """3840x2160 8-bit 4:2:0 at preset 4 or 6, qp 24 or 40."""
    return make_frame(frame_seed(2, idx * 16 + preset * 2 + (qp > 30)), 3840, 2160, 8, qp, preset, "power")


def workload_10bit_4096(idx=0):
    """4096x3072 10-bit 4:2:0, preset 2, qp 28."""
    return make_frame(frame_seed(3, idx), 4096, 3072, 10, 28, 2, "power10")


def batch_specs(n=256, seed_cfg=4, max_dim=2048):
    """(w, h, bd, qp) for the mixed batch: W,H ~ U[64, max_dim], about 20%
    odd, 70% 8-bit / 30% 10-bit, qp ~ U[20, 50], preset 6."""
    rng = np.random.default_rng(frame_seed(seed_cfg, 0xBA7C))
    specs = []
    for i in range(n):
        w = int(rng.integers(64, max_dim + 1))
        h = int(rng.integers(64, max_dim + 1))
        if rng.random() < 0.2:
            w |= 1
        else:
            w &= ~1
        if rng.random() < 0.2:
            h |= 1
        else:
            h &= ~1
        w, h = max(w, 64), max(h, 64)
        bd = 10 if rng.random() < 0.3 else 8
        qp = int(rng.integers(20, 51))
        specs.append((w, h, bd, qp))
    return specs


def batch_frame(i, spec):
    """Image i of the mixed batch with its (w, h, bd, qp) spec."""
    w, h, bd, qp = spec
    return make_frame(frame_seed(4, i), w, h, bd, qp, 6, "cosine")


def workload_batch(n=256, max_dim=2048):
    return [batch_frame(i, sp) for i, sp in enumerate(batch_specs(n, max_dim=max_dim))]


def served_specs(n=32, seed_cfg=5, max_w=6000, max_h=4000, min_dim=128):
    """(w, h, bd, qp) for served requests: sizes log-uniform from
    min_dim^2 to max_w x max_h, 80% 8-bit / 20% 10-bit, qp ~ U[18, 45],
    preset 6."""
    rng = np.random.default_rng(frame_seed(seed_cfg, 0x5E4E))
    specs = []
    for _ in range(n):
        w = int(round(np.exp(rng.uniform(np.log(min_dim), np.log(max_w)))))
        h = int(round(np.exp(rng.uniform(np.log(min_dim), np.log(max_h)))))
        bd = 10 if rng.random() < 0.2 else 8
        qp = int(rng.integers(18, 46))
        specs.append((w, h, bd, qp))
    return specs


def poisson_arrivals(rate, seconds, seed):
    """Arrival offsets (s) of a Poisson process of `rate` per second."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds:
            return out
        out.append(t)
