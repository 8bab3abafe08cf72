"""The tile symbol coder (zf_ec_*) and the filter syntax as bytes, host code
through the C ABI (no GPU).

The bytes are read back with a restatement of the AV1 specification's
symbol decoder (8.2.2 init_symbol, 8.2.6 read_symbol with its CDF update,
read_bool, read_literal) and its restoration-unit and cdef syntax (5.11.57
read_lr, 5.11.58 read_lr_unit with decode_signed_subexp_with_ref_bool,
5.11.56 read_cdef): whatever the encoder writes, a conforming decoder must
read back the stage's decisions. The reference's own coder tests
(svtav1-entropy/src/range_coder.rs:311-383, writer.rs:85-121, cdf.rs:
98-150) supply the state anchors; the reference has no committed coded
bytes for these elements (its byte parity runs against a linked C library),
so the bytes are pinned by the normative decoder, not by reference vectors.
"""
import ctypes as C

import numpy as np
import pytest

from zenav1_svt_gb300 import abi, synth

from test_lr_syntax import c_reference, make_decisions

MIN = (-5, -23, -17)
MAX = (10, 8, 46)
K = (1, 2, 3)
MID = (3, -7, 15)


class SpecReader:
    """AV1 spec 8.2: the symbol decoder over one tile's bytes."""

    def __init__(self, data):
        self.data, self.bit = bytes(data), 0
        n = min(len(self.data) * 8, 15)
        self.value = ((1 << 15) - 1) ^ (self.f(n) << (15 - n))
        self.range = 1 << 15
        self.max_bits = 8 * len(self.data) - 15

    def f(self, n):
        v = 0
        for _ in range(n):
            byte = self.data[self.bit >> 3] if (self.bit >> 3) < len(self.data) else 0
            v = (v << 1) | ((byte >> (7 - (self.bit & 7))) & 1)
            self.bit += 1
        return v

    def symbol(self, cdf, adapt=True):
        """cdf: increasing Q15 CDF of N symbols (cdf[N-1] = 32768) plus the counter."""
        n = len(cdf) - 1
        cur, sym = self.range, -1
        while True:
            sym += 1
            prev = cur
            fq = (1 << 15) - cdf[sym]
            cur = ((self.range >> 8) * (fq >> 6) >> 1) + 4 * (n - sym - 1)
            if not self.value < cur:
                break
        self.range = prev - cur
        self.value -= cur
        bits = 15 - (self.range.bit_length() - 1)
        self.range <<= bits
        nb = min(bits, max(0, self.max_bits))
        self.value = (self.f(nb) << (bits - nb)) ^ (((self.value + 1) << bits) - 1)
        self.max_bits -= bits
        if adapt:
            rate = 3 + (cdf[n] > 15) + (cdf[n] > 31) + min(n.bit_length() - 1, 2)
            tmp = 0
            for i in range(n - 1):
                if i == sym:
                    tmp = 1 << 15
                if tmp < cdf[i]:
                    cdf[i] -= (cdf[i] - tmp) >> rate
                else:
                    cdf[i] += (tmp - cdf[i]) >> rate
            cdf[n] += int(cdf[n] < 32)
        return sym

    def bool(self):
        return self.symbol([1 << 14, 1 << 15, 0], adapt=False)

    def literal(self, n):
        v = 0
        for _ in range(n):
            v = (v << 1) | self.bool()
        return v

    # 4.10.7 ns(n) in tile data, and the subexponential reads of 5.11.58
    def ns(self, n):
        w = n.bit_length()
        m = (1 << w) - n
        v = self.literal(w - 1)
        return v if v < m else (v << 1) - m + self.literal(1)

    def subexp(self, num_syms, k):
        i = mk = 0
        while True:
            b2 = k + i - 1 if i else k
            a = 1 << b2
            if num_syms <= mk + 3 * a:
                return self.ns(num_syms - mk) + mk
            if self.literal(1):
                i += 1
                mk += a
            else:
                return self.literal(b2) + mk

    def signed_subexp_with_ref(self, low, high, k, r):
        mx, r = high - low, r - low
        v = self.subexp(mx, k)

        def inverse_recenter(r, v):
            if v > 2 * r:
                return v
            return r - ((v + 1) >> 1) if v & 1 else r + (v >> 1)

        x = inverse_recenter(r, v) if (r << 1) <= mx else mx - 1 - inverse_recenter(mx - 1 - r, v)
        return x + low


def inc_cdf(icdf):
    """C-layout inverse CDF -> the spec's increasing form (same counter)."""
    return [32768 - v for v in icdf[:-1]] + [icdf[-1]]


def random_icdf(rng, n):
    cuts = np.sort(rng.choice(np.arange(1, 32768), n - 1, replace=False))
    return (C.c_uint16 * (n + 1))(*([32768 - int(c) for c in cuts] + [0, 0]))


# -- the coder against the reference's anchors --------------------------------
def test_fresh_coder_state_and_empty_stream(pkg):
    ec = pkg.RangeCoder()
    assert ec.tell() == 1  # -9 + 10 + 0 * 8 (range_coder.rs:376-381)
    assert ec.done() == b"\x80"  # the terminating bit alone
    ec.bool(1)
    assert ec.tell() > 1


def test_binary_cdf_adapts_like_the_reference(pkg):
    ec = pkg.RangeCoder()
    cdf = (C.c_uint16 * 3)(16384, 0, 0)
    ec.symbol(0, cdf)  # writer.rs:112-120: symbol 0 lowers cdf[0]
    assert list(cdf) == [16384 - (16384 >> 4), 0, 1]
    ec.symbol(1, cdf)
    assert cdf[0] == 15360 + ((32768 - 15360) >> 4) and cdf[2] == 2
    four = (C.c_uint16 * 5)(24576, 16384, 8192, 0, 0)  # writer.rs:97-110
    for s in range(4):
        ec.symbol(s, four)
    assert four[4] == 4 and len(ec.done()) > 0


def test_about_one_bit_per_equiprobable_symbol(pkg):
    ec = pkg.RangeCoder()
    cdf = (C.c_uint16 * 3)(16384, 0, 0)
    for i in range(1000):
        ec.symbol(i & 1, cdf, adapt=False)  # range_coder.rs:339-352
    out = ec.done()
    assert 120 <= len(out) <= 130
    r = SpecReader(out)
    assert [r.symbol(inc_cdf(list(cdf)), adapt=False) for _ in range(1000)] == [i & 1 for i in range(1000)]


def test_arguments_rejected(pkg):
    ec = pkg.RangeCoder()
    with pytest.raises(pkg.ZfError):
        ec.bool(1, 0)
    with pytest.raises(pkg.ZfError):
        ec.symbol(2, (C.c_uint16 * 3)(16384, 0, 0))
    with pytest.raises(pkg.ZfError):
        ec.symbol(0, (C.c_uint16 * 3)(16384, 5, 0))  # icdf[nsyms - 1] must be 0
    with pytest.raises(pkg.ZfError):
        ec.literal(0, 33)
    assert ec.tell() == 1  # nothing was coded


@pytest.mark.parametrize("seed", range(6))
def test_random_streams_decode_with_the_spec_reader(pkg, seed):
    """Bools at any probability, literals, and adaptive symbols of 2..16
    values, long enough (and skewed enough) that carries ripple into bytes
    already written."""
    rng = np.random.default_rng(seed)
    ec = pkg.RangeCoder()
    cdfs = {n: random_icdf(rng, n) for n in range(2, 17)}
    spec_cdfs = {n: inc_cdf(list(c)) for n, c in cdfs.items()}
    ops = []
    for _ in range(3000):
        kind = rng.integers(0, 3)
        if kind == 0:
            f = int(rng.choice([1, 2, 100, 16384, 32000, 32767]))
            bit = int(rng.random() < f / 32768) if rng.random() < 0.9 else int(rng.integers(0, 2))
            ec.bool(bit, f)
            ops.append(("b", f, bit))
        elif kind == 1:
            nb = int(rng.integers(0, 17))
            v = int(rng.integers(0, 1 << nb)) if nb else 0
            ec.literal(v, nb)
            ops.append(("l", nb, v))
        else:
            n = int(rng.integers(2, 17))
            s = int(rng.integers(0, n)) if rng.random() < 0.5 else 0
            ec.symbol(s, cdfs[n])
            ops.append(("s", n, s))
        if len(ops) % 700 == 0:
            mid = ec.done()  # done() leaves the coder open
            assert len(mid) == (ec.tell() + 7) // 8
    data = ec.done()
    r = SpecReader(data)
    for op in ops:
        if op[0] == "b":
            fq = op[1]
            got = r.symbol([32768 - fq, 32768, 0], adapt=False)
        elif op[0] == "l":
            got = r.literal(op[1])
        else:
            got = r.symbol(spec_cdfs[op[1]])
        assert got == op[2], (op, ops.index(op))
    for n in cdfs:
        assert inc_cdf(list(cdfs[n])) == spec_cdfs[n]  # both sides adapted alike


# -- the filter syntax of a tile, coded and read back ---------------------------
def tile_walk(ec, dec, w, h, sb, rng, skip_prob=0.5, monochrome=False, sr_denom=0, coded_w=None):
    """Per superblock in raster order: the restoration units, then 32x32
    coded blocks in Z order, each a skip flag (a stand-in for the rest of the
    block's syntax) followed by cdef_idx where due. Returns the block list.
    With superres the superblocks walk the coded width; w is the upscaled
    width the restoration units live on."""
    sb_mi = sb // 4
    blocks = []
    cw = w if coded_w is None else coded_w
    for sr in range(0, (h + sb - 1) // sb):
        for sc in range(0, (cw + sb - 1) // sb):
            ec.lr_sb(dec, sr * sb_mi, sc * sb_mi, sb_mi, w, h, monochrome, sr_denom)
            st = ec.cdef_sb(dec, sr, sc, sb)
            for q in range((sb // 64) ** 2):
                qx, qy = sc * sb + (q & 1) * 64, sr * sb + (q >> 1) * 64
                for b in range(4):
                    bx, by = qx + (b & 1) * 32, qy + (b >> 1) * 32
                    if bx >= cw or by >= h:
                        continue
                    skip = int(rng.random() < skip_prob)
                    ec.bool(skip)
                    ec.cdef_block(st, bx, by, skip)
                    blocks.append((sr, sc, bx, by, skip))
    return blocks


def read_tile(data, dec_planes, nhfb, cdef_bits, w, h, sb, blocks, monochrome=False, sr_denom=0):
    """The decoder's side of tile_walk (spec read_lr per superblock, then per
    block the skip flag and read_cdef)."""
    r = SpecReader(data)
    use_wiener = [11570, 32768, 0]
    ref = {p: [list(MID), list(MID)] for p in range(3)}
    units = {}
    sb_mi = sb // 4
    fb = {}
    last_sb = None
    for sr, sc, bx, by, skip in blocks:
        if (sr, sc) != last_sb:
            last_sb = (sr, sc)
            for p in range(1 if monochrome else 3):
                plane = dec_planes[p]
                if plane["frame_rtype"] == 0:
                    continue
                cr = c_reference(plane["unit_size"], p > 0, sr * sb_mi, sc * sb_mi, sb_mi, w, h, sr_denom)
                if cr is None:
                    continue
                for rrow in range(cr[2], cr[3]):
                    for rcol in range(cr[0], cr[1]):
                        u = rcol + rrow * plane["hunits"]
                        use = r.symbol(use_wiener)
                        taps = None
                        if use:
                            taps = []
                            for pas in range(2):
                                coeffs = [0, 0, 0]
                                for j in range(1 if p else 0, 3):
                                    v = r.signed_subexp_with_ref(MIN[j], MAX[j] + 1, K[j], ref[p][pas][j])
                                    coeffs[j] = ref[p][pas][j] = v
                                taps.append(coeffs)
                        units[(p, u)] = (use, taps)
            cdef_seen = {}
        assert r.bool() == skip, "skip flag misread at block %s" % ((bx, by),)
        key = (by >> 6, bx >> 6)
        if not skip and cdef_bits and key not in cdef_seen:
            cdef_seen[key] = r.literal(cdef_bits)
            fb[key] = cdef_seen[key]
    return units, fb


def plane_info(dec):
    return [{"frame_rtype": dec.lr[p].frame_rtype, "unit_size": dec.lr[p].unit_size, "hunits": dec.lr[p].hunits}
            for p in range(3)]


def check_units(units, dec):
    assert units, "no restoration unit was coded"
    for (p, u), (use, taps) in units.items():
        unit = dec.lr_units[p][u]
        assert use == (unit.rtype != 0), (p, u)
        if use:
            for pas, f in ((0, unit.vfilter), (1, unit.hfilter)):
                assert taps[pas] == [f[0], f[1], f[2]], (p, u, pas, taps[pas], list(f)[:3])


@pytest.mark.parametrize("w,h,sb", [(1000, 600, 64), (777, 521, 128), (200, 90, 64)])
def test_restoration_units_read_back(pkg, w, h, sb):
    rng = np.random.default_rng(w + h)
    dec, keep = make_decisions(rng, w, h, luma_win=5 if sb == 64 else 7)
    ec = pkg.RangeCoder()
    blocks = tile_walk(ec, dec, w, h, sb, rng)
    units, _ = read_tile(ec.done(), plane_info(dec), 0, 0, w, h, sb, blocks)
    check_units(units, dec)
    assert len(units) == sum(dec.lr[p].hunits * dec.lr[p].vunits for p in range(3))


def test_monochrome_and_superres_units_read_back(pkg):
    """Monochrome: luma units only. Superres (denominators 9, 12, 16): the
    superblocks walk the coded width while the units live on the upscaled
    one, so a superblock holds the corners that corners_in_sb remaps."""
    rng = np.random.default_rng(5)
    dec, keep = make_decisions(rng, 1000, 600)
    ec = pkg.RangeCoder()
    blocks = tile_walk(ec, dec, 1000, 600, 64, rng, monochrome=True)
    units, _ = read_tile(ec.done(), plane_info(dec), 0, 0, 1000, 600, 64, blocks, monochrome=True)
    check_units(units, dec)
    assert {p for p, _ in units} == {0} and len(units) == dec.lr[0].hunits * dec.lr[0].vunits
    for denom in (9, 12, 16):
        w, h = 1024, 512
        coded = pkg.lib().zf_superres_scaled_size(w, denom)
        assert 0 < coded < w
        dec, keep = make_decisions(rng, w, h)
        ec = pkg.RangeCoder()
        blocks = tile_walk(ec, dec, w, h, 64, rng, sr_denom=denom, coded_w=coded)
        units, _ = read_tile(ec.done(), plane_info(dec), 0, 0, w, h, 64, blocks, sr_denom=denom)
        check_units(units, dec)
        assert len(units) == sum(dec.lr[p].hunits * dec.lr[p].vunits for p in range(3)), denom


FRAMES = [
    ("p2_lr_mixed", (11, 512, 384, 8, 20, 2, "cosine"), 64),
    ("p2_bits3_sb128", (11, 768, 512, 8, 30, 2, "cosine"), 128),
    ("bd10_odd_plane_none", (12, 331, 203, 10, 36, 2, "cosine"), 64),
]


@pytest.mark.parametrize("case", FRAMES, ids=[c[0] for c in FRAMES])
def test_stage_decisions_read_back(pkg, oracle, case):
    """The stage's own decisions (the oracle's, which the GPU path matches
    bit for bit) coded into a tile and read back by the spec decoder: every
    unit's flag and taps, every filter block's cdef_idx."""
    name, args, sb = case
    cfg, w, h, bd, qp, preset, content = args
    fr = synth.make_frame(synth.frame_seed(cfg, w + qp * 7 + preset), w, h, bd, qp, preset, content)
    d = oracle.stage_decisions(fr)
    dec = d.c
    assert dec.cdef_bits > 0
    rng = np.random.default_rng(len(name))
    ec = pkg.RangeCoder()
    blocks = tile_walk(ec, dec, fr.true_w, fr.true_h, sb, rng, skip_prob=0.3)
    units, fb = read_tile(ec.done(), plane_info(dec), dec.nhfb, dec.cdef_bits, fr.true_w, fr.true_h, sb, blocks)
    assert fb and all(v == d.fb_idx[r * dec.nhfb + c] for (r, c), v in fb.items())
    coded_fbs = {(by >> 6, bx >> 6) for _, _, bx, by, skip in blocks if not skip}
    assert set(fb) == coded_fbs  # one literal per filter block with a coded non-skip block
    if any(dec.lr[p].frame_rtype for p in range(3)):
        check_units(units, dec)


def test_cdef_literal_placement(pkg):
    """A 128x128 superblock: each 64x64 quadrant's first non-skip block codes
    its index, later blocks and skipped blocks code nothing."""
    d = abi.Decisions(256, 128, 256, 128)
    d.c.cdef_bits = 2
    d.c.nhfb, d.c.nvfb = 4, 2
    d.fb_idx[:] = [1, 2, 3, 0, 2, 3, 1, 1]
    ec = pkg.RangeCoder()
    st = ec.cdef_sb(d.c, 0, 1, 128)  # fbs (0,2), (0,3), (1,2), (1,3)
    assert list(st.strengths) == [3, 0, 1, 1] and st.sb128 == 1
    assert ec.cdef_block(st, 128, 0, 1) == 0  # skip
    assert ec.cdef_block(st, 160, 0, 0) == 2
    assert ec.cdef_block(st, 128, 32, 0) == 0  # same quadrant: already sent
    assert ec.cdef_block(st, 192, 64, 0) == 2
    assert list(st.transmitted) == [1, 0, 0, 1]
    d.c.cdef_bits = 0
    st0 = ec.cdef_sb(d.c, 0, 0, 64)
    assert ec.cdef_block(st0, 0, 0, 0) == 0
