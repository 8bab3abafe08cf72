"""Per-superblock restoration syntax (zf_lr_corners_in_sb, zf_lr_sb_syntax),
host code through the C ABI (no GPU).

corners_in_sb is held to the formula the reference's own test restates
from C (svtav1-encoder/src/restoration.rs:1244-1320: unit sizes 64/128/256,
upscaled widths 128/256/512, superres denominators none/9/12/16, both plane
kinds, every 64-px superblock, mi rows 0/16/32) plus its anti-vacuity check
(denominator 16 remaps at least one superblock). The symbol stream is held
to a restatement of write_primitive_quniform / _subexpfin / _refsubexpfin
(svtav1-entropy/src/lr.rs:67-145) and write_wiener_filter (:154-236), and
its bit count per unit to the oracle's count_wiener_bits (the figure the
search's RD uses, itself pinned to C captures)."""
import ctypes as C

import numpy as np
import pytest

from zenav1_svt_gb300 import abi, lib

MIN = (-5, -23, -17)
MAX = (10, 8, 46)
K = (1, 2, 3)
DEFAULT = (3, -7, 15, -22, 15, -7, 3, 0)


def count_units(unit, size):
    return max((size + (unit >> 1)) // unit, 1)


def c_reference(unit_size, is_uv, mi_row, mi_col, sb_mi, upscaled_w, frame_h, denom):
    ss = 1 if is_uv else 0
    tile_w, tile_h = (upscaled_w + ss) >> ss, (frame_h + ss) >> ss
    horz, vert = count_units(unit_size, tile_w), count_units(unit_size, tile_h)
    mi_size = 4 >> ss
    mi_to_num_x = mi_size * denom if denom else mi_size
    denom_x = unit_size * 8 if denom else unit_size
    rnd_x, rnd_y = denom_x - 1, unit_size - 1
    rcol0 = (mi_col * mi_to_num_x + rnd_x) // denom_x
    rrow0 = (mi_row * mi_size + rnd_y) // unit_size
    rcol1 = min(((mi_col + sb_mi) * mi_to_num_x + rnd_x) // denom_x, horz)
    rrow1 = min(((mi_row + sb_mi) * mi_size + rnd_y) // unit_size, vert)
    return (rcol0, rcol1, rrow0, rrow1) if rcol0 < rcol1 and rrow0 < rrow1 else None


def corners(unit_size, is_uv, mi_row, mi_col, sb_mi, w, h, denom):
    out = (C.c_int32 * 4)()
    rc = lib().zf_lr_corners_in_sb(unit_size, int(is_uv), mi_row, mi_col, sb_mi, w, h, denom, out)
    assert rc in (0, 1)
    return tuple(out) if rc else None


def test_corners_match_the_c_formula_across_superres():
    n = 0
    for unit_size in (64, 128, 256):
        for w in (128, 256, 512):
            for denom in (0, 9, 12, 16):
                for is_uv in (False, True):
                    for sb in range(w // 64):
                        for mi_row in (0, 16, 32):
                            args = (unit_size, is_uv, mi_row, sb * 16, 16, w, 128, denom)
                            assert corners(*args) == c_reference(*args), args
                            n += 1
    assert n == 3 * (2 + 4 + 8) * 4 * 2 * 3


def test_superres_remaps_some_superblock():
    diff = sum(corners(64, False, 0, sb * 16, 16, 512, 128, 0) != corners(64, False, 0, sb * 16, 16, 512, 128, 16)
               for sb in range(8))
    assert diff > 0


def test_corners_reject_bad_arguments():
    out = (C.c_int32 * 4)()
    L = lib()
    assert L.zf_lr_corners_in_sb(100, 0, 0, 0, 16, 64, 64, 0, out) == -6
    assert L.zf_lr_corners_in_sb(64, 0, 0, 0, 16, 64, 64, 8, out) == -6
    assert L.zf_lr_corners_in_sb(64, 0, 0, 0, 0, 64, 64, 0, out) == -6


# -- restatement of the tap coding (lr.rs:40-236) -----------------------------
def recenter_nonneg(r, v):
    if v > (r << 1):
        return v
    if v >= r:
        return (v - r) << 1
    return ((r - v) << 1) - 1


def recenter_finite_nonneg(n, r, v):
    if (r << 1) <= n:
        return recenter_nonneg(r, v)
    return recenter_nonneg(n - 1 - r, n - 1 - v)


def quniform(out, n, v):
    if n <= 1:
        return
    l = (n - 1).bit_length()
    m = (1 << l) - n
    if v < m:
        if l - 1:
            out.append((l - 1, v))
    else:
        if l - 1:
            out.append((l - 1, m + ((v - m) >> 1)))
        out.append((1, (v - m) & 1))


def subexpfin(out, n, k, v):
    i = mk = 0
    while True:
        b = k + i - 1 if i else k
        a = 1 << b
        if n <= mk + 3 * a:
            quniform(out, n - mk, v - mk)
            return
        t = v >= mk + a
        out.append((1, int(t)))
        if not t:
            if b:
                out.append((b, v - mk))
            return
        i += 1
        mk += a


def wiener_bits(win, vf, hf, rvf, rhf):
    out = []
    for f, rf in ((vf, rvf), (hf, rhf)):
        for idx in ((0, 1, 2) if win == 7 else (1, 2)):
            n = MAX[idx] - MIN[idx] + 1
            subexpfin(out, n, K[idx], recenter_finite_nonneg(n, rf[idx] - MIN[idx], f[idx] - MIN[idx]))
    return out


def sym_taps(rng, win):
    t = [int(rng.integers(MIN[i], MAX[i] + 1)) for i in range(3)]
    if win == 5:
        t[0] = 0
    return [t[0], t[1], t[2], -2 * (t[0] + t[1] + t[2]), t[2], t[1], t[0], 0]


def make_decisions(rng, w, h, luma_win=5, rtypes=(1, 1, 1)):
    d = abi.ZfDecisions()
    keep = []
    for p in range(3):
        ss = 1 if p else 0
        pw, ph = (w + ss) >> ss, (h + ss) >> ss
        hu, vu = count_units(256, pw), count_units(256, ph)
        d.lr[p].frame_rtype, d.lr[p].unit_size, d.lr[p].hunits, d.lr[p].vunits = rtypes[p], 256, hu, vu
        units = (abi.ZfLrUnit * (hu * vu))()
        for u in range(hu * vu):
            units[u].rtype = int(rng.random() < 0.7)
            win = luma_win if p == 0 else 5
            units[u].vfilter[:] = sym_taps(rng, win)
            units[u].hfilter[:] = sym_taps(rng, win)
        keep.append(units)
        d.lr_units[p] = C.cast(units, C.POINTER(abi.ZfLrUnit))
    return d, keep


def walk(d, w, h, sb=64, monochrome=0):
    refs = abi.ZfWienerRefs()
    lib().zf_wiener_refs_reset(C.byref(refs))
    out = (abi.ZfLrSym * 4096)()
    syms = []
    sb_mi = sb // 4
    for mi_row in range(0, (h + 3) // 4, sb_mi):
        for mi_col in range(0, (w + 3) // 4, sb_mi):
            n = lib().zf_lr_sb_syntax(C.byref(d), mi_row, mi_col, sb_mi, w, h, monochrome, 0, C.byref(refs), out,
                                      4096)
            assert n >= 0
            syms += [(s.kind, s.nbits, s.value, s.plane, s.unit) for s in out[:n]]
    return syms, refs


@pytest.mark.parametrize("w,h,luma_win,sb", [(1000, 600, 5, 64), (777, 521, 7, 64), (1300, 900, 5, 128),
                                             (200, 90, 5, 64)])
def test_symbol_stream_matches_the_restatement(oracle, w, h, luma_win, sb):
    rng = np.random.default_rng(w * 7 + h)
    d, keep = make_decisions(rng, w, h, luma_win)
    syms, refs = walk(d, w, h, sb)
    # every unit of every plane codes its flag exactly once
    flags = [(p, u) for k, _, _, p, u in syms if k == abi.SYM_WIENER_RESTORE]
    want = sorted((p, u) for p in range(3) for u in range(d.lr[p].hunits * d.lr[p].vunits))
    assert sorted(flags) == want and len(set(flags)) == len(flags)
    # per unit: flag, then the taps' bits against the running reference
    ref = {p: (list(DEFAULT), list(DEFAULT)) for p in range(3)}
    i = 0
    while i < len(syms):
        k, nb, v, p, u = syms[i]
        assert k == abi.SYM_WIENER_RESTORE
        unit = keep[p][u]
        assert v == unit.rtype
        j = i + 1
        while j < len(syms) and syms[j][0] == abi.SYM_BITS:
            j += 1
        got = [(s[1], s[2]) for s in syms[i + 1:j]]
        win = 7 if p == 0 else 5
        if unit.rtype:
            vf, hf = list(unit.vfilter), list(unit.hfilter)
            assert got == wiener_bits(win, vf, hf, *ref[p])
            # the bit count is the search's count_wiener_bits (plane-based window)
            rv, rh = (C.c_int16 * 8)(*ref[p][0]), (C.c_int16 * 8)(*ref[p][1])
            assert sum(b for b, _ in got) == oracle.lib().zfo_count_wiener_bits(
                win, (C.c_int16 * 8)(*vf), (C.c_int16 * 8)(*hf), rv, rh)
            ref[p] = (vf, hf)
        else:
            assert got == []
        assert all(1 <= b <= 16 and 0 <= val < (1 << b) for b, val in got)
        i = j
    for p in range(3):
        assert list(refs.vfilter[p]) == ref[p][0] and list(refs.hfilter[p]) == ref[p][1]


def test_none_planes_and_monochrome_code_nothing():
    rng = np.random.default_rng(3)
    d, keep = make_decisions(rng, 600, 400, rtypes=(1, 0, 0))
    syms, _ = walk(d, 600, 400)
    assert {p for _, _, _, p, _ in syms} == {0}
    d2, keep2 = make_decisions(rng, 600, 400)
    syms2, _ = walk(d2, 600, 400, monochrome=1)
    assert {p for _, _, _, p, _ in syms2} == {0}


def test_small_buffer_is_rejected_without_side_effects():
    rng = np.random.default_rng(4)
    d, keep = make_decisions(rng, 512, 512)
    for p in range(3):
        for u in range(d.lr[p].hunits * d.lr[p].vunits):
            keep[p][u].rtype = 1
    refs = abi.ZfWienerRefs()
    lib().zf_wiener_refs_reset(C.byref(refs))
    before = bytes(refs)
    out = (abi.ZfLrSym * 2)()
    assert lib().zf_lr_sb_syntax(C.byref(d), 0, 0, 16, 512, 512, 0, 0, C.byref(refs), out, 2) == -6
    assert bytes(refs) == before
