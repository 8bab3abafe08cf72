"""Frame-header filter syntax (loop_filter_params, cdef_params, lr_params)
through the C ABI (zf_write_filter_params, host code) against the oracle's
restatement of write_key_frame_header (svtav1-entropy/src/obu.rs:1268-1377)
and against the field layouts the reference's own tests derive by hand
(obu.rs fh_cdef_params_bit_layout, fh_lr_params_all_none_bit_shape)."""
import ctypes as C

import numpy as np
import pytest

from zenav1_svt_gb300 import abi


def decisions(lf=(0, 0, 0, 0), damping=3, bits=0, y=(0,), uv=(0,), lr=(0, 0, 0), unit=(256, 256, 256)):
    d = abi.ZfDecisions()
    d.lf[:] = list(lf)
    d.cdef_damping, d.cdef_bits = damping, bits
    for i in range(1 << bits):
        d.cdef_y[i], d.cdef_uv[i] = y[i], uv[i]
    for p in range(3):
        d.lr[p].frame_rtype, d.lr[p].unit_size = lr[p], unit[p]
    return d


def fields(*pairs):
    return "".join(format(v, "0%db" % n) for v, n in pairs)


def lib_bits(pkg, d, **kw):
    buf, end = pkg.write_filter_params(d, **kw)
    return "".join(str((buf[i >> 3] >> (7 - (i & 7))) & 1) for i in range(end))


def test_mono_cdef_layout_of_the_reference_test(pkg):
    # obu.rs fh_cdef_params_bit_layout: mono, levels 0, sharpness 0,
    # damping 6, cdef_bits 0, y strength 43 (pri 10, sec 3), no lr_params
    d = decisions(damping=6, y=(43,))
    want = fields((0, 6), (0, 6), (0, 3), (0, 1), (3, 2), (0, 2), (43, 6))
    assert lib_bits(pkg, d, monochrome=True, enable_restoration=False) == want


def test_lr_all_none_adds_two_zero_bits_per_plane(pkg):
    # obu.rs fh_lr_params_all_none_bit_shape: +6 bits at 4:2:0, +2 mono
    d = decisions(lf=(19, 19, 9, 9), damping=4, y=(14,), uv=(14,))
    base = lib_bits(pkg, d, enable_restoration=False)
    assert base == fields((19, 6), (19, 6), (9, 6), (9, 6), (0, 3), (0, 1), (1, 2), (0, 2), (14, 6), (14, 6))
    assert lib_bits(pkg, d, enable_restoration=True) == base + "000000"
    dm = decisions(lf=(19, 19, 0, 0), damping=4, y=(14,))
    assert lib_bits(pkg, dm, monochrome=True, enable_restoration=True) == \
        lib_bits(pkg, dm, monochrome=True, enable_restoration=False) + "00"


def test_lr_types_unit_size_and_uv_shift(pkg):
    d = decisions(lr=(1, 0, 0))
    tail = lib_bits(pkg, d)[-8:]
    assert tail == "10" + "00" + "00" + "11"        # WIENER luma, unit 256 at SB64: (>64, >128)
    d = decisions(lr=(1, 2, 3))
    assert lib_bits(pkg, d)[-9:] == "10" + "11" + "01" + "11" + "0"  # + lr_uv_shift = 0
    d = decisions(lr=(0, 1, 0), unit=(256, 128, 128))
    assert lib_bits(pkg, d)[-9:] == "00" + "10" + "00" + "11" + "1"
    d = decisions(lr=(1, 0, 0), unit=(128, 128, 128))
    assert lib_bits(pkg, d, sb_size=128)[-7:] == "10" + "00" + "00" + "0"  # SB128: only (>128)


def test_intrabc_codes_nothing_and_position_is_kept(pkg):
    d = decisions(lf=(5, 6, 7, 8), damping=5, y=(3,), uv=(4,), lr=(1, 1, 1))
    buf = np.full(64, 0xFF, np.uint8)
    _, end = pkg.write_filter_params(d, allow_intrabc=True, buf=buf, bit_pos=13)
    assert end == 13 and (buf == 0xFF).all()
    buf = np.full(64, 0xFF, np.uint8)
    _, end = pkg.write_filter_params(d, buf=buf, bit_pos=3)
    assert buf[0] >> 5 == 0b111  # bits before the start position are kept


@pytest.mark.parametrize("seed", range(4))
def test_matches_oracle_on_random_decisions(pkg, oracle, seed):
    rng = np.random.default_rng(seed)
    for _ in range(200):
        bits = int(rng.integers(0, 4))
        lf = [int(v) for v in rng.integers(0, 64, 4)]
        if rng.random() < 0.3:
            lf[0] = lf[1] = 0
        d = decisions(lf=lf, damping=int(rng.integers(3, 7)), bits=bits,
                      y=[int(v) for v in rng.integers(0, 64, 8)], uv=[int(v) for v in rng.integers(0, 64, 8)],
                      lr=[int(v) for v in rng.integers(0, 4, 3)],
                      unit=(256, int(rng.choice([128, 256])), 256))
        kw = dict(monochrome=bool(rng.random() < 0.2), enable_restoration=bool(rng.random() < 0.8),
                  sb_size=64, sharpness=int(rng.integers(0, 8)))
        o = abi.ZfHeaderOpts(int(kw["monochrome"]), 0, int(kw["enable_restoration"]), 64, kw["sharpness"], 0)
        assert lib_bits(pkg, d, **kw) == oracle.write_filter_params(d, o)


def test_invalid_fields_rejected(pkg):
    with pytest.raises(pkg.ZfError):
        pkg.write_filter_params(decisions(damping=7))
    with pytest.raises(pkg.ZfError):
        pkg.write_filter_params(decisions(lr=(1, 0, 0), unit=(64, 64, 64)), sb_size=128)
    with pytest.raises(pkg.ZfError):
        pkg.write_filter_params(decisions(lf=(9, 9, 9, 9)), buf=np.zeros(2, np.uint8))
