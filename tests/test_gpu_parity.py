"""GPU (CUDA, through the C ABI) vs the CPU oracle: bit-exact on every
output -- filtered planes, deblock levels, CDEF strengths and per-filter-
block indices, restoration types and taps, evidence counters.

The path is integer end to end, so the tolerance is zero.
"""
import zlib

import numpy as np
import pytest

from zenav1_svt_gb300 import synth

pytestmark = pytest.mark.gpu


def assert_same_decisions(dg, do, lr=True):
    assert dg["lf"] == do["lf"]
    assert dg["cdef_damping"] == do["cdef_damping"]
    assert dg["cdef_bits"] == do["cdef_bits"]
    assert dg["cdef_y"] == do["cdef_y"] and dg["cdef_uv"] == do["cdef_uv"]
    if do["cdef_bits"]:
        assert (dg["cdef_fb_idx"] == do["cdef_fb_idx"]).all()
    if lr:
        for p in range(3):
            a, b = dg["lr"][p], do["lr"][p]
            assert a["frame_rtype"] == b["frame_rtype"], p
            assert (a["hunits"], a["vunits"]) == (b["hunits"], b["vunits"])
            if b["frame_rtype"]:
                for ua, ub in zip(a["units"], b["units"]):
                    assert ua[0] == ub[0]
                    if ub[0]:
                        assert ua[1] == ub[1] and ua[2] == ub[2]


def assert_same_planes(a, b, chroma=True):
    for p in range(3 if chroma else 1):
        assert a[p].dtype == b[p].dtype and a[p].shape == b[p].shape
        if not (a[p] == b[p]).all():
            idx = np.argwhere(a[p] != b[p])
            raise AssertionError("plane %d differs at %d px, first %s: gpu %s oracle %s"
                                 % (p, len(idx), idx[0], a[p][tuple(idx[0])], b[p][tuple(idx[0])]))


CASES = [
    # (name, true_w, true_h, bd, qp, preset, content)
    ("p6_512", 512, 512, 8, 32, 6, "cosine"),
    ("p6_odd", 203, 137, 8, 40, 6, "cosine"),
    ("p4_search", 256, 192, 8, 24, 4, "power"),
    ("p2_refine", 192, 128, 8, 20, 2, "power"),
    ("p0_48cand", 128, 128, 8, 45, 0, "cosine"),
    ("p8_qp", 200, 120, 8, 50, 8, "cosine"),
    ("bd10_p2", 160, 128, 10, 28, 2, "power10"),
    ("bd10_p6_odd", 171, 99, 10, 36, 6, "cosine"),
    ("small_no_lr", 56, 40, 8, 30, 6, "cosine"),
    ("wide_units", 776, 408, 8, 34, 6, "cosine"),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_filter_stage_matches_oracle(ctx, oracle, case):
    name, w, h, bd, qp, preset, content = case
    fr = synth.make_frame(synth.frame_seed(9, zlib.crc32(name.encode()) & 0xFFFF), w, h, bd, qp, preset, content)
    do, so, ro = oracle.filter_stage(fr)
    dg, sg, rg = ctx.filter_stage(fr)
    assert_same_decisions(dg, do)
    assert_same_planes(rg, ro)
    assert sg == so


def test_monochrome_and_sharpness(ctx, oracle):
    fr = synth.make_frame(synth.frame_seed(9, 77), 144, 96, 8, 40, 6, "cosine", chroma=False)
    fr.sharpness = 3
    do, so, ro = oracle.filter_stage(fr)
    dg, sg, rg = ctx.filter_stage(fr)
    assert_same_decisions(dg, do)
    assert_same_planes(rg, ro, chroma=False)


def test_all_skip_frame(ctx, oracle):
    """Every 8x8 skipped: the CDEF search has no filter block (sb_count 0)."""
    fr = synth.make_frame(synth.frame_seed(9, 78), 128, 96, 8, 40, 6, "cosine", skip_prob=1.0)
    do, so, ro = oracle.filter_stage(fr)
    dg, sg, rg = ctx.filter_stage(fr)
    assert do["cdef_y"] == [0] and do["cdef_uv"] == [0]
    assert_same_decisions(dg, do)
    assert_same_planes(rg, ro)
    assert sg["cdef_sb_count"] == 0


def test_per_call_site_entry_points(ctx, oracle):
    """Each reference call site alone: deblock pick/apply, CDEF search/apply,
    Wiener search/apply, chained exactly like pipeline.rs."""
    fr = synth.make_frame(synth.frame_seed(9, 79), 232, 168, 8, 26, 4, "power")
    ro, rg = fr.copy_rec(), fr.copy_rec()
    assert ctx.pick_filter_levels(fr, rg) == oracle.deblock_pick(fr, ro)
    lf = oracle.deblock_pick(fr, ro)
    lf = lf if lf[0] else [6, 6, 3, 3]  # make sure the apply filters something
    oracle.deblock_apply(fr, ro, lf)
    ctx.apply_deblock_frame(fr, rg, lf)
    assert_same_planes(rg, ro)
    d_o, rows, has = oracle.cdef_search(fr, ro)
    d_g = ctx.cdef_search_still(fr, rg)
    assert_same_decisions(d_g.as_dict(), d_o.as_dict(), lr=False)
    pre_o, pre_g = [p.copy() for p in ro], [p.copy() for p in rg]
    so = oracle.cdef_apply(fr, ro, d_o)
    sg = ctx.apply_cdef_frame(fr, rg, d_g)
    assert_same_planes(rg, ro)
    assert sg["cdef_filtered_px"] == so["cdef_filtered_px"]
    assert sg["cdef_changed_px"] == so["cdef_changed_px"]
    l_o = oracle.lr_search(fr, ro)
    l_g = ctx.search_restoration_still(fr, rg)
    assert_same_decisions(l_g.as_dict(), l_o.as_dict())
    oracle.lr_apply(fr, ro, pre_o, l_o)
    ctx.apply_restoration_frame(fr, rg, pre_g, l_g)
    assert_same_planes(rg, ro)


def test_cdef_apply_with_multiple_strength_sets(ctx, oracle):
    """cdef_bits > 0 with a per-filter-block index (the multi-set outcome)."""
    fr = synth.make_frame(synth.frame_seed(9, 80), 320, 256, 8, 44, 6, "cosine")
    d_o = oracle.cdef_search(fr, fr.copy_rec())[0]
    d_o.c.cdef_bits = 2
    for i, (y, uv) in enumerate([(0, 0), (9, 4), (62, 13), (33, 60)]):
        d_o.c.cdef_y[i] = y
        d_o.c.cdef_uv[i] = uv
    d_o.fb_idx[:] = np.arange(d_o.fb_idx.size) % 4
    ro, rg = fr.copy_rec(), fr.copy_rec()
    so = oracle.cdef_apply(fr, ro, d_o)
    sg = ctx.apply_cdef_frame(fr, rg, d_o)
    assert_same_planes(rg, ro)
    assert sg["cdef_filtered_px"] == so["cdef_filtered_px"]
    assert sg["cdef_changed_px"] == so["cdef_changed_px"]


def test_lr_apply_odd_widths_follow_c_border(ctx, oracle):
    """Plane widths whose last 64-px processing unit rounds up by >= 9 px:
    the GPU follows C/libaom frame borders (the oracle's C mode)."""
    for w in (74, 330, 1010):
        fr = synth.make_frame(synth.frame_seed(9, 81 + w), w, 72, 8, 30, 6, "cosine")
        do, _, ro = oracle.filter_stage(fr)
        dg, _, rg = ctx.filter_stage(fr)
        assert_same_decisions(dg, do)
        assert_same_planes(rg, ro)


def test_batch_equals_single(ctx, oracle):
    """One launch per pass over a mixed batch == each frame alone == oracle."""
    frames = synth.workload_batch(n=10, max_dim=300)
    outs = ctx.submit_batch(frames)
    for fr, (dg, sg, rg) in zip(frames, outs):
        do, so, ro = oracle.filter_stage(fr)
        assert_same_decisions(dg, do)
        assert_same_planes(rg, ro)
        d1, s1, r1 = ctx.filter_stage(fr)
        assert_same_planes(r1, rg)
        assert sg == s1


def test_repeatable(ctx):
    fr = synth.make_frame(synth.frame_seed(9, 82), 256, 256, 8, 32, 6, "cosine")
    a = ctx.filter_stage(fr)
    b = ctx.filter_stage(fr)
    assert_same_planes(a[2], b[2])
    assert_same_decisions(a[0], b[0])
