"""A seeded random sweep of the parameter space in one mixed batch: every
frame draws its size (odd sizes and frames too small for restoration
included), bit depth, qp, preset (0-8 and 10: 48 to 4 CDEF candidates, the
level search and the closed-form levels, Wiener refinement or the tiled
trial, the qp picker), sharpness, monochrome, restoration on or off, the
content and the recon model. The whole set goes through one
zf_submit_batch (so frames of different presets share every launch), each
frame is compared with the oracle bit for bit, and a few frames also run
alone (batch == single)."""
import numpy as np
import pytest

from test_gpu_parity import assert_same_decisions, assert_same_planes
from zenav1_svt_gb300 import synth

pytestmark = pytest.mark.gpu

PRESETS = [0, 1, 2, 3, 4, 5, 6, 7, 8, 10]


def sweep_frames(seed, n):
    rng = np.random.default_rng(seed)
    frames, desc = [], []
    for i in range(n):
        hi = 420 if rng.random() < 0.75 else 900  # a quarter of the frames span several units
        w, h = int(rng.integers(40, hi)), int(rng.integers(40, hi))
        bd = 10 if rng.random() < 0.4 else 8
        qp = int(rng.integers(12, 59))
        preset = int(rng.choice(PRESETS))
        chroma = rng.random() < 0.85
        content = "cosine" if rng.random() < 0.5 else ("power10" if bd == 10 else "power")
        recon = "quant" if rng.random() < 0.7 else "offset"
        skip = None if rng.random() < 0.8 else float(rng.choice([0.0, 0.9]))
        fr = synth.make_frame(synth.frame_seed(71, seed * 100 + i), w, h, bd, qp, preset, content, chroma=chroma,
                              skip_prob=skip, recon=recon)
        fr.sharpness = 0 if rng.random() < 0.6 else int(rng.integers(1, 8))
        fr.enable_restoration = 0 if rng.random() < 0.15 else 1
        frames.append(fr)
        desc.append("%dx%d bd%d qp%d p%d sharp%d %s lr%d %s %s" % (w, h, bd, qp, preset, fr.sharpness,
                                                                    "yuv" if chroma else "mono",
                                                                    fr.enable_restoration, content, recon))
    return frames, desc


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_mixed_batch_matches_oracle(ctx, oracle, seed):
    frames, desc = sweep_frames(seed, 20)
    outs = ctx.submit_batch(frames)
    for k, (fr, (dg, sg, rg)) in enumerate(zip(frames, outs)):
        do, so, ro = oracle.filter_stage(fr)
        try:
            assert_same_decisions(dg, do)
            assert_same_planes(rg, ro, chroma=fr.chroma)
            assert sg == so
        except AssertionError as e:
            raise AssertionError("frame %d (%s): %s" % (k, desc[k], e)) from e
    for k in range(3):  # the same frames alone
        d1, s1, r1 = ctx.filter_stage(frames[k])
        assert_same_planes(r1, outs[k][2], chroma=frames[k].chroma)
        assert s1 == outs[k][1]


def test_random_frames_through_each_call_site(ctx, oracle):
    """Six frames of the sweep through the per-call-site entry points, chained
    as the reference pipeline calls them (deblock pick, deblock apply, CDEF
    search, CDEF apply, Wiener search, Wiener apply), each step against the
    oracle's same step on the same input."""
    frames, desc = sweep_frames(4, 6)
    for k, fr in enumerate(frames):
        try:
            ro, rg = fr.copy_rec(), fr.copy_rec()
            lf = oracle.deblock_pick(fr, ro)
            assert ctx.pick_filter_levels(fr, rg) == lf
            oracle.deblock_apply(fr, ro, lf)
            ctx.apply_deblock_frame(fr, rg, lf)
            assert_same_planes(rg, ro, chroma=fr.chroma)
            d_o = oracle.cdef_search(fr, ro)[0]
            d_g = ctx.cdef_search_still(fr, rg)
            assert_same_decisions(d_g.as_dict(), d_o.as_dict(), lr=False)
            pre_o, pre_g = [p.copy() for p in ro], [p.copy() for p in rg]
            so = oracle.cdef_apply(fr, ro, d_o)
            sg = ctx.apply_cdef_frame(fr, rg, d_g)
            assert_same_planes(rg, ro, chroma=fr.chroma)
            assert sg["cdef_filtered_px"] == so["cdef_filtered_px"]
            assert sg["cdef_changed_px"] == so["cdef_changed_px"]
            l_o = oracle.lr_search(fr, ro)
            l_g = ctx.search_restoration_still(fr, rg)
            assert_same_decisions(l_g.as_dict(), l_o.as_dict())
            oracle.lr_apply(fr, ro, pre_o, l_o)
            ctx.apply_restoration_frame(fr, rg, pre_g, l_g)
            assert_same_planes(rg, ro, chroma=fr.chroma)
        except AssertionError as e:
            raise AssertionError("frame %d (%s): %s" % (k, desc[k], e)) from e
