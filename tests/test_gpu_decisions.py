"""Decision-branch parity: frames chosen so that every decision the stage
makes is taken at least once, each checked bit-exact against the oracle --
and the intermediate values behind the decisions compared directly:

- the deblock level search with a non-zero outcome at 8 and 10 bits, at
  presets with and without the refinement steps (conv_th 0 and 1), and every
  trial SSE of the hill-climb: the whole 64-level table of
  try_filter_plane (deblock.rs:228-293) per plane, and the trace lines of
  the climb in the reference's SVTAV1_DLFDBG format;
- the CDEF mse rows (cdef_search_still, cdef.rs:1166-1352) element by
  element, and the joint strength search at cdef_bits 1, 2 and 3;
- loop restoration with a plane mixing WIENER and NONE units and a frame
  whose plane type is NONE, and the per-unit search values
  (sse_none, score, trial SSE, taps) through the trace.

The recon of these frames is the quantised-transform stand-in
(synth.synth_recon_quant), the blocky recon the searches exist for. The
path is integer end to end: the tolerance is zero.
"""
import os

import numpy as np
import pytest

from test_gpu_parity import assert_same_decisions, assert_same_planes
from zenav1_svt_gb300 import synth

pytestmark = pytest.mark.gpu


def frame(cfg, w, h, bd, qp, preset, content, recon="quant", chroma=True):
    return synth.make_frame(synth.frame_seed(cfg, w + qp * 7 + preset), w, h, bd, qp, preset, content,
                            recon=recon, chroma=chroma)


# (name, frame args, predicate on the oracle's decisions that names the branch)
def lr_mixed(d):
    return any(0 < sum(u[0] for u in p["units"]) < len(p["units"]) for p in d["lr"] if p["frame_rtype"])


def lr_plane_none(d):
    return any(p["frame_rtype"] == 0 for p in d["lr"])


BRANCHES = [
    ("dlf_search_p4_8bit", (11, 512, 384, 8, 30, 4, "cosine"), lambda d: d["lf"][0] > 0 and d["lf"][2] > 0),
    ("dlf_search_p2_8bit_mixed_lr", (11, 512, 384, 8, 20, 2, "cosine"), lambda d: d["lf"][0] > 0 and lr_mixed(d)),
    ("dlf_search_p4_10bit", (12, 384, 256, 10, 48, 4, "power10"), lambda d: d["lf"][0] > 0),
    ("dlf_search_p2_10bit_odd", (12, 331, 203, 10, 36, 2, "cosine"), lambda d: d["lf"][0] > 0 and lr_plane_none(d)),
    ("lr_mixed_p4", (11, 512, 384, 8, 20, 4, "power"), lambda d: lr_mixed(d)),
    ("cdef_bits1", (11, 512, 384, 8, 30, 6, "power"), lambda d: d["cdef_bits"] == 1),
    ("cdef_bits2", (11, 512, 384, 8, 40, 6, "power"), lambda d: d["cdef_bits"] == 2),
    ("cdef_bits3_p6", (11, 768, 512, 8, 30, 6, "cosine"), lambda d: d["cdef_bits"] == 3),
    ("cdef_bits3_p2", (11, 768, 512, 8, 30, 2, "cosine"), lambda d: d["cdef_bits"] == 3),
    ("lr_mixed_chroma_p2", (11, 768, 512, 8, 40, 2, "cosine"), lambda d: lr_mixed(d)),
    ("lr_none_chroma_p4_10bit", (12, 331, 203, 10, 48, 4, "cosine"), lambda d: d["lr"][0]["frame_rtype"] == 0),
]


@pytest.mark.parametrize("case", BRANCHES, ids=[c[0] for c in BRANCHES])
def test_branch_taken_and_matches_oracle(ctx, oracle, case):
    name, args, taken = case
    fr = frame(*args)
    do, so, ro = oracle.filter_stage(fr)
    assert taken(do), "the frame no longer takes the branch %s: %s" % (name, do)
    dg, sg, rg = ctx.filter_stage(fr)
    assert_same_decisions(dg, do)
    assert_same_planes(rg, ro)
    assert sg == so


TABLE = [
    ("8bit_512x384_q30", (11, 512, 384, 8, 30, 4, "cosine")),
    ("8bit_odd_203x137_q40", (9, 203, 137, 8, 40, 4, "cosine")),
    ("10bit_384x256_q48", (12, 384, 256, 10, 48, 4, "power10")),
    ("10bit_sharp3_331x203_q36", (12, 331, 203, 10, 36, 2, "cosine")),
]


@pytest.mark.parametrize("case", TABLE, ids=[c[0] for c in TABLE])
def test_deblock_trial_sse_every_level(ctx, oracle, case):
    """try_filter_plane at every level 0..63 of every plane, one launch per
    plane, equal to the oracle's trial SSEs."""
    name, args = case
    fr = frame(*args)
    if "sharp3" in name:
        fr.sharpness = 3
    levels = np.arange(64, dtype=np.int32)
    for plane in range(3):
        g = ctx.deblock_sse_table(fr, plane, levels)
        o = oracle.deblock_sse_table(fr, plane, levels)
        assert (g == o).all(), (plane, np.nonzero(g != o)[0][:8], g[:8], o[:8])
        assert len(set(o.tolist())) > 8  # the levels filter differently
    # an arbitrary order and repeats, fewer than one launch's worth
    lv = np.array([17, 3, 3, 63, 0], np.int32)
    assert (ctx.deblock_sse_table(fr, 0, lv) == oracle.deblock_sse_table(fr, 0, lv)).all()


def test_deblock_table_arguments(pkg, ctx):
    fr = frame(9, 64, 64, 8, 30, 4, "cosine")
    with pytest.raises(pkg.ZfError):
        ctx.deblock_sse_table(fr, 0, np.array([64], np.int32))
    with pytest.raises(pkg.ZfError):
        ctx.deblock_sse_table(fr, 3, np.array([1], np.int32))
    with pytest.raises(pkg.ZfError):
        ctx.deblock_sse_table(fr, 0, np.zeros(65, np.int32))


ROWS = [
    ("p6_4cand", (11, 512, 384, 8, 40, 6, "power")),
    ("p4_6cand", (11, 512, 384, 8, 30, 4, "cosine")),
    ("p2_20cand", (11, 768, 512, 8, 30, 2, "cosine")),
    ("p0_48cand", (9, 256, 192, 8, 45, 0, "cosine")),
    ("bd10_p6_odd", (12, 331, 203, 10, 36, 6, "power10")),
    ("bd10_p2", (12, 384, 256, 10, 24, 2, "cosine")),
    ("offset_recon_p4", (11, 512, 384, 8, 24, 4, "power", "offset")),
]


@pytest.mark.parametrize("case", ROWS, ids=[c[0] for c in ROWS])
def test_cdef_mse_rows_match_oracle(ctx, oracle, case):
    """Every filter block's luma and joint-chroma candidate SSEs equal the
    oracle's (the SVTAV1_CDEF_DBG rows), and so do the picks they feed."""
    name, args = case
    fr = frame(*args)
    pre = fr.copy_rec()
    lf = oracle.deblock_pick(fr, pre)
    oracle.deblock_apply(fr, pre, lf)
    d_o, rows_o, has_o = oracle.cdef_search(fr, [p.copy() for p in pre])
    d_g, rows_g, has_g = ctx.cdef_search_rows(fr, [p.copy() for p in pre])
    assert (has_g == has_o).all()
    assert rows_o is not None and rows_g is not None and rows_g.shape == rows_o.shape
    sel = has_o.astype(bool)
    diff = np.argwhere(rows_g[sel] != rows_o[sel])
    assert len(diff) == 0, "mse rows differ at %d entries, first (fb, slot) %s" % (len(diff), diff[:4])
    assert_same_decisions(d_g.as_dict(), d_o.as_dict(), lr=False)


def test_cdef_mse_rows_monochrome_and_qp_picker(ctx, oracle):
    fr = frame(9, 200, 120, 8, 40, 6, "cosine", chroma=False)
    d_o, rows_o, has_o = oracle.cdef_search(fr, fr.copy_rec())
    d_g, rows_g, has_g = ctx.cdef_search_rows(fr, fr.copy_rec())
    assert (has_g == has_o).all() and (rows_g[has_o.astype(bool)] == rows_o[has_o.astype(bool)]).all()
    assert (rows_g[:, rows_g.shape[1] // 2:] == 0).all()  # no chroma rows
    fr8 = frame(9, 200, 120, 8, 50, 8, "cosine")  # preset 8: qp closed form, no search
    d_g, rows_g, has_g = ctx.cdef_search_rows(fr8, fr8.copy_rec())
    assert rows_g is None and not has_g.any()


TRACE = [
    ("p2_refine", (11, 256, 192, 8, 20, 2, "power")),
    ("p4_search", (11, 512, 384, 8, 30, 4, "cosine")),
    ("p6", (11, 768, 512, 8, 30, 6, "cosine")),
    ("bd10_p2_odd", (12, 331, 203, 10, 36, 2, "cosine")),
]


@pytest.mark.parametrize("case", TRACE, ids=[c[0] for c in TRACE])
def test_trace_matches_oracle_line_by_line(ctx, oracle, tmp_path, case):
    """The search trace of the whole stage (deblock trials, CDEF rows and
    pick, restoration units) is the oracle's, line for line."""
    name, args = case
    fr = frame(*args)
    tg, to = str(tmp_path / "gpu.txt"), str(tmp_path / "oracle.txt")
    oracle.trace(to)
    try:
        oracle.filter_stage(fr)
    finally:
        oracle.trace(None)
    ctx.trace(tg)
    try:
        ctx.filter_stage(fr)
    finally:
        ctx.trace(None)
    lg, lo = open(tg).read().splitlines(), open(to).read().splitlines()
    kinds = {l.split()[0] for l in lo}
    assert {"RS_CDEF_FB", "RS_CDEF_PICK", "LRNONE", "LRWNSCORE"} <= kinds
    if args[5] <= 5:
        assert "DLF_TRY" in kinds and "DLF_PICK" in kinds
    for k, (a, b) in enumerate(zip(lg, lo)):
        assert a == b, "trace line %d differs:\n gpu    %s\n oracle %s" % (k, a, b)
    assert len(lg) == len(lo)


def test_trace_env_and_batch_frames(pkg, tmp_path):
    """ZF_TRACE at context creation; a batch writes a ZF_FRAME line per frame."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    path = str(tmp_path / "env.txt")
    os.environ["ZF_TRACE"] = path
    try:
        c = pkg.Context(0)
    finally:
        del os.environ["ZF_TRACE"]
    try:
        frames = [frame(9, 128 + 8 * k, 96, 8, 30, 4 + k, "cosine") for k in range(3)]
        c.submit_batch(frames)
        c.trace(None)
    finally:
        c.close()
    lines = open(path).read().splitlines()
    assert [l for l in lines if l.startswith("ZF_FRAME")] == [
        "ZF_FRAME index=%d w=%d h=%d" % (k, f.true_w, f.true_h) for k, f in enumerate(frames)]


def test_saturated_samples_stay_exact(ctx, oracle):
    """Samples at 0 and 255 only (every centred product at its 2^14 bound):
    the tensor-core statistics' fp32 chains stay exact, and the whole stage
    matches the oracle, with the tensor-core and the CUDA-core statistics."""
    rng = np.random.default_rng(77)
    fr = frame(9, 384, 256, 8, 36, 6, "cosine")
    for p in range(3):
        h, w = fr.src[p].shape
        blocks = rng.integers(0, 2, size=(h // 4 + 1, w // 4 + 1)).astype(np.uint8) * 255
        fr.src[p] = np.ascontiguousarray(np.repeat(np.repeat(blocks, 4, 0), 4, 1)[:h, :w])
        fr.rec[p] = np.where(rng.random((h, w)) < 0.5, 0, 255).astype(np.uint8)
    do, so, ro = oracle.filter_stage(fr)
    before = ctx.get_tune()
    try:
        for tc in (1, 0):
            ctx.set_tune(before["graphs"], before["stats_tma"], before["apply_group"], tc)
            dg, sg, rg = ctx.filter_stage(fr)
            assert_same_decisions(dg, do)
            assert_same_planes(rg, ro)
            assert sg == so
    finally:
        ctx.set_tune(before["graphs"], before["stats_tma"], before["apply_group"], before["stats_tc"])
