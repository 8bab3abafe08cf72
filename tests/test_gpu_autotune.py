"""Launch settings and the autotuner (zf_get_tune / zf_set_tune /
zf_autotune): every setting gives the same bytes, the tuner times every
candidate on private copies (the caller's recon is not written), keeps the
fastest on the context, and rejects settings out of range."""
import ctypes as C

import numpy as np
import pytest

from zenav1_svt_gb300 import ZfError, abi, pack_geom, synth

pytestmark = pytest.mark.gpu


def _frames():
    return [synth.make_frame(synth.frame_seed(12, 1), 520, 264, 8, 30, 6, "cosine"),
            synth.make_frame(synth.frame_seed(12, 2), 203, 137, 10, 40, 6, "cosine"),
            synth.make_frame(synth.frame_seed(12, 3), 384, 320, 8, 22, 4, "power")]


def _same(outs_a, outs_b):
    for (da, sa, ra), (db, sb, rb) in zip(outs_a, outs_b):
        for p in range(3):
            assert np.array_equal(ra[p], rb[p]), p
        for k in ("lf", "cdef_damping", "cdef_bits", "cdef_y", "cdef_uv", "lr"):
            assert da[k] == db[k], k
        assert sa == sb


def test_tune_roundtrip_and_range(ctx):
    before = ctx.get_tune()
    try:
        ctx.set_tune(1, 0, 4, 1, 32, 4)
        t = ctx.get_tune()
        assert (t["graphs"], t["stats_tma"], t["apply_group"], t["stats_tc"], t["trial_tile"], t["db_levels"]) == (
            1, 0, 4, 1, 32, 4)
        for bad in ((2, 1, 8), (0, -1, 8), (0, 1, 0), (0, 1, 17), (0, 1, 8, 2), (0, 1, 8, 0, 48),
                    (0, 1, 8, 0, 64, 1), (0, 1, 8, 0, 64, 9)):
            with pytest.raises(ZfError):
                ctx.set_tune(*bad)
        assert ctx.get_tune() == t  # a rejected setting changes nothing
    finally:
        ctx.set_tune_dict(before)


def test_every_setting_gives_the_same_bytes(ctx):
    frames = _frames()
    before = ctx.get_tune()
    try:
        ctx.set_tune(0, 1, 8, 0)  # the default setting as the reference
        ref = ctx.submit_batch(frames)
        for setting in ((0, 0, 1, 0), (1, 1, 16, 1), (0, 1, 2, 0, 32, 2), (1, 0, 3, 1, 32, 8), (0, 1, 8, 1, 64, 4)):
            ctx.set_tune(*setting)
            _same(ctx.submit_batch(frames), ref)
            _same([ctx.filter_stage(frames[0])], ref[:1])
    finally:
        ctx.set_tune_dict(before)


def test_autotune_picks_the_fastest_and_leaves_inputs(ctx):
    frames = _frames()
    before = ctx.get_tune()
    try:
        ctx.set_tune(0, 1, 8)
        ref = ctx.submit_batch(frames)
        mis = [pack_geom(f.geom) for f in frames]
        recs = [f.copy_rec() for f in frames]
        keep = [[p.copy() for p in r] for r in recs]
        arr = (abi.ZfFrame * len(frames))()
        for i, f in enumerate(frames):
            arr[i] = abi.make_frame_struct(f, f.src, recs[i], mis[i])
        best, cands = ctx.autotune_raw(arr, len(frames), reps=2)
        # coordinate descent: every value of every knob is timed once
        keys = ("graphs", "stats_tma", "apply_group", "stats_tc", "trial_tile", "db_levels")
        settings = {tuple(c[k] for k in keys) for c in cands}
        assert len(settings) == len(cands) >= 11
        assert {c["graphs"] for c in cands} == {0, 1}
        assert {(c["stats_tc"], c["stats_tma"]) for c in cands} >= {(0, 1), (0, 0), (1, 1)}
        assert {c["apply_group"] for c in cands} == {1, 2, 4, 8, 16}
        assert {c["trial_tile"] for c in cands} == {32, 64}
        assert {c["db_levels"] for c in cands} == {2, 4, 8}
        assert all(c["ms"] > 0 for c in cands)
        assert best["ms"] == min(c["ms"] for c in cands)
        t = ctx.get_tune()
        assert {k: t[k] for k in keys} == {k: best[k] for k in keys}
        for r, k in zip(recs, keep):  # the caller's recon was not written
            for p in range(3):
                assert np.array_equal(r[p], k[p])
        _same(ctx.submit_batch(frames), ref)  # the tuned setting gives the same bytes
        # a single frame goes through zf_filter_stage
        one = (abi.ZfFrame * 1)()
        one[0] = arr[0]
        best1, cands1 = ctx.autotune_raw(one, 1, reps=1)
        assert len(cands1) >= 11 and best1["ms"] == min(c["ms"] for c in cands1)
        _same([ctx.filter_stage(frames[0])], ref[:1])
    finally:
        ctx.set_tune_dict(before)


def test_autotune_rejects_bad_arguments(ctx):
    f = _frames()[0]
    mi = pack_geom(f.geom)
    rec = f.copy_rec()
    arr = (abi.ZfFrame * 1)()
    arr[0] = abi.make_frame_struct(f, f.src, rec, mi)
    lib = __import__("zenav1_svt_gb300").lib()
    best = abi.ZfTune()
    assert lib.zf_autotune(ctx.h, arr, 0, 1, C.byref(best), None, 0) == -6
    assert lib.zf_autotune(ctx.h, arr, 1, 0, C.byref(best), None, 0) == -6
    assert lib.zf_autotune(ctx.h, arr, 1, 1, None, None, 0) == -6
