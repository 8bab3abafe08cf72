"""Served request loop on the GPU: every request's filtered recon and
decisions are identical alone (one zf_filter_stage call) and in the mix
(continuous batching over two worker contexts whose batches overlap on the
device). The stage is integer-exact, so the tolerance is zero."""
import copy
import random
import time

import numpy as np
import pytest

from zenav1_svt_gb300 import serve, synth

pytestmark = pytest.mark.gpu


def _mixed_frames(n, seed):
    rng = random.Random(seed)
    out = []
    for i in range(n):
        w, h = rng.randint(64, 720), rng.randint(64, 560)
        bd = 10 if rng.random() < 0.3 else 8
        qp = rng.randint(18, 45)
        preset = 4 if i % 5 == 0 else 6  # a few frames with the deblock level search
        out.append(synth.make_frame(synth.frame_seed(5, 1000 + i), w, h, bd, qp, preset, "cosine"))
    return out


def _same(a, b):
    assert a["lf"] == b["lf"]
    assert (a["cdef_damping"], a["cdef_bits"], a["cdef_y"], a["cdef_uv"]) == \
           (b["cdef_damping"], b["cdef_bits"], b["cdef_y"], b["cdef_uv"])
    assert (a["cdef_fb_idx"] == b["cdef_fb_idx"]).all()
    assert a["lr"] == b["lr"]


def test_served_results_equal_alone(pkg, ctx):
    frames = _mixed_frames(14, 7)
    alone = []
    for fr in frames:
        d, st, rec = ctx.filter_stage(fr)
        alone.append((d, rec))
    executors = [serve.FilterExecutor(0), serve.FilterExecutor(0)]
    srv = serve.Server(executors, hbm_budget_bytes=8 << 30, max_batch=4)
    rng = random.Random(3)
    reqs = []
    for i, fr in enumerate(frames):
        mine = copy.copy(fr)
        mine.rec = fr.copy_rec()  # filtered in place
        reqs.append(srv.submit(serve.Request(mine, rid=i)))
        time.sleep(rng.random() * 0.004)  # arrivals while earlier batches run
    srv.drain(timeout=120)
    srv.close()
    for ex in executors:
        ex.close()
    batches = {(r.worker, r.batch) for r in reqs}
    assert len(batches) >= 2
    for r, (d, rec) in zip(reqs, alone):
        r.wait(0)
        _same(r.decisions, d)
        for p in range(3):
            assert np.array_equal(r.frame.rec[p], rec[p]), (r.rid, p)
