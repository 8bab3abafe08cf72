"""zf_cdef_search_noalloc: the allocation-free CDEF strength search.

Callers that cannot allocate device memory once running (an encoder loop
that reserves everything at start-up, code running while another stream is
being captured, a process on a fully reserved GPU slice) use this entry
point; it
keeps its scratch in a static device array instead of a context arena. These
tests call it through the C ABI and check it against the existing
zf_cdef_search entry point and the oracle -- the integer decisions must be
identical -- on two calls in a row per frame (the shared static scratch
keeps the previous call's contents, which must not leak into the next
result).

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from zenav1_svt_gb300 import abi, synth

pytestmark = pytest.mark.gpu


def _bind(pkg):
    L = pkg.lib()
    L.zf_cdef_search_noalloc.argtypes = [C.c_void_p, C.POINTER(abi.ZfFrame), C.POINTER(abi.ZfDecisions)]
    L.zf_cdef_search_noalloc.restype = C.c_int32
    return L


def _on_device(fr, mi):
    import torch
    dev = torch.device("cuda", 0)
    src = [torch.from_numpy(p.copy()).to(dev) for p in fr.src]
    rec = [torch.from_numpy(p.copy()).to(dev) for p in fr.rec]
    m = torch.from_numpy(mi.view(np.int32).copy()).to(dev)
    s = abi.make_frame_struct(fr, [x.data_ptr() for x in src], [x.data_ptr() for x in rec], m.data_ptr(),
                              on_device=True)
    torch.cuda.synchronize()
    return s, (src, rec, m)


def _same(a, b):
    assert a["cdef_damping"] == b["cdef_damping"]
    assert a["cdef_bits"] == b["cdef_bits"]
    assert a["cdef_y"] == b["cdef_y"] and a["cdef_uv"] == b["cdef_uv"]
    assert (a["cdef_fb_idx"] == b["cdef_fb_idx"]).all()


NOALLOC_FRAMES = [
    # (seed, w, h, bd, qp, preset, content): 4 candidates (single CTA rows),
    # 6 candidates, 20 candidates (preset 2), and the largest frame the
    # scratch takes (3840x2160: 2040 filter blocks, the 8-CTA cluster's
    # biggest per-CTA share of rows) at presets 4 and 2
    (synth.frame_seed(12, 1), 1000, 600, 8, 44, 6, "cosine"),
    (synth.frame_seed(12, 2), 512, 384, 10, 30, 4, "power10"),
    (synth.frame_seed(12, 3), 640, 480, 8, 30, 2, "cosine"),
    (synth.frame_seed(2, 1), 3840, 2160, 8, 40, 4, "power"),
    (synth.frame_seed(2, 5), 3840, 2160, 8, 28, 2, "power"),
]


def test_noalloc_search_matches_cdef_search_twice(pkg, ctx, oracle):
    """Each frame searched twice in a row through the allocation-free entry
    point: equal to zf_cdef_search and to the oracle both times."""
    L = _bind(pkg)
    for args in NOALLOC_FRAMES:
        fr = synth.make_frame(*args)
        mi = pkg.pack_geom(fr.geom)
        want = ctx.cdef_search_still(fr, fr.copy_rec(), mi=mi).as_dict()
        ref = oracle.cdef_search(fr, fr.copy_rec())[0].as_dict()
        _same(want, ref)
        s, keep = _on_device(fr, mi)
        for _ in range(2):
            got = abi.Decisions(fr.w, fr.h, fr.true_w, fr.true_h)
            rc = L.zf_cdef_search_noalloc(None, C.byref(s), C.byref(got.c))
            assert rc == 0, rc
            _same(got.as_dict(), want)
            _same(got.as_dict(), ref)
        del keep


def test_noalloc_refuses_a_capturing_stream(pkg):
    """The call synchronises its stream, so a stream under capture is
    refused instead of being invalidated."""
    import torch
    L = _bind(pkg)
    fr = synth.make_frame(*NOALLOC_FRAMES[0])
    s, keep = _on_device(fr, pkg.pack_geom(fr.geom))
    side = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    d = abi.Decisions(fr.w, fr.h, fr.true_w, fr.true_h)
    with torch.cuda.graph(g, stream=side):
        rc = L.zf_cdef_search_noalloc(C.c_void_p(side.cuda_stream), C.byref(s), C.byref(d.c))
    assert rc == -3  # UnsupportedConfig
    del keep


def test_noalloc_rejects_frames_beyond_its_limits(pkg):
    L = _bind(pkg)
    dummy = [np.zeros((8, 8), np.uint8)] * 3  # never read: the limits are checked first
    fr = synth.Frame(8, 4096, 2176, dummy, dummy, synth.Geometry(8, 8), 128, 6)
    fr.w, fr.h = 4096, 2176  # 64 x 34 = 2176 filter blocks > 2048
    s = abi.make_frame_struct(fr, [1, 1, 1], [1, 1, 1], 1, on_device=True)
    d = abi.Decisions(fr.w, fr.h, fr.true_w, fr.true_h)
    assert L.zf_cdef_search_noalloc(None, C.byref(s), C.byref(d.c)) == -2  # InvalidDimensions
    fr.w, fr.h, fr.true_w, fr.true_h, fr.preset = 128, 128, 128, 128, 0  # 48 candidates
    s = abi.make_frame_struct(fr, [1, 1, 1], [1, 1, 1], 1, on_device=True)
    assert L.zf_cdef_search_noalloc(None, C.byref(s), C.byref(d.c)) == -3  # UnsupportedConfig
