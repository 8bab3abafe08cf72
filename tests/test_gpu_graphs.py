"""CUDA-graph mode (zf_use_graphs): the captured launch sequence gives the
same decisions and planes as direct launches, for repeated frame shapes
(in-place graph update), changing shapes (re-instantiation), presets with
the host-driven deblock level search before the capture, and batches."""
import numpy as np
import pytest

from zenav1_svt_gb300 import synth

from test_gpu_parity import assert_same_decisions, assert_same_planes

pytestmark = pytest.mark.gpu


FRAMES = [
    (203, 137, 8, 40, 6, "cosine"),
    (203, 137, 8, 36, 6, "cosine"),   # same shape: update in place
    (256, 192, 8, 24, 4, "power"),     # deblock search before the capture
    (171, 99, 10, 36, 6, "cosine"),
    (192, 128, 8, 20, 2, "power"),     # refinement trial (clusters)
]


def test_graph_mode_matches_direct_launches(pkg):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    direct, graph = pkg.Context(0), pkg.Context(0)
    graph.use_graphs(True)
    try:
        for k, (w, h, bd, qp, preset, content) in enumerate(FRAMES):
            fr = synth.make_frame(synth.frame_seed(13, k), w, h, bd, qp, preset, content)
            d0, s0, r0 = direct.filter_stage(fr)
            d1, s1, r1 = graph.filter_stage(fr)
            assert_same_decisions(d1, d0)
            assert_same_planes(r1, r0)
            assert s1 == s0
        launches, updates, inst = graph.graph_stats()
        assert launches == len(FRAMES) and updates + inst == launches and updates >= 1
        assert direct.graph_stats() == (0, 0, 0)
        frames = [synth.make_frame(synth.frame_seed(14, k), w, h, bd, qp, 6, "cosine")
                  for k, (w, h, bd, qp) in enumerate([(120, 88, 8, 30), (96, 64, 10, 44), (264, 136, 8, 28)])]
        for (d0, s0, r0), (d1, s1, r1) in zip(direct.submit_batch(frames), graph.submit_batch(frames)):
            assert_same_decisions(d1, d0)
            assert_same_planes(r1, r0)
    finally:
        direct.close()
        graph.close()


def test_tma_rows_match_thread_staging(pkg):
    """The statistics kernel's TMA-loaded rows (8-bit planes with 16-byte
    row pitch) give the same stage as thread-staged rows, including units at
    every plane edge, odd true sizes and the zero-copy device path."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from zenav1_svt_gb300 import abi
    a, b = pkg.Context(0), pkg.Context(0, flags=abi.OPT_NO_TMA)
    try:
        for k, (w, h, qp, preset) in enumerate([(1024, 576, 30, 6), (1000, 600, 44, 4), (517, 389, 36, 6),
                                                 (640, 1152, 24, 6), (96, 64, 40, 6), (1018, 571, 34, 6)]):
            fr = synth.make_frame(synth.frame_seed(15, k), w, h, 8, qp, preset, "power")
            d0, s0, r0 = a.filter_stage(fr)
            d1, s1, r1 = b.filter_stage(fr)
            assert_same_decisions(d1, d0)
            assert_same_planes(r1, r0)
    finally:
        a.close()
        b.close()
