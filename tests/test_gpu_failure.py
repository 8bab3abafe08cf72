"""Failure detection without a GPU fault.

- Cancellation (the reference's enough::Stop, surfaced as
  EncodeError::Cancelled): a context whose cancel flag is set refuses the
  call with Cancelled and writes no output; once the flag is cleared the
  same context runs the frame bit-exact against the oracle.
- The one device-side wait of the stage (the Wiener statistics kernel
  waiting for its TMA tile loads) has an iteration limit. ZF_WAIT_GIVE_UP
  makes it give up before its first step, as if the loads never arrived:
  the call returns Timeout, the CTAs drain their loads before they end, and
  the same context then runs the frame with the default limit bit-exact
  against the oracle. Nothing faults, traps or hangs: the kernels return and
  the host reads the status.
"""
import ctypes as C

import numpy as np
import pytest

from test_gpu_parity import assert_same_decisions, assert_same_planes
from zenav1_svt_gb300 import synth

pytestmark = pytest.mark.gpu


def test_cancel_flag_refuses_then_recovers(pkg, oracle):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    flag = (C.c_int32 * 1)(1)
    c = pkg.Context(0, cancel_flag=C.addressof(flag))
    try:
        fr = synth.make_frame(synth.frame_seed(13, 1), 320, 192, 8, 30, 4, "cosine")
        rec = fr.copy_rec()
        with pytest.raises(pkg.ZfError) as e:
            c.filter_stage(fr, rec=rec)
        assert e.value.kind == "Cancelled"
        assert all(np.array_equal(a, b) for a, b in zip(rec, fr.rec))  # nothing written
        flag[0] = 0
        do, so, ro = oracle.filter_stage(fr)
        dg, sg, rg = c.filter_stage(fr)
        assert_same_decisions(dg, do)
        assert_same_planes(rg, ro)
    finally:
        c.close()


@pytest.mark.parametrize("stats_tc", [0, 1], ids=["tma_rows", "tensor_core_mma"])
def test_statistics_wait_limit_times_out_and_context_recovers(ctx, pkg, oracle, stats_tc):
    """Both statistics forms: the CUDA-core kernel waits for its TMA tile
    loads, the tensor-core kernel for its MMAs."""
    # 8-bit, 16-aligned planes: the statistics rows come by TMA
    fr = synth.make_frame(synth.frame_seed(13, 2), 1024, 768, 8, 30, 6, "cosine")
    before = ctx.get_tune()
    ctx.set_tune(before["graphs"], 1, before["apply_group"], stats_tc)
    ctx.set_wait_limit(0xFFFFFFFF)  # ZF_WAIT_GIVE_UP: give up before the first step
    try:
        with pytest.raises(pkg.ZfError) as e:
            ctx.filter_stage(fr)
        assert e.value.kind == "Timeout"
    finally:
        ctx.set_wait_limit(0)
    try:
        do, so, ro = oracle.filter_stage(fr)
        dg, sg, rg = ctx.filter_stage(fr)
        assert_same_decisions(dg, do)
        assert_same_planes(rg, ro)
        assert sg == so
    finally:
        ctx.set_tune(before["graphs"], before["stats_tma"], before["apply_group"], before["stats_tc"])
