"""Full-size parity: every configuration the bench times, at its real size,
through the C ABI against the oracle, bit-exact on every plane and decision.

- the plain per-image 4K workload: the bench's own four 3840x2160 8-bit
  frames (presets {4, 6} x qp {24, 40}, synth.workload_4k), preset 4 with
  the deblock level search;
- the 10-bit high-resolution frame (4096x3072, preset 2: 20 CDEF
  candidates, deblock search, Wiener refinement), synth.workload_10bit_4096;
- a 24-image slice of the bench's 256-image mixed batch in one
  zf_submit_batch call: the four largest images (~2000x2000, 8- and 10-bit),
  10-bit and odd-size images;
- a 6000x4000 preset-6 frame, the served workload's largest size: 3818
  filter blocks with 4 candidates, beyond the register-row joint search, so
  the joint strength search runs on the cluster form (a warp per pair);
- a 2560x1664 preset-0 frame: 1040 filter blocks at 48 candidates, the
  cluster form's pair-per-thread step (the 4096x3072 frame takes it at 20);
- the 4K frame with device-resident planes filtered in place (zero copy).

The oracle needs ~2-20 s per frame on one host core.
"""
import numpy as np
import pytest

from test_gpu_parity import assert_same_decisions, assert_same_planes
from zenav1_svt_gb300 import abi, synth

pytestmark = pytest.mark.gpu

FULL = [
    ("4k_p4_q24", lambda: synth.workload_4k(4, 24)),
    ("4k_p4_q40", lambda: synth.workload_4k(4, 40)),
    ("4k_p6_q24", lambda: synth.workload_4k(6, 24)),
    ("4k_p6_q40", lambda: synth.workload_4k(6, 40)),
    ("4096x3072_bd10_p2_q28", synth.workload_10bit_4096),
    ("6000x4000_p6_q30", lambda: synth.make_frame(synth.frame_seed(5, 6000), 6000, 4000, 8, 30, 6, "cosine")),
    # 1040 filter blocks at 48 candidates (2304 strength pairs): the cluster
    # joint search's pair-per-thread step at its widest
    ("2560x1664_p0_q36", lambda: synth.make_frame(synth.frame_seed(7, 2560), 2560, 1664, 8, 36, 0, "cosine")),
]


@pytest.mark.parametrize("case", FULL, ids=[c[0] for c in FULL])
def test_full_size_matches_oracle(ctx, oracle, case):
    name, make = case
    fr = make()
    do, so, ro = oracle.filter_stage(fr)
    dg, sg, rg = ctx.filter_stage(fr)
    assert_same_decisions(dg, do)
    assert_same_planes(rg, ro)
    assert sg == so
    if name.startswith("4k_p4") or name.startswith("4096"):
        assert do["lf"][0] > 0  # the level search picks a non-zero level


def batch_slice():
    """24 images of the bench's 256-image batch: the four largest, then
    10-bit and odd-size ones, in batch order."""
    specs = synth.batch_specs(256)
    area = np.array([w * h for w, h, _, _ in specs])
    pick = [int(i) for i in np.argsort(area)[::-1][:4]]
    for i, (w, h, bd, _) in enumerate(specs):
        if len(pick) >= 24:
            break
        if i not in pick and (bd == 10 or (w | h) & 1):
            pick.append(i)
    pick.sort()
    return pick, [synth.batch_frame(i, specs[i]) for i in pick]


def test_bench_batch_slice_matches_oracle(ctx, oracle):
    pick, frames = batch_slice()
    assert any(f.bd == 10 for f in frames) and any((f.true_w | f.true_h) & 1 for f in frames)
    assert max(f.true_w * f.true_h for f in frames) > 3_500_000
    outs = ctx.submit_batch(frames)
    for i, fr, (dg, sg, rg) in zip(pick, frames, outs):
        do, so, ro = oracle.filter_stage(fr)
        assert_same_decisions(dg, do)
        assert_same_planes(rg, ro)
        assert sg == so, i


def test_full_size_device_planes_in_place(pkg, ctx, oracle):
    import torch
    fr = synth.workload_4k(6, 40)
    do, so, ro = oracle.filter_stage(fr)
    dev = torch.device("cuda", 0)
    mi = pkg.pack_geom(fr.geom)
    src = [torch.from_numpy(p.copy()).to(dev) for p in fr.src]
    rec = [torch.from_numpy(p.copy()).to(dev) for p in fr.rec]
    m = torch.from_numpy(mi.view(np.int32).copy()).to(dev)
    s = abi.make_frame_struct(fr, [x.data_ptr() for x in src], [x.data_ptr() for x in rec], m.data_ptr(),
                              on_device=True)
    d = abi.Decisions(fr.w, fr.h, fr.true_w, fr.true_h)
    st = abi.ZfStats()
    torch.cuda.synchronize()
    ctx.filter_stage_raw(s, d, st)
    assert_same_decisions(d.as_dict(), do)
    assert_same_planes([x.cpu().numpy() for x in rec], ro)
    for p in range(3):  # the source is only read
        assert np.array_equal(src[p].cpu().numpy(), fr.src[p])
