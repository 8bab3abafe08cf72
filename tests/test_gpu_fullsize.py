"""Full-size parity: the plain per-image 4K configuration (3840x2160 8-bit,
preset 4 with the deblock level search, qp 24; preset 6, qp 40) and the
10-bit high-resolution configuration (4096x3072 10-bit, preset 2 with 20
CDEF candidates and the Wiener refinement, qp 28) through the C ABI against
the oracle, bit-exact on every plane and decision. Also the 4K frame with
device-resident planes (the zero-copy path, in place on the caller's
buffers). The oracle needs ~5-15 s per frame on one host core."""
import numpy as np
import pytest

from test_gpu_parity import assert_same_decisions, assert_same_planes
from zenav1_svt_gb300 import abi, synth

pytestmark = pytest.mark.gpu

FULL = [
    # (name, seed, w, h, bd, qp, preset, content)
    ("4k_p4_q24", synth.frame_seed(2, 0), 3840, 2160, 8, 24, 4, "power"),
    ("4k_p6_q40", synth.frame_seed(2, 3), 3840, 2160, 8, 40, 6, "power"),
    ("4096x3072_bd10_p2_q28", synth.frame_seed(3, 0), 4096, 3072, 10, 28, 2, "power10"),
]


@pytest.mark.parametrize("case", FULL, ids=[c[0] for c in FULL])
def test_full_size_matches_oracle(ctx, oracle, case):
    name, seed, w, h, bd, qp, preset, content = case
    fr = synth.make_frame(seed, w, h, bd, qp, preset, content)
    do, so, ro = oracle.filter_stage(fr)
    dg, sg, rg = ctx.filter_stage(fr)
    assert_same_decisions(dg, do)
    assert_same_planes(rg, ro)
    assert sg == so


def test_full_size_device_planes_in_place(pkg, ctx, oracle):
    import torch
    fr = synth.make_frame(synth.frame_seed(2, 3), 3840, 2160, 8, 40, 6, "power")
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
