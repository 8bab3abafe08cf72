"""Self-guided restoration on the GPU (through the C ABI) vs the CPU
oracle: the per-unit search (best set, weights, SSEs) and the
decoder-exact apply, bit-exact (tolerance zero: the arithmetic is integer).
The reference encoder has no SGRPROJ, so the oracle here is the
specification restatement in oracle/zf_oracle.cpp."""
import zlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def planes(seed, h, w, bd, noise=6.0):
    rng = np.random.default_rng(seed)
    top = (1 << bd) - 1
    yy, xx = np.mgrid[0:h, 0:w]
    base = (top + 1) / 2 + (top + 1) / 5 * np.sin(xx / 11.0 + seed) * np.cos(yy / 13.0) \
        + (top + 1) / 10 * (((xx // 37 + yy // 29) % 2) - 0.5)
    src = np.clip(np.rint(base), 0, top)
    dgd = np.clip(np.rint(src + rng.normal(0, noise * (top + 1) / 256, (h, w))), 0, top)
    pre = np.clip(np.rint(dgd + rng.normal(0, 3 * (top + 1) / 256, (h, w))), 0, top)
    dt = np.uint8 if bd == 8 else np.uint16
    return dgd.astype(dt), src.astype(dt), pre.astype(dt)


CASES = [
    # (name, h, w, bd, ss_y)
    ("luma_small", 70, 90, 8, 0),
    ("luma_units_tails", 530, 700, 8, 0),
    ("chroma_10bit_odd", 389, 523, 10, 1),
    ("tiny", 9, 17, 8, 0),
    ("luma_10bit", 300, 260, 10, 0),
    ("chroma_8bit", 131, 277, 8, 1),
]


def assert_units_equal(g, o):
    for f in ("set", "w0", "w1", "sse", "sse_none"):
        assert (g[f] == o[f]).all(), (f, g[f], o[f])


def assert_planes_equal(a, b):
    if not (a == b).all():
        idx = np.argwhere(a != b)
        raise AssertionError("differs at %d px, first %s: gpu %s oracle %s"
                             % (len(idx), idx[0], a[tuple(idx[0])], b[tuple(idx[0])]))


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_sgr_search_and_apply_match_oracle(ctx, oracle, case):
    name, h, w, bd, ss = case
    dgd, src, pre = planes(zlib.crc32(name.encode()) & 0xffff, h, w, bd)
    ug = ctx.sgr_search(bd, dgd, src, ss_y=ss)
    uo = oracle.sgr_search(bd, dgd, src, ss=ss)
    assert_units_equal(ug, uo)
    # apply the searched units, then a mix: copied units and other sets
    assert_planes_equal(ctx.sgr_apply(bd, dgd, pre, uo, ss_y=ss), oracle.sgr_apply(bd, dgd, pre, uo, ss=ss))
    rng = np.random.default_rng(len(name))
    mix = uo.copy()
    for k in range(len(mix)):
        if k % 3 == 1:
            mix[k]["set"] = -1
        elif k % 3 == 2:
            mix[k]["set"] = rng.integers(0, 16)
            mix[k]["w0"] = rng.integers(-96, 32)
            mix[k]["w1"] = rng.integers(-32, 96)
    assert_planes_equal(ctx.sgr_apply(bd, dgd, pre, mix, ss_y=ss), oracle.sgr_apply(bd, dgd, pre, mix, ss=ss))


def test_sgr_set_masks(ctx, oracle):
    dgd, src, _ = planes(7, 200, 330, 8)
    for mask in (1, 1 << 10, 1 << 15, 0x5A5A, 0xFFFF):
        assert_units_equal(ctx.sgr_search(8, dgd, src, set_mask=mask), oracle.sgr_search(8, dgd, src, set_mask=mask))


def test_sgr_device_planes(ctx, oracle):
    import torch
    dgd, src, pre = planes(9, 280, 300, 10)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(a.astype(np.int16)).to(dev)  # u16 storage, values < 1024
    td, ts, tp = t(dgd), t(src), t(pre)
    ug = ctx.sgr_search(10, td, ts, on_device=True)
    uo = oracle.sgr_search(10, dgd, src)
    assert_units_equal(ug, uo)
    out = torch.empty_like(td)
    ctx.sgr_apply(10, td, tp, uo, dst=out, on_device=True)
    assert_planes_equal(out.cpu().numpy().astype(np.uint16), oracle.sgr_apply(10, dgd, pre, uo))


def test_sgr_argument_errors(ctx, pkg):
    dgd, src, pre = planes(11, 64, 64, 8)
    with pytest.raises(pkg.ZfError) as e:
        ctx.sgr_search(8, dgd, src, set_mask=0)
    assert e.value.kind == "InvalidArgument"
    u = ctx.sgr_search(8, dgd, src)
    bad = u.copy()
    bad[0]["w0"] = 40  # outside [-96, 31]
    with pytest.raises(pkg.ZfError) as e:
        ctx.sgr_apply(8, dgd, pre, bad)
    assert e.value.kind == "InvalidArgument"
    with pytest.raises(pkg.ZfError) as e:
        ctx.sgr_apply(9, dgd, pre, u)
    assert e.value.kind == "UnsupportedConfig"
