"""Self-guided restoration oracle (CPU): properties of the AV1 box filter and
projection, and the search's consistency. The reference encoder never
searches or signals SGRPROJ, so nothing here is pinned to it; these checks
hold the restatement of the specification to its own identities."""
import numpy as np
import pytest


def planes(seed, h, w, bd, noise=6.0):
    rng = np.random.default_rng(seed)
    top = (1 << bd) - 1
    yy, xx = np.mgrid[0:h, 0:w]
    base = (top + 1) / 2 + (top + 1) / 6 * np.sin(xx / 9.0 + 0.3 * seed) + (top + 1) / 8 * np.cos(yy / 7.0)
    src = np.clip(np.rint(base), 0, top)
    dgd = np.clip(np.rint(src + rng.normal(0, noise * (top + 1) / 256, (h, w))), 0, top)
    dt = np.uint8 if bd == 8 else np.uint16
    return dgd.astype(dt), src.astype(dt)


def test_sgr_params_scale_formula(oracle):
    # s = ((1 << 20) + n^2 eps / 2) / (n^2 eps), radii 2/1 or a disabled pass
    for k in range(16):
        r0, s0, r1, s1 = oracle.sgr_params(k)
        assert r0 in (0, 2) and r1 in (0, 1) and (r0 or r1)
        for r, s in ((r0, s0), (r1, s1)):
            if r == 0:
                assert s == -1
            else:
                assert s > 0


@pytest.mark.parametrize("bd", [8, 10])
def test_box_filter_flat_plane(oracle, bd):
    c = 100 << (bd - 8)
    flat = np.full((24, 24), c, np.uint8 if bd == 8 else np.uint16)
    for k in range(16):
        for p in range(2):
            f = oracle.sgr_box_filter(bd, flat, k, p, 4, 4, 8, 8)
            if oracle.sgr_params(k)[2 * p] == 0:
                assert (f == 0).all()
            else:  # a flat window filters to the sample (x16) up to the spec's rounding
                assert np.abs(f - 16 * c).max() <= 2 << (bd - 8)


@pytest.mark.parametrize("bd", [8, 10])
def test_identity_weights_and_copy_units(oracle, bd):
    dgd, src = planes(1, 70, 90, bd)
    pre = dgd.copy()
    u = np.zeros(oracle.sgr_units_shape(90, 70), oracle.SGR_UNIT)
    u["set"] = -1
    assert (oracle.sgr_apply(bd, dgd, pre, u) == dgd).all()
    # sets 14 / 15 have no radius-1 pass: w0 = 0 leaves 128 * u
    for k in (14, 15):
        u["set"], u["w0"], u["w1"] = k, 0, 37
        assert (oracle.sgr_apply(bd, dgd, pre, u) == dgd).all()


@pytest.mark.parametrize("bd", [8, 10])
def test_search_is_min_over_sets(oracle, bd):
    dgd, src = planes(2, 40, 700, bd)  # three units across: 256, 256 and a 188-column tail
    full = oracle.sgr_search(bd, dgd, src)
    per = np.stack([oracle.sgr_search(bd, dgd, src, set_mask=1 << k) for k in range(16)])
    for u in range(len(full)):
        sse = per[:, u]["sse"]
        k = int(np.argmin(sse))  # first minimum: the lowest set on ties
        assert full[u]["set"] == k and full[u]["sse"] == sse[k]
        assert full[u]["w0"] == per[k, u]["w0"] and full[u]["w1"] == per[k, u]["w1"]
        cols = slice(256 * u, 256 * (u + 1) if u < 2 else 700)
        assert full[u]["sse_none"] == ((dgd.astype(np.int64) - src) ** 2)[:, cols].sum()
    assert len(full) == 3 and (full["sse"] < full["sse_none"]).all()  # noisy input: the projection helps


@pytest.mark.parametrize("bd", [8, 10])
def test_search_sse_equals_apply_within_one_stripe(oracle, bd):
    # One stripe (rows < 56) and pre_cdef == dgd: the decoder's fetch equals
    # the search's clamped fetch, so the applied unit has the searched SSE.
    dgd, src = planes(3, 50, 120, bd)
    u = oracle.sgr_search(bd, dgd, src)
    out = oracle.sgr_apply(bd, dgd, dgd, u)
    assert ((out.astype(np.int64) - src) ** 2).sum() == u[0]["sse"]


def test_apply_reads_pre_cdef_only_across_stripes(oracle):
    # rows of the pre-CDEF plane matter only within 2 rows... of interior
    # stripe edges (luma edges at 56, 120, ...): changing pre_cdef elsewhere
    # leaves the output alone
    dgd, src = planes(4, 130, 80, 8)
    u = oracle.sgr_search(8, dgd, src)
    pre = dgd.copy()
    a = oracle.sgr_apply(8, dgd, pre, u)
    far = pre.copy()
    far[:50] ^= 0x55
    far[62:114] ^= 0x33
    assert (oracle.sgr_apply(8, dgd, far, u) == a).all()
    near = pre.copy()
    near[54:58] ^= 0x55
    assert not (oracle.sgr_apply(8, dgd, near, u) == a).all()
