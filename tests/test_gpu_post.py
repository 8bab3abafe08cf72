"""Superres upscale and film grain on the GPU (through the C ABI) vs the CPU
oracle, bit-exact (integer arithmetic; the film-grain variance and its
scaling point are the same double-precision operations on the host)."""
import ctypes as C

import numpy as np
import pytest

from zenav1_svt_gb300 import abi

pytestmark = pytest.mark.gpu


def contents(width, bd=8):
    rng = np.random.default_rng(width)
    top = (1 << bd) - 1
    return {
        "step": np.where(np.arange(width) < width // 2, 16 << (bd - 8), 235 << (bd - 8)),
        "ramp": np.arange(width) * top // max(width, 1),
        "noise": rng.integers(0, top + 1, width),
        "edges": np.where((np.arange(width) == 0) | (np.arange(width) == width - 1), top, 0),
    }


def test_superres_rows_across_denominators(ctx, oracle, pkg):
    # the reference's sweep shape (c_parity_superres.rs): frame widths x
    # denominators 9..16 x four row contents
    cells = 0
    for frame_w in (64, 96, 128, 176, 256, 320, 512, 1920):
        for denom in range(9, 17):
            coded = pkg.lib().zf_superres_scaled_size(frame_w, denom)
            rows = np.stack([v.astype(np.uint8) for v in contents(coded).values()])
            g = ctx.superres_upscale(rows, frame_w)
            o = oracle.superres_upscale(rows, frame_w)
            assert (g == o).all(), (frame_w, denom)
            cells += rows.shape[0]
    assert cells >= 200


def test_superres_plane_10bit(ctx, oracle, pkg):
    rng = np.random.default_rng(3)
    for frame_w, denom, rows in ((1000, 13, 37), (4096, 16, 9), (77, 9, 5)):
        coded = pkg.lib().zf_superres_scaled_size(frame_w, denom)
        src = rng.integers(0, 1024, (rows, coded)).astype(np.uint16)
        assert (ctx.superres_upscale(src, frame_w, bit_depth=10) == oracle.superres_upscale(src, frame_w, bd=10)).all()
        s8 = rng.integers(0, 256, (rows, coded)).astype(np.uint8)
        assert (ctx.superres_upscale(s8, frame_w) == oracle.superres_upscale(s8, frame_w)).all()


def grain_fields(p):
    return {f: (list(getattr(p, f)) if hasattr(getattr(p, f), "__len__") else getattr(p, f))
            for f, _ in abi.ZfFilmGrain._fields_}


@pytest.mark.parametrize("shape,noise", [((64, 64), 0), ((64, 64), 20), ((1080, 1920), 6), ((37, 129), 9),
                                         ((2160, 3840), 2)])
def test_film_grain_estimate_matches_oracle(ctx, oracle, shape, noise):
    rng = np.random.default_rng(shape[0] + noise)
    clean = rng.integers(40, 216, shape).astype(np.uint8)
    src = np.clip(clean.astype(np.int32) + rng.integers(-noise, noise + 1, shape), 0, 255).astype(np.uint8)
    g, o = ctx.film_grain_estimate(src, clean), oracle.film_grain_estimate(src, clean)
    assert grain_fields(g) == grain_fields(o)
    assert bool(g.apply_grain) == (noise >= 4)


@pytest.mark.parametrize("shape,scaling", [((16, 16), 20), ((301, 517), 7), ((1080, 1920), 33), ((5, 3), 0)])
def test_film_grain_synthesize_matches_oracle(ctx, oracle, shape, scaling):
    rng = np.random.default_rng(scaling)
    frame = rng.integers(0, 256, shape).astype(np.uint8)
    p = abi.ZfFilmGrain()
    p.apply_grain, p.grain_seed, p.num_y_points = 1, 42 + scaling, 2
    p.point_y_scaling[0] = scaling
    g = ctx.film_grain_synthesize(frame.copy(), p)
    o = oracle.film_grain_synthesize(frame.copy(), p)
    assert (g == o).all()


def test_film_grain_strided_planes(ctx, oracle, pkg):
    # rows padded past the width (stride > width): the row-block path
    rng = np.random.default_rng(5)
    h, w, stride = 133, 250, 272
    clean = rng.integers(40, 216, (h, stride)).astype(np.uint8)
    src = np.clip(clean.astype(np.int32) + rng.integers(-7, 8, (h, stride)), 0, 255).astype(np.uint8)
    g, o = abi.ZfFilmGrain(), abi.ZfFilmGrain()
    ctx._check(pkg.lib().zf_film_grain_estimate(ctx.h, src.ctypes.data, clean.ctypes.data, w, h, stride, 0,
                                                C.byref(g)))
    oracle.lib().zfo_film_grain_estimate(src.ctypes.data, clean.ctypes.data, w, h, stride, C.byref(o))
    assert grain_fields(g) == grain_fields(o)
    frame = clean.copy()
    p = abi.ZfFilmGrain()
    p.apply_grain, p.grain_seed, p.num_y_points = 1, 7, 1
    p.point_y_scaling[0] = 12
    a, b = frame.copy(), frame.copy()
    ctx._check(pkg.lib().zf_film_grain_synthesize(ctx.h, a.ctypes.data, w, h, stride, 0, C.byref(p)))
    oracle.lib().zfo_film_grain_synthesize(b.ctypes.data, w, h, stride, C.byref(p))
    assert (a == b).all() and (a[:, w:] == frame[:, w:]).all()
