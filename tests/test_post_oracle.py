"""Superres and film grain (CPU): the normative upscale table pinned to the
reference's, scaled_size of the library against the oracle, and the
reference's own film-grain unit tests (film_grain.rs tests) restated on the
oracle."""
import os

import numpy as np

from zenav1_svt_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_superres_filter_table_matches_reference(golden):
    hdr = open(os.path.join(ROOT, "include", "zf_av1_tables.h")).read()
    i = hdr.index("#define ZF_SUPERRES_FILTER_INIT")
    j = hdr.index("static const int16_t zf_superres_filter", i)
    import re
    nums = [int(v) for v in re.findall(r"-?\d+", hdr[i + len("#define ZF_SUPERRES_FILTER_INIT"):j])]
    table = [nums[k * 8:(k + 1) * 8] for k in range(64)]
    assert table == golden["tables"]["superres_filter"]
    assert all(sum(r) == 128 for r in table) and table[0] == [0, 0, 0, 128, 0, 0, 0, 0]


def test_scaled_size_library_matches_oracle(pkg, oracle):
    L, O = pkg.lib(), oracle.lib()
    for dim in list(range(1, 300)) + [511, 1024, 1920, 3840, 4096, 16384]:
        for denom in range(8, 18):
            a, b = L.zf_superres_scaled_size(dim, denom), O.zfo_superres_scaled_size(dim, denom)
            assert a == b
            if 9 <= denom <= 16:
                assert 0 < a <= dim and a >= min(16, dim)


def lcg_noisy(clean):
    state = 42
    noisy = clean.astype(np.int32).copy().ravel()
    for k in range(noisy.size):
        state = (state * 1103515245 + 12345) & 0xFFFFFFFF
        noisy[k] = noisy[k] + ((state >> 16) % 41) - 20
    return np.clip(noisy, 0, 255).astype(np.uint8).reshape(clean.shape)


def test_reference_film_grain_unit_tests(oracle):
    frame = np.full((64, 64), 128, np.uint8)
    assert not oracle.film_grain_estimate(frame, frame).apply_grain          # estimate_no_grain_for_identical
    p = oracle.film_grain_estimate(lcg_noisy(frame), frame)                  # estimate_detects_noise
    assert p.apply_grain and p.num_y_points > 0
    f = np.full((16, 16), 128, np.uint8)
    q = abi.ZfFilmGrain()
    q.apply_grain, q.grain_seed, q.num_y_points = 1, 42, 1
    q.point_y_scaling[0] = 20
    assert not (oracle.film_grain_synthesize(f.copy(), q) == f).all()      # synthesize_modifies_frame
    assert (oracle.film_grain_synthesize(f.copy(), abi.ZfFilmGrain()) == f).all()  # no-op when disabled
