"""C-ABI surface on the CPU: the library loads, exports every entry point
declared in include/zf_filter.h, and its host-only functions (geometry
packing, size queries, argument validation) behave without a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from zenav1_svt_gb300 import abi, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            syms += re.findall(r"^\s*(?:int32_t|uint64_t|void|const char \*)\s*\**\s*(zf_\w+)\s*\(", txt, re.M)
    return sorted(set(syms))


def test_library_exports_every_declared_symbol(pkg):
    L = pkg.lib()
    syms = declared_symbols()
    assert len(syms) >= 14
    for s in syms:
        assert hasattr(L, s), s
    assert L.zf_abi_version() == 2


def test_pack_geom_roundtrip_and_rejects_misaligned(pkg):
    fr = synth.make_frame(7, 96, 64, 8, 30, 6, "cosine")
    mi = pkg.pack_geom(fr.geom)
    g = fr.geom
    bw = 4 << (mi & 7)
    assert (bw.reshape(g.bw.shape) == g.bw).all()
    assert (((mi >> 12) & 1).reshape(g.skip.shape) == g.skip).all()
    bad = synth.Geometry(96, 64)
    for y in range(0, 64, 8):
        for x in range(0, 96, 8):
            bad.record_block(x, y, 8, 8, False, 0)
    bad.block_id[0, 1] = 5  # not the aligned origin
    with pytest.raises(pkg.ZfError) as e:
        pkg.pack_geom(bad)
    assert e.value.kind == "InvalidGeometry"


def test_query_sizes(pkg):
    fr = synth.make_frame(7, 1000, 600, 8, 30, 6, "cosine")
    z = pkg.query_sizes(fr)
    assert (z.nhfb, z.nvfb) == (16, 10)
    assert list(z.lr_hunits) == [abi.count_units(1000), abi.count_units(500), abi.count_units(500)]
    assert z.device_bytes > 3 * 1000 * 600


def test_invalid_dimensions_rejected(pkg):
    fr = synth.make_frame(7, 64, 64, 8, 30, 6, "cosine")
    mi = pkg.pack_geom(fr.geom)
    s = abi.make_frame_struct(fr, fr.src, fr.rec, mi)
    s.width = 66
    z = abi.ZfSizes()
    assert pkg.lib().zf_query_sizes(C.byref(s), C.byref(z)) == -2
    s.width = 64
    s.bit_depth = 12
    assert pkg.lib().zf_query_sizes(C.byref(s), C.byref(z)) == -3
