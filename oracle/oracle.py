"""ctypes binding of the CPU ORACLE (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline load this
module, as the checker; the product library never calls it.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _pkg():
    import importlib.util
    name = "zenav1_svt_gb300"
    if name in sys.modules:
        return sys.modules[name]
    path = os.path.join(ROOT, "zenav1-svt_gb300", "__init__.py")
    spec = importlib.util.spec_from_file_location(name, path, submodule_search_locations=[os.path.dirname(path)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


abi = _pkg().abi

BORDER_C, BORDER_PORT = 0, 1


class ZfoGeom(C.Structure):
    _fields_ = [("mi_cols", C.c_int32), ("mi_rows", C.c_int32), ("block_id", C.c_void_p),
                ("bw", C.c_void_p), ("bh", C.c_void_p), ("tw", C.c_void_p), ("th", C.c_void_p),
                ("skip", C.c_void_p), ("skip_inter", C.c_void_p)]


_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    sys.path.insert(0, HERE)
    import build as obuild  # oracle/build.py
    sys.path.pop(0)
    path = obuild.build()
    L = C.CDLL(path)
    P = C.POINTER
    L.zfo_filter_stage.argtypes = [P(abi.ZfFrame), P(ZfoGeom), P(abi.ZfDecisions), P(abi.ZfStats), C.c_int32]
    L.zfo_deblock_pick.argtypes = [P(abi.ZfFrame), P(ZfoGeom), P(C.c_uint8)]
    L.zfo_deblock_apply.argtypes = [P(abi.ZfFrame), P(ZfoGeom), P(C.c_uint8)]
    L.zfo_deblock_sse_table.argtypes = [P(abi.ZfFrame), P(ZfoGeom), C.c_int32, C.c_void_p, C.c_int32, C.c_void_p]
    L.zfo_trace.argtypes = [C.c_char_p]
    L.zfo_trace.restype = None
    L.zfo_cdef_search.argtypes = [P(abi.ZfFrame), P(ZfoGeom), P(abi.ZfDecisions), C.c_void_p, C.c_void_p,
                                  P(C.c_int32)]
    L.zfo_cdef_apply.argtypes = [P(abi.ZfFrame), P(ZfoGeom), P(abi.ZfDecisions), P(abi.ZfStats)]
    L.zfo_lr_search.argtypes = [P(abi.ZfFrame), P(abi.ZfDecisions), C.c_int32]
    L.zfo_lr_apply.argtypes = [P(abi.ZfFrame), P(C.c_void_p), P(abi.ZfDecisions), C.c_int32]
    L.zfo_lf_thresholds.argtypes = [C.c_int32, C.c_int32, P(C.c_int32)]
    L.zfo_lpf.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
    L.zfo_cdef_find_dir.argtypes = [C.c_void_p, C.c_int32, C.c_int32, P(C.c_int32), P(C.c_int32)]
    L.zfo_cdef_filter_block.argtypes = [C.c_void_p] + [C.c_int32] * 3 + [C.c_void_p] + [C.c_int32] * 9
    L.zfo_adjust_strength.argtypes = [C.c_int32, C.c_int32]
    L.zfo_cdef_finish_rd.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, P(C.c_int32),
                                     P(C.c_int32)]
    L.zfo_cdef_qp_params.argtypes = [C.c_int32, C.c_int32, C.c_int32, P(C.c_int32)]
    L.zfo_deblock_key_frame_levels.argtypes = [C.c_int32, C.c_int32, P(C.c_uint8)]
    L.zfo_dlf_hillclimb_replay.argtypes = [P(C.c_int64), C.c_int32, P(C.c_int32), P(C.c_int32)]
    L.zfo_lambda.argtypes = [C.c_int32, C.c_int32]
    L.zfo_lambda.restype = C.c_uint32
    L.zfo_compute_stats.argtypes = [C.c_int32, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_int64,
                                    C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                    C.c_void_p, C.c_int32]
    L.zfo_wiener_solve.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, P(C.c_int32), P(C.c_int32),
                                   P(C.c_int16), P(C.c_int16)]
    L.zfo_wiener_solve.restype = C.c_int64
    L.zfo_count_wiener_bits.argtypes = [C.c_int32] + [P(C.c_int16)] * 4
    L.zfo_count_units_in_tile.argtypes = [C.c_int32, C.c_int32]
    L.zfo_rdcost_dbl.argtypes = [C.c_int64, C.c_int64, C.c_int64]
    L.zfo_rdcost_dbl.restype = C.c_double
    L.zfo_wiener_convolve.argtypes = [C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_int64, C.c_int32,
                                      P(C.c_int16), P(C.c_int16), C.c_int32, C.c_int32, C.c_int32]
    L.zfo_sse_region.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
    L.zfo_sse_region.restype = C.c_int64
    L.zfo_sgr_search.argtypes = [C.c_int32] * 4 + [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]
    L.zfo_sgr_apply.argtypes = [C.c_int32] * 4 + [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.zfo_sgr_box_filter.argtypes = [C.c_int32] * 3 + [C.c_void_p] + [C.c_int32] * 6 + [C.c_void_p]
    L.zfo_sgr_params.argtypes = [C.c_int32, P(C.c_int32)]
    L.zfo_superres_scaled_size.argtypes = [C.c_int32, C.c_int32]
    L.zfo_superres_upscale.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.c_int32,
                                       C.c_int32, C.c_int32]
    L.zfo_superres_upscale.restype = None
    L.zfo_film_grain_estimate.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                          P(abi.ZfFilmGrain)]
    L.zfo_film_grain_estimate.restype = None
    L.zfo_film_grain_synthesize.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, P(abi.ZfFilmGrain)]
    L.zfo_film_grain_synthesize.restype = None
    L.zfo_write_filter_params.argtypes = [P(abi.ZfDecisions), P(abi.ZfHeaderOpts), C.c_void_p, C.c_int32,
                                          P(C.c_int32)]
    _lib = L
    return L


def geom_struct(geom):
    arrs = geom.arrays()
    g = ZfoGeom()
    g.mi_cols, g.mi_rows = geom.mi_cols, geom.mi_rows
    g.block_id, g.bw, g.bh, g.tw, g.th, g.skip, g.skip_inter = [a.ctypes.data for a in arrs]
    g._keep = arrs
    return g


def _frame(fr, rec):
    mi = np.zeros(1, np.uint32)  # the oracle reads the explicit geometry
    s = abi.make_frame_struct(fr, fr.src, rec, mi)
    s._keep = mi
    return s


def filter_stage(fr, rec=None, border=BORDER_C):
    rec = fr.copy_rec() if rec is None else rec
    g = geom_struct(fr.geom)
    s = _frame(fr, rec)
    d = abi.Decisions(fr.w, fr.h, fr.true_w, fr.true_h)
    st = abi.ZfStats()
    rc = lib().zfo_filter_stage(C.byref(s), C.byref(g), C.byref(d.c), C.byref(st), border)
    assert rc == 0, rc
    return d.as_dict(), {"cdef_filtered_px": st.cdef_filtered_px, "cdef_changed_px": st.cdef_changed_px,
                         "cdef_sb_count": st.cdef_sb_count, "lr_wiener_units": st.lr_wiener_units,
                         "lr_frame_rtype": list(st.lr_frame_rtype)}, rec


def stage_decisions(fr):
    """The oracle's whole-stage decisions as an abi.Decisions (the
    zf_decisions struct with its caller arrays), for the syntax writers."""
    g = geom_struct(fr.geom)
    rec = fr.copy_rec()  # held here: the frame struct only points at it
    s = _frame(fr, rec)
    d = abi.Decisions(fr.w, fr.h, fr.true_w, fr.true_h)
    st = abi.ZfStats()
    assert lib().zfo_filter_stage(C.byref(s), C.byref(g), C.byref(d.c), C.byref(st), BORDER_C) == 0
    return d


def deblock_pick(fr, rec):
    g = geom_struct(fr.geom)
    s = _frame(fr, rec)
    lf = (C.c_uint8 * 4)()
    assert lib().zfo_deblock_pick(C.byref(s), C.byref(g), lf) == 0
    return list(lf)


def deblock_sse_table(fr, plane, levels, rec=None):
    """try_filter_plane's SSE of one plane at each level (int64 array)."""
    rec = fr.rec if rec is None else rec
    g = geom_struct(fr.geom)
    s = _frame(fr, rec)
    lv = np.ascontiguousarray(levels, np.int32)
    out = np.zeros(len(lv), np.int64)
    assert lib().zfo_deblock_sse_table(C.byref(s), C.byref(g), plane, lv.ctypes.data, len(lv), out.ctypes.data) == 0
    return out


def trace(path):
    """Write the search trace lines to path (None stops)."""
    lib().zfo_trace(None if path is None else path.encode())


def deblock_apply(fr, rec, lf):
    g = geom_struct(fr.geom)
    s = _frame(fr, rec)
    assert lib().zfo_deblock_apply(C.byref(s), C.byref(g), (C.c_uint8 * 4)(*lf)) == 0


def cdef_search(fr, rec):
    """Returns (Decisions, mse rows [nfb, 2*ncand] or None, has_row [nfb])."""
    g = geom_struct(fr.geom)
    s = _frame(fr, rec)
    d = abi.Decisions(fr.w, fr.h, fr.true_w, fr.true_h)
    nfb = d.nhfb * d.nvfb
    mse = np.zeros((nfb, 2 * 48), np.uint64)
    has = np.zeros(nfb, np.uint8)
    nc = C.c_int32()
    # the oracle writes rows with stride 2*ncand; pass a scratch and reshape.
    flat = np.zeros(nfb * 2 * 48, np.uint64)
    assert lib().zfo_cdef_search(C.byref(s), C.byref(g), C.byref(d.c), flat.ctypes.data, has.ctypes.data,
                                 C.byref(nc)) == 0
    n = nc.value
    rows = flat[:nfb * 2 * n].reshape(nfb, 2 * n) if n else None
    del mse
    return d, rows, has


def cdef_apply(fr, rec, dec):
    g = geom_struct(fr.geom)
    s = _frame(fr, rec)
    st = abi.ZfStats()
    assert lib().zfo_cdef_apply(C.byref(s), C.byref(g), C.byref(dec.c), C.byref(st)) == 0
    return {"cdef_filtered_px": st.cdef_filtered_px, "cdef_changed_px": st.cdef_changed_px}


def lr_search(fr, rec, border=BORDER_C):
    s = _frame(fr, rec)
    d = abi.Decisions(fr.w, fr.h, fr.true_w, fr.true_h)
    assert lib().zfo_lr_search(C.byref(s), C.byref(d.c), border) == 0
    return d


def lr_apply(fr, rec, pre_cdef, dec, border=BORDER_C):
    s = _frame(fr, rec)
    pre = (C.c_void_p * 3)(*[p.ctypes.data for p in pre_cdef])
    assert lib().zfo_lr_apply(C.byref(s), pre, C.byref(dec.c), border) == 0


# Self-guided restoration (AV1 spec 7.17.3; the reference encoder has none).
SGR_UNIT = np.dtype([("set", np.int32), ("w0", np.int32), ("w1", np.int32), ("pad", np.int32),
                     ("sse", np.int64), ("sse_none", np.int64)])


def sgr_units_shape(pw, ph):
    L = lib()
    return L.zfo_count_units_in_tile(256, pw) * L.zfo_count_units_in_tile(256, ph)


def sgr_search(bd, dgd, src, ss=0, set_mask=0xFFFF):
    """Per restoration unit of the plane: best set of the mask, weights, SSEs."""
    ph, pw = dgd.shape
    dgd, src = np.ascontiguousarray(dgd), np.ascontiguousarray(src)
    units = np.zeros(sgr_units_shape(pw, ph), SGR_UNIT)
    assert lib().zfo_sgr_search(bd, pw, ph, ss, dgd.ctypes.data, src.ctypes.data, set_mask, units.ctypes.data) == 0
    return units


def sgr_apply(bd, dgd, pre_cdef, units, ss=0):
    """Decoder-exact SGRPROJ apply of one plane (units with set < 0 copy)."""
    ph, pw = dgd.shape
    dgd, pre_cdef = np.ascontiguousarray(dgd), np.ascontiguousarray(pre_cdef)
    units = np.ascontiguousarray(units, SGR_UNIT)
    out = np.empty_like(dgd)
    assert lib().zfo_sgr_apply(bd, pw, ph, ss, dgd.ctypes.data, pre_cdef.ctypes.data, units.ctypes.data,
                               out.ctypes.data) == 0
    return out


def sgr_box_filter(bd, dgd, set_, pass_, x, y, w, h):
    ph, pw = dgd.shape
    dgd = np.ascontiguousarray(dgd)
    out = np.zeros((h, w), np.int32)
    lib().zfo_sgr_box_filter(bd, pw, ph, dgd.ctypes.data, set_, pass_, x, y, w, h, out.ctypes.data)
    return out


def sgr_params(set_):
    out = (C.c_int32 * 4)()
    lib().zfo_sgr_params(set_, out)
    return list(out)


def write_filter_params(dec, opts, nbytes=64):
    """Bits of loop_filter_params / cdef_params / lr_params as a '0'/'1' string."""
    buf = np.zeros(nbytes, np.uint8)
    pos = C.c_int32(0)
    rc = lib().zfo_write_filter_params(C.byref(dec), C.byref(opts), buf.ctypes.data, nbytes, C.byref(pos))
    assert rc == 0, rc
    return "".join(str((buf[i >> 3] >> (7 - (i & 7))) & 1) for i in range(pos.value))


def superres_upscale(src, dst_width, bd=8):
    rows, w = src.shape
    src = np.ascontiguousarray(src)
    dst = np.empty((rows, dst_width), src.dtype)
    lib().zfo_superres_upscale(src.ctypes.data, w, w, dst.ctypes.data, dst_width, dst_width, rows, bd)
    return dst


def film_grain_estimate(src, recon):
    h, w = src.shape
    p = abi.ZfFilmGrain()
    lib().zfo_film_grain_estimate(np.ascontiguousarray(src).ctypes.data, np.ascontiguousarray(recon).ctypes.data,
                                  w, h, w, C.byref(p))
    return p


def film_grain_synthesize(frame, params):
    h, w = frame.shape
    lib().zfo_film_grain_synthesize(frame.ctypes.data, w, h, w, C.byref(params))
    return frame
