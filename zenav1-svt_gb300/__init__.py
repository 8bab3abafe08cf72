"""GB300 in-loop filter stage for the zenav1-svt AV1 still-image encoder.

Python binding of the C ABI in include/zf_filter.h (libzf.so, built by
build.py). The functions mirror the reference encoder's filter-stage entry
points (rust/crates/svtav1-encoder/src/{deblock,cdef,restoration}.rs) with
the same argument meaning and the same error behaviour (the EncodeError
variants surface as ZfError with the reference's variant name):

  pick_filter_levels        deblock::pick_filter_levels_full_search /
                            pick_filter_levels_key_frame      (deblock.rs:481, :55)
  apply_deblock_frame       deblock::apply_deblock_frame[_hbd] (deblock.rs:938, :976)
  cdef_search_still         the CDEF pick of pipeline.rs:3042-3144
  apply_cdef_frame          cdef::apply_cdef_frame[_hbd]      (cdef.rs:343, :556)
  search_restoration_still  restoration::search_restoration_still[_bd]
  apply_restoration_frame   restoration::save_lr_boundaries +
                            apply_restoration_frame           (restoration.rs:938, :992)
  filter_stage              the whole stage (pipeline.rs:2886-3455)
  submit_batch              many frames, one launch per pass
  sgr_search / sgr_apply    self-guided restoration (AV1 spec 7.17.3); the
                            reference encoder never searches SGRPROJ

There is no CPU fallback: every call runs the CUDA kernels, and loading
fails loudly when the library has not been built.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from .abi import Decisions, ZfDecisions, ZfFrame, ZfOpts, ZfSizes, ZfStats

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libzf.so")

_lib = None


class ZfError(RuntimeError):
    def __init__(self, code, msg=""):
        self.code = code
        self.kind = abi.ERRORS.get(code, "Unknown")
        super().__init__("%s (%d): %s" % (self.kind, code, msg))


def lib():
    """Load libzf.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libzf.so is not built (%s); run __graft_entry__.build() or "
                           "python zenav1-svt_gb300/build.py" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    P = C.POINTER
    L.zf_abi_version.restype = C.c_int32
    L.zf_create.argtypes = [P(C.c_void_p), P(ZfOpts)]
    L.zf_destroy.argtypes = [C.c_void_p]
    L.zf_destroy.restype = None
    L.zf_last_error.argtypes = [C.c_void_p]
    L.zf_last_error.restype = C.c_char_p
    L.zf_sync.argtypes = [C.c_void_p]
    L.zf_query_sizes.argtypes = [P(ZfFrame), P(ZfSizes)]
    L.zf_pack_geom.argtypes = [C.c_int32, C.c_int32] + [C.c_void_p] * 8
    L.zf_filter_stage.argtypes = [C.c_void_p, P(ZfFrame), P(ZfDecisions), P(ZfStats)]
    L.zf_submit_batch.argtypes = [C.c_void_p, P(ZfFrame), C.c_int32, P(ZfDecisions), P(ZfStats)]
    L.zf_deblock_pick.argtypes = [C.c_void_p, P(ZfFrame), P(C.c_uint8)]
    L.zf_deblock_apply.argtypes = [C.c_void_p, P(ZfFrame), P(C.c_uint8)]
    L.zf_deblock_sse_table.argtypes = [C.c_void_p, P(ZfFrame), C.c_int32, C.c_void_p, C.c_int32, C.c_void_p]
    L.zf_cdef_search_rows.argtypes = [C.c_void_p, P(ZfFrame), P(ZfDecisions), C.c_void_p, C.c_void_p,
                                      P(C.c_int32)]
    L.zf_trace.argtypes = [C.c_void_p, C.c_char_p]
    L.zf_set_wait_limit.argtypes = [C.c_void_p, C.c_uint32]
    L.zf_cdef_search.argtypes = [C.c_void_p, P(ZfFrame), P(ZfDecisions)]
    L.zf_cdef_apply.argtypes = [C.c_void_p, P(ZfFrame), P(ZfDecisions), P(ZfStats)]
    L.zf_lr_search.argtypes = [C.c_void_p, P(ZfFrame), P(ZfDecisions)]
    L.zf_lr_apply.argtypes = [C.c_void_p, P(ZfFrame), P(C.c_void_p), P(ZfDecisions)]
    L.zf_stream.argtypes = [C.c_void_p]
    L.zf_stream.restype = C.c_void_p
    L.zf_launch_count.argtypes = [C.c_void_p]
    L.zf_launch_count.restype = C.c_uint64
    L.zf_device_bytes.argtypes = [C.c_void_p]
    L.zf_device_bytes.restype = C.c_uint64
    L.zf_trim.argtypes = [C.c_void_p]
    L.zf_trim.restype = C.c_int32
    L.zf_reserve.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64]
    L.zf_reserve.restype = C.c_int32
    L.zf_profile_enable.argtypes = [C.c_void_p, C.c_int32]
    L.zf_profile_reset.argtypes = [C.c_void_p]
    L.zf_profile_reset.restype = None
    L.zf_profile_read.argtypes = [C.c_void_p, C.c_void_p, C.c_int32]
    L.zf_profile_read.restype = C.c_int32
    L.zf_sgr_search.argtypes = [C.c_void_p, P(abi.ZfSgrPlane), C.c_uint32, C.c_void_p, C.c_int32]
    L.zf_sgr_apply.argtypes = [C.c_void_p, P(abi.ZfSgrPlane), C.c_void_p, C.c_int32, C.c_void_p]
    L.zf_write_filter_params.argtypes = [P(ZfDecisions), P(abi.ZfHeaderOpts), C.c_void_p, C.c_int32,
                                         P(C.c_int32)]
    L.zf_use_graphs.argtypes = [C.c_void_p, C.c_int32]
    L.zf_wiener_refs_reset.argtypes = [P(abi.ZfWienerRefs)]
    L.zf_wiener_refs_reset.restype = None
    L.zf_lr_corners_in_sb.argtypes = [C.c_int32] * 8 + [P(C.c_int32)]
    L.zf_lr_sb_syntax.argtypes = [P(ZfDecisions)] + [C.c_int32] * 7 + [P(abi.ZfWienerRefs), P(abi.ZfLrSym),
                                                                     C.c_int32]
    L.zf_ec_create.argtypes = []
    L.zf_ec_create.restype = C.c_void_p
    L.zf_ec_destroy.argtypes = [C.c_void_p]
    L.zf_ec_destroy.restype = None
    L.zf_ec_reset.argtypes = [C.c_void_p]
    L.zf_ec_reset.restype = None
    L.zf_ec_bool.argtypes = [C.c_void_p, C.c_int32, C.c_uint32]
    L.zf_ec_literal.argtypes = [C.c_void_p, C.c_uint32, C.c_int32]
    L.zf_ec_symbol.argtypes = [C.c_void_p, C.c_int32, P(C.c_uint16), C.c_int32, C.c_int32]
    L.zf_ec_tell.argtypes = [C.c_void_p]
    L.zf_ec_done.argtypes = [C.c_void_p, C.c_void_p, C.c_int32]
    L.zf_wiener_restore_cdf_init.argtypes = [P(C.c_uint16)]
    L.zf_wiener_restore_cdf_init.restype = None
    L.zf_ec_lr_syms.argtypes = [C.c_void_p, P(abi.ZfLrSym), C.c_int32, P(C.c_uint16)]
    L.zf_ec_lr_sb.argtypes = [C.c_void_p, P(ZfDecisions)] + [C.c_int32] * 7 + [P(abi.ZfWienerRefs),
                                                                             P(C.c_uint16)]
    L.zf_cdef_sb_begin.argtypes = [P(ZfDecisions), C.c_int32, C.c_int32, C.c_int32, P(abi.ZfCdefSb)]
    L.zf_ec_cdef_block.argtypes = [C.c_void_p, P(abi.ZfCdefSb), C.c_int32, C.c_int32, C.c_int32]
    L.zf_get_tune.argtypes = [C.c_void_p, P(abi.ZfTune)]
    L.zf_set_tune.argtypes = [C.c_void_p, P(abi.ZfTune)]
    L.zf_autotune.argtypes = [C.c_void_p, P(ZfFrame), C.c_int32, C.c_int32, P(abi.ZfTune), P(abi.ZfTune),
                              C.c_int32]
    L.zf_graph_stats.argtypes = [C.c_void_p, P(C.c_uint64)]
    L.zf_superres_scaled_size.argtypes = [C.c_int32, C.c_int32]
    L.zf_superres_upscale.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_int32,
                                      C.c_int32, C.c_int32, C.c_int32, C.c_int32]
    L.zf_film_grain_estimate.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                                         C.c_int32, P(abi.ZfFilmGrain)]
    L.zf_film_grain_synthesize.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                           P(abi.ZfFilmGrain)]
    for name in ("zf_lr_corners_in_sb", "zf_lr_sb_syntax", "zf_get_tune", "zf_set_tune", "zf_autotune", "zf_use_graphs", "zf_graph_stats", "zf_superres_scaled_size", "zf_superres_upscale", "zf_film_grain_estimate",
                 "zf_film_grain_synthesize", "zf_write_filter_params", "zf_sgr_search", "zf_sgr_apply", "zf_create", "zf_sync", "zf_query_sizes", "zf_pack_geom", "zf_filter_stage",
                 "zf_submit_batch", "zf_deblock_pick", "zf_deblock_apply", "zf_cdef_search",
                 "zf_deblock_sse_table", "zf_cdef_search_rows", "zf_trace", "zf_set_wait_limit",
                 "zf_cdef_apply", "zf_lr_search", "zf_lr_apply", "zf_ec_bool", "zf_ec_literal", "zf_ec_symbol",
                 "zf_ec_tell", "zf_ec_done", "zf_ec_lr_syms", "zf_ec_lr_sb", "zf_cdef_sb_begin", "zf_ec_cdef_block"):
        getattr(L, name).restype = C.c_int32
    _lib = L
    return L


def pack_geom(geom):
    """DeblockGeom arrays -> packed uint32 mi records (zf_pack_geom)."""
    arrs = geom.arrays()
    out = np.zeros(geom.mi_rows * geom.mi_cols, np.uint32)
    rc = lib().zf_pack_geom(geom.mi_cols, geom.mi_rows, *[a.ctypes.data for a in arrs], out.ctypes.data)
    if rc != 0:
        raise ZfError(rc, "geometry is not an aligned AV1 block/transform tiling")
    return out


def stats_dict(s):
    return {"cdef_filtered_px": s.cdef_filtered_px, "cdef_changed_px": s.cdef_changed_px,
            "cdef_sb_count": s.cdef_sb_count, "lr_wiener_units": s.lr_wiener_units,
            "lr_frame_rtype": list(s.lr_frame_rtype)}


class Context:
    """One CUDA stream + device arena (zf_create); not thread-safe."""

    def __init__(self, device=0, hbm_budget_bytes=0, cancel_flag=None, flags=0):
        """flags: abi.OPT_GRAPHS / abi.OPT_NO_TMA (zf_opts.flags)."""
        L = lib()
        self._cancel = cancel_flag
        opts = ZfOpts()
        opts.device = device
        opts.flags = flags
        opts.hbm_budget_bytes = hbm_budget_bytes
        if cancel_flag is not None:
            opts.cancel_flag = C.cast(cancel_flag, C.POINTER(C.c_int32))
        h = C.c_void_p()
        rc = L.zf_create(C.byref(h), C.byref(opts))
        if rc != 0:
            raise ZfError(rc, "zf_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().zf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise ZfError(rc, lib().zf_last_error(self.h).decode())

    def sync(self):
        self._check(lib().zf_sync(self.h))

    def stream_handle(self):
        return lib().zf_stream(self.h)

    def launch_count(self):
        return lib().zf_launch_count(self.h)

    def device_bytes(self):
        """Device memory the context holds (its arena)."""
        return lib().zf_device_bytes(self.h)

    def trim(self):
        """Release the arena (the next call allocates again)."""
        self._check(lib().zf_trim(self.h))

    def reserve(self, device_bytes, host_bytes=8 << 20):
        """Grow the arena and the pinned staging buffers ahead of time."""
        self._check(lib().zf_reserve(self.h, int(device_bytes), int(host_bytes)))

    def profile(self, enable=True):
        self._check(lib().zf_profile_enable(self.h, 1 if enable else 0))

    def profile_reset(self):
        lib().zf_profile_reset(self.h)

    def use_graphs(self, enable=True):
        """Run each call's launch sequence as a CUDA graph (zf_use_graphs)."""
        self._check(lib().zf_use_graphs(self.h, 1 if enable else 0))

    def get_tune(self):
        """The context's launch settings (zf_get_tune) as a dict."""
        t = abi.ZfTune()
        self._check(lib().zf_get_tune(self.h, C.byref(t)))
        return t.as_dict()

    def set_tune(self, graphs, stats_tma, apply_group, stats_tc=0, trial_tile=64, db_levels=8):
        """Set the launch settings (zf_set_tune)."""
        t = abi.ZfTune(graphs, stats_tma, apply_group, stats_tc, trial_tile, db_levels, 0.0)
        self._check(lib().zf_set_tune(self.h, C.byref(t)))

    def set_tune_dict(self, t):
        """zf_set_tune from a get_tune()-style dict."""
        self.set_tune(t["graphs"], t["stats_tma"], t["apply_group"], t["stats_tc"], t["trial_tile"], t["db_levels"])

    def autotune_raw(self, frames_arr, n, reps=3):
        """zf_autotune over n ZfFrame structs: (best dict, [candidate dicts]).
        The context keeps the best setting."""
        best = abi.ZfTune()
        cands = (abi.ZfTune * 32)()
        rc = lib().zf_autotune(self.h, frames_arr, n, reps, C.byref(best), cands, 32)
        if rc < 0:
            self._check(rc)
        return best.as_dict(), [cands[i].as_dict() for i in range(min(rc, 32))]

    def graph_stats(self):
        """(graph launches, in-place updates, instantiations)."""
        out = (C.c_uint64 * 3)()
        self._check(lib().zf_graph_stats(self.h, out))
        return tuple(out)

    def profile_read(self):
        """{kernel name: (launches, total_ms)} measured with CUDA events."""
        return {k: v[:2] for k, v in self.profile_read_bytes().items()}

    def profile_read_bytes(self):
        """{kernel name: (launches, total_ms, algorithmic bytes or 0)}."""
        buf = (abi.ZfKernelTime * 64)()
        n = lib().zf_profile_read(self.h, buf, 64)
        return {buf[i].name.decode(): (buf[i].launches, buf[i].total_ms, buf[i].bytes) for i in range(min(n, 64))}

    def filter_stage_raw(self, s, dec, st):
        """zf_filter_stage on a prepared zf_frame / Decisions / ZfStats."""
        self._check(lib().zf_filter_stage(self.h, C.byref(s), C.byref(dec.c), C.byref(st)))

    def submit_batch_raw(self, frames_arr, n, decs_arr, stats_arr):
        self._check(lib().zf_submit_batch(self.h, frames_arr, n, decs_arr, stats_arr))

    # -- whole stage --------------------------------------------------------
    def filter_stage(self, fr, mi=None, rec=None):
        """Run the whole stage on a synth.Frame. Returns (decisions dict,
        stats dict, filtered planes)."""
        mi = pack_geom(fr.geom) if mi is None else mi
        rec = fr.copy_rec() if rec is None else rec
        s = abi.make_frame_struct(fr, fr.src, rec, mi)
        d = Decisions(fr.w, fr.h, fr.true_w, fr.true_h)
        st = ZfStats()
        self._check(lib().zf_filter_stage(self.h, C.byref(s), C.byref(d.c), C.byref(st)))
        return d.as_dict(), stats_dict(st), rec

    def submit_batch(self, frames, mis=None, recs=None):
        n = len(frames)
        mis = [pack_geom(f.geom) for f in frames] if mis is None else mis
        recs = [f.copy_rec() for f in frames] if recs is None else recs
        arr = (ZfFrame * n)()
        decs = [Decisions(f.w, f.h, f.true_w, f.true_h) for f in frames]
        darr = (ZfDecisions * n)()
        for i, f in enumerate(frames):
            arr[i] = abi.make_frame_struct(f, f.src, recs[i], mis[i])
            darr[i] = decs[i].c
        st = (ZfStats * n)()
        self._check(lib().zf_submit_batch(self.h, arr, n, darr, st))
        out = []
        for i in range(n):
            decs[i].c = darr[i]
            out.append((decs[i].as_dict(), stats_dict(st[i]), recs[i]))
        return out

    # -- per call site ------------------------------------------------------
    def pick_filter_levels(self, fr, rec, mi=None):
        mi = pack_geom(fr.geom) if mi is None else mi
        s = abi.make_frame_struct(fr, fr.src, rec, mi)
        lf = (C.c_uint8 * 4)()
        self._check(lib().zf_deblock_pick(self.h, C.byref(s), lf))
        return list(lf)

    def deblock_sse_table(self, fr, plane, levels, rec=None, mi=None):
        """try_filter_plane's SSE of one plane at each level, one launch
        (zf_deblock_sse_table); rec is the pre-deblock recon."""
        mi = pack_geom(fr.geom) if mi is None else mi
        rec = fr.rec if rec is None else rec
        s = abi.make_frame_struct(fr, fr.src, rec, mi)
        lv = np.ascontiguousarray(levels, np.int32)
        out = np.zeros(len(lv), np.int64)
        self._check(lib().zf_deblock_sse_table(self.h, C.byref(s), plane, lv.ctypes.data, len(lv),
                                               out.ctypes.data))
        return out

    def cdef_search_rows(self, fr, rec, mi=None):
        """zf_cdef_search_rows on the post-deblock recon: (Decisions, mse rows
        [nfb, 2 * ncand] or None, has_row [nfb])."""
        mi = pack_geom(fr.geom) if mi is None else mi
        s = abi.make_frame_struct(fr, fr.src, rec, mi)
        d = Decisions(fr.w, fr.h, fr.true_w, fr.true_h)
        nfb = d.nhfb * d.nvfb
        flat = np.zeros(nfb * 2 * 48, np.uint64)
        has = np.zeros(nfb, np.uint8)
        nc = C.c_int32()
        self._check(lib().zf_cdef_search_rows(self.h, C.byref(s), C.byref(d.c), flat.ctypes.data, has.ctypes.data,
                                              C.byref(nc)))
        n = nc.value
        return d, (flat[:nfb * 2 * n].reshape(nfb, 2 * n) if n else None), has

    def set_wait_limit(self, iterations):
        """Iteration limit of the statistics kernel's TMA wait (0: default)."""
        self._check(lib().zf_set_wait_limit(self.h, int(iterations)))

    def trace(self, path):
        """Search trace lines to path ("-" stderr, None stops): zf_trace."""
        self._check(lib().zf_trace(self.h, None if path is None else path.encode()))

    def apply_deblock_frame(self, fr, rec, lf, mi=None):
        mi = pack_geom(fr.geom) if mi is None else mi
        s = abi.make_frame_struct(fr, fr.src, rec, mi)
        lv = (C.c_uint8 * 4)(*lf)
        self._check(lib().zf_deblock_apply(self.h, C.byref(s), lv))

    def cdef_search_still(self, fr, rec, mi=None):
        mi = pack_geom(fr.geom) if mi is None else mi
        s = abi.make_frame_struct(fr, fr.src, rec, mi)
        d = Decisions(fr.w, fr.h, fr.true_w, fr.true_h)
        self._check(lib().zf_cdef_search(self.h, C.byref(s), C.byref(d.c)))
        return d

    def apply_cdef_frame(self, fr, rec, dec, mi=None):
        mi = pack_geom(fr.geom) if mi is None else mi
        s = abi.make_frame_struct(fr, fr.src, rec, mi)
        st = ZfStats()
        self._check(lib().zf_cdef_apply(self.h, C.byref(s), C.byref(dec.c), C.byref(st)))
        return stats_dict(st)

    def search_restoration_still(self, fr, rec, mi=None):
        mi = pack_geom(fr.geom) if mi is None else mi
        s = abi.make_frame_struct(fr, fr.src, rec, mi)
        d = Decisions(fr.w, fr.h, fr.true_w, fr.true_h)
        self._check(lib().zf_lr_search(self.h, C.byref(s), C.byref(d.c)))
        return d

    def apply_restoration_frame(self, fr, rec, pre_cdef, dec, mi=None):
        mi = pack_geom(fr.geom) if mi is None else mi
        s = abi.make_frame_struct(fr, fr.src, rec, mi)
        pre = (C.c_void_p * 3)(*[p.ctypes.data for p in pre_cdef])
        self._check(lib().zf_lr_apply(self.h, C.byref(s), pre, C.byref(dec.c)))

    # -- superres and film grain -----------------------------------------
    def superres_upscale(self, src, dst_width, bit_depth=8):
        """Normative horizontal upscale of a (rows, width) host plane."""
        rows, w = src.shape
        src = np.ascontiguousarray(src)
        dst = np.empty((rows, dst_width), src.dtype)
        self._check(lib().zf_superres_upscale(self.h, src.ctypes.data, w, w, dst.ctypes.data, dst_width,
                                              dst_width, rows, bit_depth, 0))
        return dst

    def film_grain_estimate(self, src, recon):
        h, w = src.shape
        p = abi.ZfFilmGrain()
        self._check(lib().zf_film_grain_estimate(self.h, np.ascontiguousarray(src).ctypes.data,
                                                 np.ascontiguousarray(recon).ctypes.data, w, h, w, 0,
                                                 C.byref(p)))
        return p

    def film_grain_synthesize(self, frame, params):
        """Adds the grain to a (rows, width) u8 host plane in place."""
        h, w = frame.shape
        assert frame.flags.c_contiguous
        self._check(lib().zf_film_grain_synthesize(self.h, frame.ctypes.data, w, h, w, 0, C.byref(params)))
        return frame

    # -- self-guided restoration ------------------------------------------
    @staticmethod
    def _sgr_plane(bd, dgd, src=None, pre_cdef=None, ss_y=0, on_device=False):
        """zf_sgr_plane over numpy arrays (host) or torch CUDA tensors
        (on_device=True, data_ptr())."""
        addr = (lambda a: None if a is None else a.data_ptr()) if on_device else \
            (lambda a: None if a is None else a.ctypes.data)
        h, w = dgd.shape
        return abi.ZfSgrPlane(bd, w, h, ss_y, 1 if on_device else 0, addr(dgd), addr(src), addr(pre_cdef))

    def sgr_search(self, bd, dgd, src, ss_y=0, set_mask=0xFFFF, on_device=False):
        """Per restoration unit: the best set of the mask, its weights, the
        SSE with it and without filtering (a SGR_UNIT record array)."""
        h, w = dgd.shape
        n = abi.count_units(w) * abi.count_units(h)
        units = np.zeros(n, abi.SGR_UNIT)
        p = self._sgr_plane(bd, dgd, src, None, ss_y, on_device)
        self._check(lib().zf_sgr_search(self.h, C.byref(p), set_mask, units.ctypes.data, n))
        return units

    def sgr_apply(self, bd, dgd, pre_cdef, units, ss_y=0, dst=None, on_device=False):
        """Decoder-exact SGRPROJ apply; returns dst (a new host array when
        dst is None and the planes are host arrays)."""
        units = np.ascontiguousarray(units, abi.SGR_UNIT)
        if dst is None:
            dst = np.empty_like(dgd)
        p = self._sgr_plane(bd, dgd, None, pre_cdef, ss_y, on_device)
        d = dst.data_ptr() if on_device else dst.ctypes.data
        self._check(lib().zf_sgr_apply(self.h, C.byref(p), units.ctypes.data, len(units), d))
        return dst


def write_filter_params(dec, monochrome=False, allow_intrabc=False, enable_restoration=True, sb_size=64,
                        sharpness=0, buf=None, bit_pos=0):
    """Frame-header loop_filter_params / cdef_params / lr_params bits for a
    ZfDecisions (zf_write_filter_params). Returns (buffer, end bit)."""
    buf = np.zeros(64, np.uint8) if buf is None else buf
    o = abi.ZfHeaderOpts(int(monochrome), int(allow_intrabc), int(enable_restoration), sb_size, sharpness, 0)
    pos = C.c_int32(bit_pos)
    rc = lib().zf_write_filter_params(C.byref(dec), C.byref(o), buf.ctypes.data, len(buf), C.byref(pos))
    if rc != 0:
        raise ZfError(rc, "zf_write_filter_params")
    return buf, pos.value


class RangeCoder:
    """The tile symbol coder (zf_ec_*): AV1's arithmetic coder, with the
    filter stage's per-superblock restoration syntax and cdef_idx literals."""

    def __init__(self):
        self._ec = lib().zf_ec_create()
        if not self._ec:
            raise MemoryError("zf_ec_create")
        self.wiener_cdf = (C.c_uint16 * 3)()
        lib().zf_wiener_restore_cdf_init(self.wiener_cdf)
        self.refs = abi.ZfWienerRefs()
        lib().zf_wiener_refs_reset(C.byref(self.refs))

    def __del__(self):
        if getattr(self, "_ec", None):
            lib().zf_ec_destroy(self._ec)
            self._ec = None

    def _chk(self, rc, what):
        if rc < 0:
            raise ZfError(rc, what)
        return rc

    def bool(self, bit, f=16384):
        self._chk(lib().zf_ec_bool(self._ec, int(bit), int(f)), "zf_ec_bool")

    def literal(self, value, nbits):
        self._chk(lib().zf_ec_literal(self._ec, int(value), int(nbits)), "zf_ec_literal")

    def symbol(self, s, icdf, adapt=True):
        """icdf: a ctypes uint16 array of nsyms + 1 entries (C layout), updated in place when adapt."""
        self._chk(lib().zf_ec_symbol(self._ec, int(s), icdf, len(icdf) - 1, int(adapt)), "zf_ec_symbol")

    def tell(self):
        return lib().zf_ec_tell(self._ec)

    def done(self):
        n = (self.tell() + 7) // 8
        buf = np.zeros(max(n, 1), np.uint8)
        n = self._chk(lib().zf_ec_done(self._ec, buf.ctypes.data, len(buf)), "zf_ec_done")
        return bytes(buf[:n])

    def lr_sb(self, dec, mi_row, mi_col, sb_mi, frame_w, frame_h, monochrome=False, sr_denom=0):
        """Codes the restoration units whose corner lies in the superblock
        (at its start); returns the element count."""
        return self._chk(lib().zf_ec_lr_sb(self._ec, C.byref(dec), mi_row, mi_col, sb_mi, frame_w, frame_h,
                                           int(monochrome), sr_denom, C.byref(self.refs), self.wiener_cdf),
                         "zf_ec_lr_sb")

    @staticmethod
    def cdef_sb(dec, sb_row, sb_col, sb_size=64):
        st = abi.ZfCdefSb()
        rc = lib().zf_cdef_sb_begin(C.byref(dec), sb_row, sb_col, sb_size, C.byref(st))
        if rc < 0:
            raise ZfError(rc, "zf_cdef_sb_begin")
        return st

    def cdef_block(self, st, block_x, block_y, skip):
        """After a coded block's skip flag; returns the cdef_idx bits coded."""
        return self._chk(lib().zf_ec_cdef_block(self._ec, C.byref(st), block_x, block_y, int(skip)),
                         "zf_ec_cdef_block")


def query_sizes(fr, mi=None):
    mi = pack_geom(fr.geom) if mi is None else mi
    s = abi.make_frame_struct(fr, fr.src, fr.rec, mi)
    z = ZfSizes()
    rc = lib().zf_query_sizes(C.byref(s), C.byref(z))
    if rc != 0:
        raise ZfError(rc, "zf_query_sizes")
    return z
