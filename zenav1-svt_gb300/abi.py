"""ctypes mirror of include/zf_filter.h (shared by the product binding and
the test-side oracle binding)."""
import ctypes as C

import numpy as np

ZF_OK = 0
ERRORS = {
    -1: "AllocFailed", -2: "InvalidDimensions", -3: "UnsupportedConfig", -4: "Cancelled",
    -5: "CudaError", -6: "InvalidArgument", -7: "InvalidGeometry", -8: "Timeout",
}
RESTORE_NONE, RESTORE_WIENER = 0, 1
OPT_GRAPHS, OPT_NO_TMA = 1, 2  # zf_opts.flags


class ZfFrame(C.Structure):
    _fields_ = [
        ("bit_depth", C.c_int32), ("width", C.c_int32), ("height", C.c_int32),
        ("true_width", C.c_int32), ("true_height", C.c_int32), ("chroma_420", C.c_int32),
        ("preset", C.c_int32), ("qindex", C.c_int32), ("sharpness", C.c_int32),
        ("sc_class5", C.c_int32), ("enable_restoration", C.c_int32), ("planes_on_device", C.c_int32),
        ("src", C.c_void_p * 3), ("rec", C.c_void_p * 3), ("mi", C.c_void_p),
    ]


class ZfLrUnit(C.Structure):
    _fields_ = [("vfilter", C.c_int16 * 8), ("hfilter", C.c_int16 * 8), ("rtype", C.c_uint8),
                ("pad", C.c_uint8 * 7)]


class ZfLrPlane(C.Structure):
    _fields_ = [("frame_rtype", C.c_int32), ("unit_size", C.c_int32), ("hunits", C.c_int32),
                ("vunits", C.c_int32)]


class ZfDecisions(C.Structure):
    _fields_ = [
        ("lf", C.c_uint8 * 4), ("cdef_damping", C.c_uint8), ("cdef_bits", C.c_uint8),
        ("cdef_y", C.c_uint8 * 8), ("cdef_uv", C.c_uint8 * 8),
        ("nhfb", C.c_int32), ("nvfb", C.c_int32), ("cdef_fb_idx", C.POINTER(C.c_uint8)),
        ("lr", ZfLrPlane * 3), ("lr_units", C.POINTER(ZfLrUnit) * 3),
    ]


class ZfStats(C.Structure):
    _fields_ = [("cdef_filtered_px", C.c_uint64), ("cdef_changed_px", C.c_uint64),
                ("cdef_sb_count", C.c_int32), ("lr_wiener_units", C.c_int32),
                ("lr_frame_rtype", C.c_int32 * 3), ("pad", C.c_int32)]


class ZfSizes(C.Structure):
    _fields_ = [("nhfb", C.c_int32), ("nvfb", C.c_int32), ("lr_hunits", C.c_int32 * 3),
                ("lr_vunits", C.c_int32 * 3), ("lr_unit_size", C.c_int32), ("pad", C.c_int32),
                ("device_bytes", C.c_uint64)]


SYM_WIENER_RESTORE, SYM_BITS = 1, 2  # zf_lr_sym.kind


class ZfLrSym(C.Structure):
    _fields_ = [("kind", C.c_int32), ("nbits", C.c_int32), ("value", C.c_uint32), ("plane", C.c_int16),
                ("pad", C.c_int16), ("unit", C.c_int32)]


class ZfWienerRefs(C.Structure):
    _fields_ = [("vfilter", (C.c_int16 * 8) * 3), ("hfilter", (C.c_int16 * 8) * 3)]


class ZfCdefSb(C.Structure):
    _fields_ = [("bits", C.c_int32), ("sb128", C.c_int32), ("strengths", C.c_uint8 * 4),
                ("transmitted", C.c_uint8 * 4)]


class ZfTune(C.Structure):
    _fields_ = [("graphs", C.c_int32), ("stats_tma", C.c_int32), ("apply_group", C.c_int32),
                ("stats_tc", C.c_int32), ("trial_tile", C.c_int32), ("db_levels", C.c_int32),
                ("ms", C.c_double)]

    def as_dict(self):
        return {"graphs": self.graphs, "stats_tma": self.stats_tma, "apply_group": self.apply_group,
                "stats_tc": self.stats_tc, "trial_tile": self.trial_tile, "db_levels": self.db_levels,
                "ms": round(self.ms, 4)}


class ZfOpts(C.Structure):
    _fields_ = [("device", C.c_int32), ("flags", C.c_int32), ("hbm_budget_bytes", C.c_uint64),
                ("cancel_flag", C.POINTER(C.c_int32))]


class ZfHeaderOpts(C.Structure):
    _fields_ = [("monochrome", C.c_int32), ("allow_intrabc", C.c_int32), ("enable_restoration", C.c_int32),
                ("sb_size", C.c_int32), ("sharpness", C.c_int32), ("pad", C.c_int32)]


class ZfFilmGrain(C.Structure):
    _fields_ = [("apply_grain", C.c_int32), ("grain_seed", C.c_uint16), ("num_y_points", C.c_uint8),
                ("num_cb_points", C.c_uint8), ("num_cr_points", C.c_uint8),
                ("point_y_value", C.c_uint8 * 14), ("point_y_scaling", C.c_uint8 * 14),
                ("point_cb_value", C.c_uint8 * 10), ("point_cb_scaling", C.c_uint8 * 10),
                ("point_cr_value", C.c_uint8 * 10), ("point_cr_scaling", C.c_uint8 * 10),
                ("ar_coeffs_y", C.c_int8 * 24), ("ar_coeffs_cb", C.c_int8 * 25), ("ar_coeffs_cr", C.c_int8 * 25),
                ("ar_coeff_lag", C.c_uint8), ("ar_coeff_shift", C.c_uint8), ("grain_scale_shift", C.c_uint8),
                ("cb_mult", C.c_uint8), ("cb_luma_mult", C.c_uint8), ("cr_mult", C.c_uint8),
                ("cr_luma_mult", C.c_uint8), ("overlap_flag", C.c_uint8), ("clip_to_restricted_range", C.c_uint8),
                ("chroma_scaling_from_luma", C.c_uint8), ("cb_offset", C.c_uint16), ("cr_offset", C.c_uint16),
                ("noise_var", C.c_double)]


class ZfSgrPlane(C.Structure):
    _fields_ = [("bit_depth", C.c_int32), ("width", C.c_int32), ("height", C.c_int32), ("ss_y", C.c_int32),
                ("on_device", C.c_int32), ("dgd", C.c_void_p), ("src", C.c_void_p), ("pre_cdef", C.c_void_p)]


# zf_sgr_unit as a numpy record (32 bytes)
SGR_UNIT = np.dtype([("set", np.int32), ("w0", np.int32), ("w1", np.int32), ("pad", np.int32),
                     ("sse", np.int64), ("sse_none", np.int64)])


class ZfKernelTime(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_uint64), ("total_ms", C.c_double), ("bytes", C.c_uint64)]


def ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def count_units(size, unit=256):
    return max((size + (unit >> 1)) // unit, 1)


class Decisions:
    """A zf_decisions with caller-owned arrays sized for a frame."""

    def __init__(self, width, height, true_w, true_h):
        self.nhfb, self.nvfb = (width + 63) // 64, (height + 63) // 64
        self.fb_idx = np.zeros(self.nhfb * self.nvfb, np.uint8)
        self.units = []
        for p in range(3):
            pw = true_w if p == 0 else (true_w + 1) // 2
            ph = true_h if p == 0 else (true_h + 1) // 2
            self.units.append((ZfLrUnit * (count_units(pw) * count_units(ph)))())
        self.c = ZfDecisions()
        self.c.cdef_fb_idx = self.fb_idx.ctypes.data_as(C.POINTER(C.c_uint8))
        for p in range(3):
            self.c.lr_units[p] = C.cast(self.units[p], C.POINTER(ZfLrUnit))

    def as_dict(self):
        c = self.c
        bits = c.cdef_bits
        d = {
            "lf": list(c.lf),
            "cdef_damping": c.cdef_damping,
            "cdef_bits": bits,
            "cdef_y": list(c.cdef_y)[:1 << bits],
            "cdef_uv": list(c.cdef_uv)[:1 << bits],
            "cdef_fb_idx": self.fb_idx.copy() if bits else np.zeros_like(self.fb_idx),
            "lr": [],
        }
        for p in range(3):
            lp = c.lr[p]
            n = lp.hunits * lp.vunits
            units = [(self.units[p][u].rtype, tuple(self.units[p][u].vfilter), tuple(self.units[p][u].hfilter))
                     for u in range(n)]
            d["lr"].append({"frame_rtype": lp.frame_rtype, "hunits": lp.hunits, "vunits": lp.vunits,
                            "units": units})
        return d


def make_frame_struct(fr, src, rec, mi, on_device=False):
    """zf_frame for a synth.Frame-like object; src/rec/mi are numpy arrays
    (host) or integer device addresses (on_device)."""
    s = ZfFrame()
    s.bit_depth, s.width, s.height = fr.bd, fr.w, fr.h
    s.true_width, s.true_height = fr.true_w, fr.true_h
    s.chroma_420 = 1 if fr.chroma else 0
    s.preset, s.qindex, s.sharpness = fr.preset, fr.qindex, fr.sharpness
    s.sc_class5, s.enable_restoration = fr.sc_class5, fr.enable_restoration
    s.planes_on_device = 1 if on_device else 0
    for p in range(3):
        if on_device:
            s.src[p] = src[p]
            s.rec[p] = rec[p]
        else:
            s.src[p] = src[p].ctypes.data
            s.rec[p] = rec[p].ctypes.data
    s.mi = mi if on_device else mi.ctypes.data
    return s
