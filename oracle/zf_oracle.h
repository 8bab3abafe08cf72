/*
 * zf_oracle.h -- CPU ORACLE for the in-loop filter stage. TEST
 * INFRASTRUCTURE ONLY: the parity tests, the smoke check and the timed CPU
 * baseline load it as the checker. The product library never links it.
 *
 * It restates the reference encoder's scalar filter code (Rust, cited per
 * function in zf_oracle.cpp) in C++17 and exposes it through C entry points
 * that take the same zf_frame / zf_decisions structs as the product ABI,
 * with the geometry given as the reference's explicit DeblockGeom arrays
 * (block_id, bw, bh, tw, th, skip, skip_inter) instead of packed records.
 */
#ifndef ZF_ORACLE_H
#define ZF_ORACLE_H

#include <stdint.h>
#include "../include/zf_filter.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct zfo_geom {
    int32_t mi_cols, mi_rows;
    const uint32_t *block_id;
    const uint8_t *bw, *bh, *tw, *th, *skip, *skip_inter;
} zfo_geom;

/* Restoration-plane padding model. ZFO_LR_BORDER_C gives the plane a wide
 * right border like C SVT-AV1 / libaom frame buffers (the 16-rounded Wiener
 * processing unit writes into it and the result is discarded).
 * ZFO_LR_BORDER_PORT reproduces the reference port's 4-px PaddedPlane, in
 * which those writes land in the next row of the flat buffer. */
enum { ZFO_LR_BORDER_C = 0, ZFO_LR_BORDER_PORT = 1 };

/* Whole stage (pipeline.rs:2886-3455 for a key frame). rec[] in place. */
int32_t zfo_filter_stage(const zf_frame *f, const zfo_geom *g, zf_decisions *out,
                         zf_stats *stats, int32_t lr_border_mode);

/* Per-call-site pieces, same meaning as the zf_* functions. */
int32_t zfo_deblock_pick(const zf_frame *f, const zfo_geom *g, uint8_t lf[4]);
int32_t zfo_deblock_apply(const zf_frame *f, const zfo_geom *g, const uint8_t lf[4]);
/* try_filter_plane (ENC/deblock.rs:228-293) of one plane at each of n
 * levels (lvl0 = lvl1 = level): SSE vs the source over the aligned plane. */
int32_t zfo_deblock_sse_table(const zf_frame *f, const zfo_geom *g, int32_t plane, const int32_t *levels, int32_t n,
                              int64_t *sse);
/* Search trace in the reference's debug-dump line formats (path "-" is
 * stderr; NULL or "" stops): DLF_TRY / DLF_PICK, RS_CDEF_FB / RS_CDEF_SUM /
 * RS_CDEF_PICK, LRNONE / LRWNSCORE / LRWNSEG. Process-wide. */
void zfo_trace(const char *path);
/* mse_out (optional): per filter block in raster order, 2*ncand u64
 * ([luma row][joint uv row]); rows of all-skip fbs are left untouched and
 * fb_has_row[fb] (optional) says which ones were written. */
int32_t zfo_cdef_search(const zf_frame *f, const zfo_geom *g, zf_decisions *out,
                        uint64_t *mse_out, uint8_t *fb_has_row, int32_t *ncand_out);
int32_t zfo_cdef_apply(const zf_frame *f, const zfo_geom *g, const zf_decisions *d,
                       zf_stats *stats);
int32_t zfo_lr_search(const zf_frame *f, zf_decisions *out, int32_t lr_border_mode);
int32_t zfo_lr_apply(const zf_frame *f, const void *const pre_cdef[3], const zf_decisions *d,
                     int32_t lr_border_mode);

/* --- Kernel-level pieces for the fine-grained parity tests -------------- */
void zfo_lf_thresholds(int32_t level, int32_t sharpness, int32_t out[3]);
/* One lpf call on a plane (u8 when bd == 8 else u16): vert != 0 selects
 * lpf_vertical_N, len in {4,6,8,14}. */
void zfo_lpf(void *buf, int32_t bd, int32_t off, int32_t pitch, int32_t vert, int32_t len,
             int32_t level, int32_t sharpness);
void zfo_cdef_find_dir(const uint16_t *img, int32_t stride, int32_t coeff_shift,
                       int32_t *dir, int32_t *var);
/* inb: CDEF_BSTRIDE(144)-strided u16 buffer, ioff = block (0,0). dst is u8
 * when dst_is_u16 == 0. */
void zfo_cdef_filter_block(void *dst, int32_t dst_is_u16, int32_t doff, int32_t dstride,
                           const uint16_t *inb, int32_t ioff, int32_t pri, int32_t sec,
                           int32_t dir, int32_t pri_damping, int32_t sec_damping,
                           int32_t bsize, int32_t coeff_shift, int32_t sub);
int32_t zfo_adjust_strength(int32_t strength, int32_t var);
/* finish_cdef_rd over mse rows (n_fb x 2 x n_cand): returns bits, writes
 * lev0/lev1 (1 << bits entries). */
int32_t zfo_cdef_finish_rd(const uint64_t *mse, int32_t n_fb, int32_t n_cand, int32_t qindex,
                           int32_t bit_depth, int32_t *lev0, int32_t *lev1);
void zfo_cdef_qp_params(int32_t qindex, int32_t bit_depth, int32_t screen, int32_t out[3]);
void zfo_deblock_key_frame_levels(int32_t qindex, int32_t bit_depth, uint8_t out[4]);
/* search_filter_level replay over a table of trial SSEs (errs[level],
 * -1 = not available): returns the level; *n_tries gets the number of
 * try_filter_frame calls and tried[] the levels in call order. */
int32_t zfo_dlf_hillclimb_replay(const int64_t *errs, int32_t conv_th, int32_t *tried,
                                 int32_t *n_tries);
uint32_t zfo_lambda(int32_t which, int32_t qindex);
/* compute_stats (u8 when bd == 8); dgd/src at their origins, coordinates
 * relative to origin. m: win^2, h: win^4. */
void zfo_compute_stats(int32_t win, const void *dgd, int64_t dgd_origin, int32_t dgd_stride,
                       const void *src, int64_t src_origin, int32_t src_stride, int32_t h_start,
                       int32_t h_end, int32_t v_start, int32_t v_end, int64_t *m, int64_t *h,
                       int32_t bd);
/* wiener_decompose_sep_sym + finalize_sym_filter + compute_score. */
int64_t zfo_wiener_solve(int32_t win, const int64_t *m, const int64_t *h, int32_t vd[7],
                         int32_t hd[7], int16_t vf[8], int16_t hf[8]);
int32_t zfo_count_wiener_bits(int32_t win, const int16_t vf[8], const int16_t hf[8],
                              const int16_t rvf[8], const int16_t rhf[8]);
int32_t zfo_count_units_in_tile(int32_t unit_size, int32_t tile_size);
double zfo_rdcost_dbl(int64_t rdmult, int64_t rate, int64_t dist);
/* wiener_convolve_add_src[_hbd]: src/dst at origins (u8 when bd == 8). */
void zfo_wiener_convolve(const void *src, int64_t src_origin, int32_t src_stride, void *dst,
                         int64_t dst_origin, int32_t dst_stride, const int16_t hf[8],
                         const int16_t vf[8], int32_t w, int32_t h, int32_t bd);
int64_t zfo_sse_region(const void *a, int32_t a_stride, const void *b, int32_t b_stride,
                       int32_t w, int32_t h, int32_t bd);

/* --- Self-guided restoration (AV1 spec 7.17.3; not in the reference) ---- */
typedef struct zfo_sgr_unit {
    int32_t set, w0, w1, pad;
    int64_t sse, sse_none;
} zfo_sgr_unit;
/* Planes tight (stride = pw), u8 when bd == 8 else u16; units hunits*vunits
 * of the 256-px restoration-unit grid, row-major. */
int32_t zfo_sgr_search(int32_t bd, int32_t pw, int32_t ph, int32_t ss, const void *dgd, const void *src,
                       uint32_t set_mask, zfo_sgr_unit *units);
int32_t zfo_sgr_apply(int32_t bd, int32_t pw, int32_t ph, int32_t ss, const void *dgd, const void *pre_cdef,
                      const zfo_sgr_unit *units, void *dst);
void zfo_sgr_box_filter(int32_t bd, int32_t pw, int32_t ph, const void *dgd, int32_t set, int32_t pass, int32_t x,
                        int32_t y, int32_t w, int32_t h, int32_t *out);
void zfo_sgr_params(int32_t set, int32_t out[4]);
/* Superres and film grain (DSP/superres.rs, ENC/film_grain.rs). */
int32_t zfo_superres_scaled_size(int32_t dim, int32_t denom);
void zfo_superres_upscale(const void *src, int32_t src_stride, int32_t src_width, void *dst, int32_t dst_stride,
                          int32_t dst_width, int32_t rows, int32_t bd);
void zfo_film_grain_estimate(const uint8_t *source, const uint8_t *denoised, int32_t width, int32_t height,
                             int32_t stride, zf_film_grain *p);
void zfo_film_grain_synthesize(uint8_t *frame, int32_t width, int32_t height, int32_t stride,
                               const zf_film_grain *p);
/* Frame-header loop_filter / cdef / lr params (ENT/obu.rs:1268-1377). */
int32_t zfo_write_filter_params(const zf_decisions *d, const zf_header_opts *o, uint8_t *buf, int32_t cap,
                                int32_t *bit_pos);

#ifdef __cplusplus
}
#endif
#endif /* ZF_ORACLE_H */
