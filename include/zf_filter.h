/*
 * zf_filter.h -- C ABI of the GB300 in-loop filter stage (deblock, CDEF,
 * Wiener loop restoration) for the zenav1-svt AV1 still-image encoder.
 *
 * Every entry point here replaces one call site of the reference encoder's
 * filter stage (rust/crates/svtav1-encoder/src/pipeline.rs:2813-3482). The
 * reference functions are safe Rust over tight planes; this library takes
 * the same planes as plain pointers and sizes so that a thin Rust crate
 * outside the encoder's #![forbid(unsafe_code)] crates can bind it.
 *
 * Conventions
 *  - Planes are tight: luma stride = width, chroma stride = width/2 (4:2:0).
 *    8-bit planes are uint8_t, 10-bit planes are uint16_t (values < 1024).
 *  - width/height are the 8-aligned canvas the deblock/CDEF passes run on;
 *    true_width/true_height are the coded dims (<= aligned) that the
 *    deblock onScreen guard and loop restoration use.
 *  - Return codes: ZF_OK (0) or a negative ZF_ERR_* code; the reference's
 *    EncodeError variants map onto AllocFailed, InvalidDimensions,
 *    UnsupportedConfig and Cancelled. No C++ exception crosses the ABI.
 *  - A zf_ctx owns one CUDA stream and its device scratch; it is not
 *    thread-safe (one caller at a time, as &mut EncodePipeline is).
 *  - Decision outputs use caller-owned arrays sized by zf_query_sizes().
 */
#ifndef ZF_FILTER_H
#define ZF_FILTER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ZF_ABI_VERSION 2

enum {
    ZF_OK = 0,
    ZF_ERR_ALLOC = -1,        /* EncodeError::AllocFailed */
    ZF_ERR_INVALID_DIMS = -2, /* EncodeError::InvalidDimensions */
    ZF_ERR_UNSUPPORTED = -3,  /* EncodeError::UnsupportedConfig */
    ZF_ERR_CANCELLED = -4,    /* EncodeError::Cancelled */
    ZF_ERR_CUDA = -5,         /* a CUDA runtime call or kernel failed */
    ZF_ERR_ARG = -6,          /* NULL pointer or malformed argument */
    ZF_ERR_GEOM = -7,         /* packed mi geometry is not a valid AV1 tiling */
    ZF_ERR_TIMEOUT = -8       /* a bounded device-side wait gave up */
};

/* Restoration types (C enum order, svtav1-dsp/src/restoration.rs:87-90). */
enum { ZF_RESTORE_NONE = 0, ZF_RESTORE_WIENER = 1, ZF_RESTORE_SGRPROJ = 2 };

/*
 * Packed per-4x4 (mode-info unit) deblock geometry, one uint32 per mi in
 * raster order over (width/4) x (height/4). It carries what the reference's
 * DeblockGeom (svtav1-encoder/src/deblock.rs:532-579) records per mi:
 *   bits  0..2  log2(block width)  - 2   (block 4..128 px)
 *   bits  3..5  log2(block height) - 2
 *   bits  6..8  log2(luma TX width)  - 2 (TX 4..64 px)
 *   bits  9..11 log2(luma TX height) - 2
 *   bit  12     skip        (signaled skip_txfm, read by CDEF)
 *   bit  13     skip_inter  (skip && is_inter, read by deblock)
 * DeblockGeom's explicit block_id is not stored: AV1 blocks are aligned to
 * their own dimensions, so two mi units share a block exactly when their
 * aligned block origins coincide. zf_pack_geom() builds the record from the
 * reference's arrays and rejects inputs for which that does not hold.
 */
#define ZF_MI_SKIP (1u << 12)
#define ZF_MI_SKIP_INTER (1u << 13)

typedef struct zf_frame {
    int32_t bit_depth;          /* 8 or 10 */
    int32_t width, height;      /* aligned canvas, multiples of 8 */
    int32_t true_width, true_height;
    int32_t chroma_420;         /* 1: U and V planes present (width/2 x height/2) */
    int32_t preset;             /* encoder preset 0..13 */
    int32_t qindex;             /* base_q_idx 0..255 */
    int32_t sharpness;          /* loop_filter_sharpness 0..7 */
    int32_t sc_class5;          /* screen-content arm of the qp CDEF picker */
    int32_t enable_restoration; /* sequence-level enable_restoration */
    int32_t planes_on_device;   /* 1: src/rec/mi are device pointers */
    const void *src[3];         /* source planes */
    void *rec[3];               /* in: pre-deblock recon; out: final filtered recon */
    const uint32_t *mi;         /* packed geometry, (width/4)*(height/4) */
} zf_frame;

typedef struct zf_lr_unit {
    int16_t vfilter[8];
    int16_t hfilter[8];
    uint8_t rtype;
    uint8_t pad[7];
} zf_lr_unit;

typedef struct zf_lr_plane {
    int32_t frame_rtype;
    int32_t unit_size;
    int32_t hunits, vunits;
} zf_lr_plane;

typedef struct zf_decisions {
    uint8_t lf[4];              /* [luma vert, luma horz, U, V] (LfLevels) */
    uint8_t cdef_damping;
    uint8_t cdef_bits;
    uint8_t cdef_y[8], cdef_uv[8]; /* packed strengths, 1 << cdef_bits used */
    int32_t nhfb, nvfb;         /* 64x64 filter blocks per row / column */
    uint8_t *cdef_fb_idx;       /* caller array nhfb*nvfb, may be NULL */
    zf_lr_plane lr[3];
    zf_lr_unit *lr_units[3];    /* caller arrays hunits*vunits, may be NULL */
} zf_decisions;

typedef struct zf_stats {
    uint64_t cdef_filtered_px;  /* CdefStats::filtered_px (8-bit apply) */
    uint64_t cdef_changed_px;   /* CdefStats::changed_px */
    int32_t cdef_sb_count;      /* filter blocks with a non-skip 8x8 */
    int32_t lr_wiener_units;    /* units applied with RESTORE_WIENER */
    int32_t lr_frame_rtype[3];
    int32_t pad;
} zf_stats;

typedef struct zf_sizes {
    int32_t nhfb, nvfb;
    int32_t lr_hunits[3], lr_vunits[3];
    int32_t lr_unit_size;
    int32_t pad;
    uint64_t device_bytes;      /* device footprint of one frame in flight */
} zf_sizes;

#define ZF_OPT_GRAPHS 1          /* zf_opts.flags: run each call's launch sequence as a CUDA graph */
#define ZF_OPT_NO_TMA 2          /* zf_opts.flags: stage the statistics rows with thread loads, not TMA */

typedef struct zf_opts {
    int32_t device;             /* CUDA device ordinal */
    int32_t flags;              /* ZF_OPT_* (0: launches issued directly on the stream) */
    uint64_t hbm_budget_bytes;  /* 0: no limit */
    volatile int32_t *cancel_flag; /* polled between passes; non-zero => ZF_ERR_CANCELLED */
} zf_opts;

typedef struct zf_ctx zf_ctx;

/* Library/ABI identification. */
int32_t zf_abi_version(void);

/* Context lifetime: one CUDA stream + device scratch per context. */
int32_t zf_create(zf_ctx **out, const zf_opts *opts);
void zf_destroy(zf_ctx *ctx);
/* Text of the last error recorded on this context ("" when none). */
const char *zf_last_error(const zf_ctx *ctx);
/* Synchronise the context's stream. */
int32_t zf_sync(zf_ctx *ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that order their
 * own work or timing events against the library's launches. */
void *zf_stream(const zf_ctx *ctx);
/* Device memory the context holds now (its arena; grows to the largest
 * batch seen, never shrinks by itself). No counterpart in the reference:
 * the served request loop admits work against an HBM budget with it. */
uint64_t zf_device_bytes(const zf_ctx *ctx);
/* Release the context's arena (after synchronising its stream); the next
 * call allocates again. No counterpart in the reference. */
int32_t zf_trim(zf_ctx *ctx);
/* Grow the arena to at least device_bytes and each pinned host staging
 * buffer (metadata up, decisions down) to at least host_bytes now, and the
 * gathered host-plane copies' job lists to 400 frames' worth, so that later
 * calls up to that size allocate nothing (allocation and release
 * synchronise the device). No counterpart in the reference. */
int32_t zf_reserve(zf_ctx *ctx, uint64_t device_bytes, uint64_t host_bytes);

/* Output array sizes for a frame (filter blocks, restoration units). */
int32_t zf_query_sizes(const zf_frame *f, zf_sizes *out);

/*
 * Pack the reference DeblockGeom arrays (deblock.rs:532-579: block_id, bw,
 * bh, tw, th, skip, skip_inter per mi) into the uint32 records above.
 * Returns ZF_ERR_GEOM when a block or transform is not aligned to its own
 * dimensions or block_id disagrees with the aligned block origin.
 */
int32_t zf_pack_geom(int32_t mi_cols, int32_t mi_rows, const uint32_t *block_id,
                     const uint8_t *bw, const uint8_t *bh, const uint8_t *tw,
                     const uint8_t *th, const uint8_t *skip, const uint8_t *skip_inter,
                     uint32_t *out);

/*
 * The whole filter stage for one key frame, replacing
 * pipeline.rs:2886-3455: deblock level pick + apply, CDEF pick + apply,
 * Wiener search + stripe-boundary save + apply. rec[] is overwritten with
 * the final filtered recon; the decisions the frame header and tile syntax
 * need are written to *out. stats may be NULL.
 */
int32_t zf_filter_stage(zf_ctx *ctx, const zf_frame *f, zf_decisions *out, zf_stats *stats);

/*
 * Batched form: n frames of any size and bit depth go through one launch
 * per filter pass (device work lists over (frame, tile) descriptors).
 * Per-frame results are identical to n separate zf_filter_stage calls.
 */
int32_t zf_submit_batch(zf_ctx *ctx, const zf_frame *frames, int32_t n,
                        zf_decisions *outs, zf_stats *stats);

/* --- Per-call-site entry points (one per reference function) ----------- */

/* deblock::pick_filter_levels_full_search (presets <= 5, deblock.rs:481)
 * or pick_filter_levels_key_frame (deblock.rs:55). Reads src and the
 * pre-deblock rec; writes lf[4]. */
int32_t zf_deblock_pick(zf_ctx *ctx, const zf_frame *f, uint8_t lf[4]);

/* The trial of the deblock level search for a table of levels:
 * try_filter_plane (deblock.rs:228-293) for each levels[k] (0..63; luma
 * filters both edge directions at the level, as the search's dir = 2 does),
 * i.e. the SSE between the source plane and the pre-deblock plane filtered
 * at that level, over the full aligned plane. n <= 64; the whole table runs
 * as one launch (the level search itself uses the same trials, several
 * levels per launch). rec is not modified. */
int32_t zf_deblock_sse_table(zf_ctx *ctx, const zf_frame *f, int32_t plane, const int32_t *levels, int32_t n,
                             int64_t *sse);

/* deblock::apply_deblock_frame[_hbd] (deblock.rs:938, :976): rec in place. */
int32_t zf_deblock_apply(zf_ctx *ctx, const zf_frame *f, const uint8_t lf[4]);

/* The CDEF pick of pipeline.rs:3042-3144: cdef_search_still[_hbd]
 * (cdef.rs:1166, :1374), the all-skip outcome (cdef.rs:282) or the qp
 * closed form (cdef.rs:151). Reads src and the post-deblock rec. */
int32_t zf_cdef_search(zf_ctx *ctx, const zf_frame *f, zf_decisions *out);

/* zf_cdef_search plus the search's per-filter-block mse rows, the values
 * the reference's SVTAV1_CDEF_DBG dump prints (cdef_search_still[_hbd],
 * cdef.rs:1166-1322): for filter block fb (raster order) with a non-skip
 * 8x8, mse[fb * 2 * ncand + gi] is the luma SSE of candidate gi and
 * mse[fb * 2 * ncand + ncand + gi] the joint U+V one, in candidate-slot
 * order; has_row[fb] = 1 for those blocks, 0 for all-skip ones (whose rows
 * are left untouched). mse must hold nhfb * nvfb * 2 * 48 entries and
 * has_row nhfb * nvfb (either may be NULL); *ncand gets the candidate
 * count, 0 when no search ran (presets >= 7: has_row is then all 0). */
int32_t zf_cdef_search_rows(zf_ctx *ctx, const zf_frame *f, zf_decisions *out, uint64_t *mse, uint8_t *has_row,
                            int32_t *ncand);

/* cdef::apply_cdef_frame[_hbd] (cdef.rs:343, :556): rec in place (the
 * pre-CDEF snapshot is taken internally). */
int32_t zf_cdef_apply(zf_ctx *ctx, const zf_frame *f, const zf_decisions *d, zf_stats *stats);

/* restoration::search_restoration_still[_bd] (restoration.rs:644, :675):
 * reads src and the post-CDEF rec, writes out->lr / out->lr_units. */
int32_t zf_lr_search(zf_ctx *ctx, const zf_frame *f, zf_decisions *out);

/* restoration::save_lr_boundaries + apply_restoration_frame
 * (restoration.rs:938, :992): f->rec holds the post-CDEF planes (updated in
 * place), pre_cdef[] the post-deblock planes the stripe boundaries come
 * from (same layout and memory kind as rec). */
int32_t zf_lr_apply(zf_ctx *ctx, const zf_frame *f, const void *const pre_cdef[3],
                    const zf_decisions *d);

/*
 * Allocation-free CDEF strength search. No counterpart in the reference: it
 * computes the same decisions as zf_cdef_search, for callers that cannot
 * allocate device memory once running (an encoder loop that reserves all
 * memory at start-up, code running while another component holds a stream
 * capture open on a different stream, during which cudaMalloc is not
 * allowed, a process on a fully reserved GPU slice). It needs no zf_ctx and
 * calls no allocator: its scratch is a static device array of about 1.9 MiB
 * (mse rows 640 KiB, compacted rows 1.25 MiB, ids 32 KiB) that every GPU
 * loading the library keeps until exit.
 *  - f must have planes_on_device = 1: rec = post-deblock planes, src, mi
 *    are device pointers; out (and out->cdef_fb_idx) are host memory.
 *  - stream is a cudaStream_t (NULL: the legacy default stream); the call
 *    returns after synchronising it. The stream itself must not be capturing
 *    (nor be the legacy stream while another stream captures in global
 *    mode): such calls return ZF_ERR_UNSUPPORTED.
 *  - Limits: at most 2048 64x64 filter blocks (3840x2160 has 2040) ->
 *    ZF_ERR_INVALID_DIMS beyond; at most 20 candidate strengths (presets
 *    1..6; preset 0) -> ZF_ERR_UNSUPPORTED. Presets >= 7 return the qp
 *    closed form without device work.
 *  - The first call on a device (and the first after the device's context
 *    was reset) looks up the array's device address with that device
 *    current; make that first call before any stream capture.
 *  - All calls share the one array: calls that overlap on the GPU (other
 *    streams, other host threads) race and must be serialised by the caller.
 */
int32_t zf_cdef_search_noalloc(void *stream, const zf_frame *f, zf_decisions *out);

/* --- Observability ------------------------------------------------------- */

/* Search trace, the counterpart of the reference's debug dumps
 * SVTAV1_DLFDBG (deblock.rs:274-276, :406-408), SVTAV1_CDEF_DBG
 * (cdef.rs:1296-1322) and SVTAV1_LR_DBG (restoration.rs:768-842), in the
 * same line formats so that a trace of this library and one of the
 * reference (or of a CPU restatement of it) diff line by line:
 *   DLF_TRY plane= lvl0= lvl1= w= h= sse=      every level the hill-climb
 *                                              evaluated, in climb order
 *   DLF_PICK plane= dir= level= sse=
 *   RS_CDEF_FB fbr= fbc= Y=[..] UV=[..]        per filter block with a row
 *   RS_CDEF_SUM sb_count= fs=[..] Ysum=[..] UVsum=[..]
 *   RS_CDEF_PICK bits= lev0=[..] lev1=[..]
 *   LRNONE plane= unit= lim=[h0,h1,v0,v1] sse=  every unit, then per unit
 *   LRWNSCORE plane= unit= score=
 *   LRWNSEG plane= unit= sse_wn= v=[7 taps] h=[7 taps]   (score <= 0)
 * (the reference's LRWNSOLVE and per-step LRSTEP lines are not produced:
 * the refinement runs on the device without a per-step record). A batch
 * call writes "ZF_FRAME index= w= h=" before each frame's lines. path
 * "-" is stderr, NULL or "" stops tracing; the environment variable
 * ZF_TRACE=<path> turns it on at zf_create. Tracing synchronises and reads
 * the search buffers back after every call: a diagnostic mode. */
int32_t zf_trace(zf_ctx *ctx, const char *path);

/* ---- Frame-header filter syntax ------------------------------------------
 * The loop_filter_params(), cdef_params() and lr_params() fields of an
 * uncompressed frame header for a frame's decisions, as the reference's
 * write_key_frame_header writes them (svtav1-entropy/src/obu.rs:1268-1377;
 * AV1 spec 5.9.11, 5.9.19, 5.9.20). Host code; no device work. */
typedef struct zf_header_opts {
    int32_t monochrome;         /* NumPlanes = 1 (no chroma levels, strengths or lr types) */
    int32_t allow_intrabc;      /* 1: none of the three blocks is coded */
    int32_t enable_restoration; /* sequence header enable_restoration */
    int32_t sb_size;            /* 64 or 128 */
    int32_t sharpness;          /* loop_filter_sharpness 0..7 */
    int32_t pad;
} zf_header_opts;

/* Appends the fields MSB-first at bit *bit_pos of buf (cap bytes; bits past
 * *bit_pos are overwritten, earlier ones kept) and advances *bit_pos. The
 * chroma restoration unit size is d->lr[1].unit_size (lr_uv_shift is coded
 * when it differs from luma's). */
int32_t zf_write_filter_params(const zf_decisions *d, const zf_header_opts *o, uint8_t *buf, int32_t cap,
                               int32_t *bit_pos);

/* ---- Per-superblock restoration syntax -----------------------------------
 * The coded elements of a superblock's loop-restoration syntax, in coding
 * order, for the caller's range coder: what the reference's
 * write_lr_for_sb (svtav1-encoder/src/restoration.rs:1127-1182) codes for
 * every restoration unit whose top-left corner lies in the superblock
 * (corners_in_sb, :1070-1106), with write_wiener_filter's subexponential
 * tap coding against the running per-plane reference filter
 * (svtav1-entropy/src/lr.rs:67-236; plane-based window: 7-tap luma, so a
 * 5-tap luma solve codes TAP0 as 0; 5-tap chroma). Host code; no device
 * work. The range coder itself (AomWriter) stays the caller's. */
#define ZF_SYM_WIENER_RESTORE 1 /* one symbol on the adaptive wiener_restore CDF, value 0/1 */
#define ZF_SYM_BITS 2           /* nbits equiprobable bits of value, most significant first
                                   (write_literal; nbits 1 is write_bit) */
typedef struct zf_lr_sym {
    int32_t kind;               /* ZF_SYM_* */
    int32_t nbits;              /* ZF_SYM_BITS: 1..16 */
    uint32_t value;
    int16_t plane, pad;
    int32_t unit;               /* restoration unit (row-major in its plane) */
} zf_lr_sym;
/* Running reference filters of the three planes (C wiener_info[3]). */
typedef struct zf_wiener_refs {
    int16_t vfilter[3][8], hfilter[3][8];
} zf_wiener_refs;
/* The default filter in every plane: call at the first superblock of each
 * tile (svt_av1_reset_loop_restoration). */
void zf_wiener_refs_reset(zf_wiener_refs *r);
/* corners_in_sb: 1 and out = {rcol0, rcol1, rrow0, rrow1} when units of a
 * plane (unit_size, is_uv) have their corner in the superblock at
 * (mi_row, mi_col) of sb_mi mi, else 0 (negative: bad argument). frame_w is
 * the upscaled width under superres; sr_denom 9..16, or 0 for none. */
int32_t zf_lr_corners_in_sb(int32_t unit_size, int32_t is_uv, int32_t mi_row, int32_t mi_col, int32_t sb_mi,
                            int32_t frame_w, int32_t frame_h, int32_t sr_denom, int32_t out[4]);
/* Appends the superblock's elements to out (capacity cap) and returns
 * their count, updating refs as the coder would; ZF_ERR_ARG when out is
 * too small (nothing written, refs unchanged). Planes whose frame_rtype is
 * NONE code nothing; a WIENER plane codes, per unit, the restore flag and,
 * when set, the taps (d->lr_units[plane] must hold the plane's units). */
int32_t zf_lr_sb_syntax(const zf_decisions *d, int32_t mi_row, int32_t mi_col, int32_t sb_mi, int32_t frame_w,
                        int32_t frame_h, int32_t monochrome, int32_t sr_denom, zf_wiener_refs *refs,
                        zf_lr_sym *out, int32_t cap);

/* ---- Tile symbol coder: the filter syntax as bytes ------------------------
 * AV1's multi-symbol arithmetic coder (the encoder side of the AV1 spec's
 * symbol decoding process, 8.2.2-8.2.6), in place of the reference's
 * AomWriter over OdEcEnc (svtav1-entropy/src/writer.rs:18-80,
 * range_coder.rs:24-300): the same interval arithmetic, CDF adaptation
 * (cdf.rs:64-82) and final flush, so the same symbols give the same bytes.
 * The caller's entropy walk codes its own symbols through it and, at the
 * filter stage's places, the restoration units of each superblock
 * (zf_ec_lr_sb, at the superblock's start, write_lr_for_sb) and the
 * cdef_idx literal of each 64x64 filter block (zf_ec_cdef_block, after the
 * skip flag of every coded block). Host code; no device work. */
typedef struct zf_ec zf_ec;
zf_ec *zf_ec_create(void);                 /* NULL when out of host memory */
void zf_ec_destroy(zf_ec *ec);
void zf_ec_reset(zf_ec *ec);               /* an empty stream (OdEcEnc::reset) */
/* encode_bool_q15: bit with probability f / 32768 of a one (0 < f < 32768) */
int32_t zf_ec_bool(zf_ec *ec, int32_t bit, uint32_t f);
/* write_literal: nbits (0..32) equiprobable bits, most significant first */
int32_t zf_ec_literal(zf_ec *ec, uint32_t value, int32_t nbits);
/* write_symbol / write_cdf: symbol s of nsyms (2..16) under the inverse CDF
 * icdf (C layout, nsyms + 1 entries: icdf[nsyms - 1] = 0, the adaptation
 * counter at icdf[nsyms]); adapt != 0 updates icdf as the decoder will. */
int32_t zf_ec_symbol(zf_ec *ec, int32_t s, uint16_t *icdf, int32_t nsyms, int32_t adapt);
/* OdEcEnc::tell: bits used so far, the terminating bit included */
int32_t zf_ec_tell(const zf_ec *ec);
/* OdEcEnc::done: the stream's bytes into out (cap bytes); returns their
 * count, ZF_ERR_ARG when cap is too small. The coder stays usable: more
 * symbols may follow, and a later call returns the longer stream. */
int32_t zf_ec_done(zf_ec *ec, uint8_t *out, int32_t cap);
/* The default wiener_restore (use_wiener) CDF of a tile: {32768 - 11570, 0, 0}. */
void zf_wiener_restore_cdf_init(uint16_t cdf[3]);
/* Codes elements from zf_lr_sb_syntax: restore flags on wiener_cdf (adapted),
 * bits as literals. ZF_ERR_ARG on a malformed element (nothing coded). */
int32_t zf_ec_lr_syms(zf_ec *ec, const zf_lr_sym *syms, int32_t n, uint16_t wiener_cdf[3]);
/* zf_lr_sb_syntax for the superblock, coded at once: returns the element
 * count (refs and wiener_cdf advanced) or a negative code (nothing coded). */
int32_t zf_ec_lr_sb(zf_ec *ec, const zf_decisions *d, int32_t mi_row, int32_t mi_col, int32_t sb_mi, int32_t frame_w,
                    int32_t frame_h, int32_t monochrome, int32_t sr_denom, zf_wiener_refs *refs,
                    uint16_t wiener_cdf[3]);
/* Per-superblock cdef_idx state (the reference's CdefSbState,
 * svtav1-encoder/src/pipeline.rs:3965-3980; C cdef_transmitted[4]). */
typedef struct zf_cdef_sb {
    int32_t bits;                /* cdef_bits: 0 codes nothing */
    int32_t sb128;               /* 128x128 superblock: four filter blocks */
    uint8_t strengths[4];        /* strength index per 64x64 quadrant (TL, TR, BL, BR) */
    uint8_t transmitted[4];
} zf_cdef_sb;
/* At each superblock's start (superblock row/column sb_row, sb_col of
 * sb_size 64 or 128): reads the quadrants' indices from d->cdef_fb_idx
 * (pipeline.rs:2707-2745). */
int32_t zf_cdef_sb_begin(const zf_decisions *d, int32_t sb_row, int32_t sb_col, int32_t sb_size, zf_cdef_sb *st);
/* After a coded block's skip flag (block at luma sample block_x, block_y):
 * the first non-skip block of each 64x64 filter block codes that filter
 * block's index as cdef_bits literal bits (pipeline.rs:4995-5017; C
 * write_cdef; spec read_cdef). Returns the bits coded (0 or cdef_bits). */
int32_t zf_ec_cdef_block(zf_ec *ec, zf_cdef_sb *st, int32_t block_x, int32_t block_y, int32_t skip);

/* ---- Self-guided restoration (RESTORE_SGRPROJ) ---------------------------
 * No counterpart in the reference encoder: it never searches or signals
 * SGRPROJ (svtav1-dsp/src/restoration.rs:1280, svtav1-encoder/src/
 * restoration.rs:8); the reference project documents the filter in
 * specs/08-loop-filters.md:371-421. The filter is the AV1 specification's
 * box filter and self-guided projection (section 7.17.3, Sgr_Params); the
 * apply is decoder-exact (stripe-aware sample fetch). The search is this
 * library's: for every restoration unit and every parameter set of the
 * mask, the least-squares projection weights (solved exactly), then the SSE
 * of the unit filtered with them; the set of the smallest SSE wins (the
 * lowest set on ties). Units are the plane's 256-sample restoration units
 * (count_units_in_tile per dimension, rows offset by 8 >> ss_y), row-major;
 * the search filters each unit with samples clamped to the plane (no
 * stripes), like the Wiener search. */
typedef struct zf_sgr_plane {
    int32_t bit_depth;          /* 8 or 10 (u8 or u16 samples) */
    int32_t width, height;      /* plane dims; rows are width samples apart */
    int32_t ss_y;               /* 1 for 4:2:0 chroma (32-row stripes, offset 4) */
    int32_t on_device;          /* 1: the plane pointers are device pointers */
    const void *dgd;            /* post-CDEF plane (filter input) */
    const void *src;            /* source plane (search only) */
    const void *pre_cdef;       /* post-deblock plane (apply only: stripe edges) */
} zf_sgr_plane;

typedef struct zf_sgr_unit {
    int32_t set;                /* Sgr_Params index 0..15; -1: unit not filtered */
    int32_t xqd[2];             /* weights w0, w1 (w2 = 128 - w0 - w1) */
    int32_t pad;
    int64_t sse;                /* search: SSE of the unit filtered with set, xqd */
    int64_t sse_none;           /* search: SSE of the unfiltered unit */
} zf_sgr_unit;

/* Per-unit search over the sets of set_mask (bit k = set k, non-zero).
 * nunits must be the plane's unit count. */
int32_t zf_sgr_search(zf_ctx *ctx, const zf_sgr_plane *p, uint32_t set_mask, zf_sgr_unit *units,
                      int32_t nunits);
/* Decoder-exact apply into dst (width x height, same memory kind as the
 * planes, distinct from dgd and pre_cdef); units with set < 0 are copied. */
int32_t zf_sgr_apply(zf_ctx *ctx, const zf_sgr_plane *p, const zf_sgr_unit *units, int32_t nunits,
                     void *dst);

/* ---- Steps on either side of loop restoration ------------------------------
 * Superres: svtav1-dsp/src/superres.rs (scaled_size :140, the normative
 * upscale of one plane with one tile column, upscale_normative_plane :252);
 * the encoder upscales the post-CDEF recon with it before restoration
 * (pipeline.rs superres hook). Film grain: svtav1-encoder/src/film_grain.rs
 * (estimate_film_grain :74, run after the restoration apply at
 * pipeline.rs:3484-3485; synthesize_grain :127, the matching add). */
typedef struct zf_film_grain {
    int32_t apply_grain;
    uint16_t grain_seed;
    uint8_t num_y_points, num_cb_points, num_cr_points;
    uint8_t point_y_value[14], point_y_scaling[14];
    uint8_t point_cb_value[10], point_cb_scaling[10];
    uint8_t point_cr_value[10], point_cr_scaling[10];
    int8_t ar_coeffs_y[24], ar_coeffs_cb[25], ar_coeffs_cr[25];
    uint8_t ar_coeff_lag, ar_coeff_shift, grain_scale_shift;
    uint8_t cb_mult, cb_luma_mult, cr_mult, cr_luma_mult;
    uint8_t overlap_flag, clip_to_restricted_range, chroma_scaling_from_luma;
    uint16_t cb_offset, cr_offset;
    double noise_var;           /* the estimate's noise variance (not signalled) */
} zf_film_grain;

/* scaled_size: the coded (downscaled) dimension for a superres denominator
 * 9..16 (8 or > 16: unchanged). Host only. */
int32_t zf_superres_scaled_size(int32_t dim, int32_t denom);
/* Normative horizontal upscale src_width -> dst_width of rows rows (u8 when
 * bit_depth == 8, else u16 clipped to the bit depth; strides in samples). */
int32_t zf_superres_upscale(zf_ctx *ctx, const void *src, int32_t src_width, int32_t src_stride, void *dst,
                            int32_t dst_width, int32_t dst_stride, int32_t rows, int32_t bit_depth,
                            int32_t on_device);
/* Film-grain estimate from the u8 luma source and the filtered recon. */
int32_t zf_film_grain_estimate(zf_ctx *ctx, const uint8_t *src, const uint8_t *recon, int32_t width,
                               int32_t height, int32_t stride, int32_t on_device, zf_film_grain *out);
/* Adds synthesize_grain's noise to a u8 plane in place. */
int32_t zf_film_grain_synthesize(zf_ctx *ctx, uint8_t *frame, int32_t width, int32_t height, int32_t stride,
                                 int32_t on_device, const zf_film_grain *p);

typedef struct zf_kernel_time {
    char name[32];
    uint64_t launches;
    double total_ms;            /* CUDA-event time on the context's stream */
    uint64_t bytes;             /* algorithmic bytes of the launches (planes read and
                                   written once), where the library records them
                                   (the deblock level trials); else 0 */
} zf_kernel_time;

/* CUDA graphs (no counterpart in the reference). enable != 0: every
 * filter-stage / batch call captures its launch sequence after the deblock
 * level search (metadata upload, kernels, decision readback) into a graph,
 * updates the context's executable graph with it (instantiating a new one
 * when the sequence's shape changed) and launches that; passes are then not
 * separated by cancel checks (the flag is polled before and after).
 * Ignored while event profiling is on. */
int32_t zf_use_graphs(zf_ctx *ctx, int32_t enable);
/* out[0] graph launches, out[1] in-place updates, out[2] instantiations. */
int32_t zf_graph_stats(const zf_ctx *ctx, uint64_t out[3]);

/* Launch settings of a context (no counterpart in the reference: they
 * change how the stage runs on the GPU, never its results). */
typedef struct zf_tune {
    int32_t graphs;             /* 0/1: CUDA-graph launch mode (zf_use_graphs) */
    int32_t stats_tma;          /* 0/1: Wiener statistics rows of 8-bit planes by TMA */
    int32_t apply_group;        /* 64-px column tiles per restoration-apply CTA: 1..16 */
    int32_t stats_tc;           /* 0/1: Wiener statistics of 8-bit planes on the tensor cores
                                   (default 0: the CUDA-core form measured faster) */
    int32_t trial_tile;         /* Wiener trial tile edge without refinement: 32 or 64 (default) */
    int32_t db_levels;          /* deblock level trials per launch of the level search after a
                                   climb's first two launches: 2..8 (default 8) */
    double ms;                  /* zf_autotune: mean device time of one call (else 0) */
} zf_tune;
int32_t zf_get_tune(const zf_ctx *ctx, zf_tune *out);
/* ZF_ERR_ARG for a setting out of range. */
int32_t zf_set_tune(zf_ctx *ctx, const zf_tune *t);
/* Autotuner (no counterpart in the reference). Coordinate descent from the
 * context's current setting: each knob in turn -- graphs, the statistics
 * form (CUDA cores with TMA rows / with thread-staged rows / tensor cores),
 * apply_group in {1, 2, 4, 8, 16}, trial_tile in {64, 32}, db_levels in
 * {8, 4, 2} -- takes every value with the other knobs at the best setting
 * so far; a setting is timed once (one warm-up call, then `reps` calls timed
 * with CUDA events on the context's stream), each call the whole filter
 * stage on private copies of the frames' recon restored before every call
 * (zf_filter_stage for n == 1, zf_submit_batch otherwise), so the caller's
 * buffers are not written. Sets the fastest setting on the context and
 * writes it to *best; writes up to `max` timed settings with their times to
 * `cands` (may be NULL). Returns the number of settings timed (>= 1) or a
 * negative ZF_ERR_*. Allocates device memory for the copies (device
 * frames) and runs O(settings x reps) stage calls: a set-up step, not a
 * per-frame one. */
int32_t zf_autotune(zf_ctx *ctx, const zf_frame *frames, int32_t n, int32_t reps, zf_tune *best,
                    zf_tune *cands, int32_t max);

/* Iteration limit of the one device-side wait of the stage (the Wiener
 * statistics kernels waiting for their TMA tile loads or, in the tensor-
 * core form, for their MMAs), in steps of about
 * 100 ns (mbarrier try_wait with a suspend-time hint); 0 restores the
 * default of 2^20 steps, far beyond any real load. A CTA that gives up
 * drains its loads, records the timeout and the call returns
 * ZF_ERR_TIMEOUT; the context stays usable. No counterpart in the
 * reference. */
int32_t zf_set_wait_limit(zf_ctx *ctx, uint32_t iterations);
/* zf_set_wait_limit value under which the wait gives up before its first
 * step, as if the loads never arrived: the test of the timeout path. */
#define ZF_WAIT_GIVE_UP 0xFFFFFFFFu

/* Kernel launches issued by this context since zf_create. */
uint64_t zf_launch_count(const zf_ctx *ctx);
/* enable != 0: bracket every kernel launch with CUDA events (adds a little
 * host overhead); the per-kernel totals accumulate until zf_profile_reset. */
int32_t zf_profile_enable(zf_ctx *ctx, int32_t enable);
void zf_profile_reset(zf_ctx *ctx);
/* Copies up to max entries; returns the number of distinct kernels. */
int32_t zf_profile_read(const zf_ctx *ctx, zf_kernel_time *out, int32_t max);

#ifdef __cplusplus
}
#endif
#endif /* ZF_FILTER_H */
