// zf_host.cu -- host orchestration and the C ABI (include/zf_filter.h).
//
// One call runs a batch of frames through the selected passes. Everything a
// pass needs is laid out in one device arena: three working plane sets per
// frame (A: input recon, reused for the post-CDEF planes; B: post-deblock;
// C: post-restoration), the source planes, the packed geometry and the
// search scratch. Decisions are computed on the device (CDEF joint search,
// Wiener solve and frame RD) so the passes after the deblock level search
// are one fixed sequence of launches; only the deblock hill-climb of
// presets <= 5 round-trips to the host, one step per launch.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "../../include/zf_av1_tables.h"
#include "../../include/zf_filter.h"
#include "zf_kernels.cuh"

using zf::CdefParams;
using zf::FrameDesc;
using zf::LrPlane;
using zf::LrUnit;
using zf::UnitRect;
using zf::WorkItem;

static_assert(sizeof(zf::PackedUnit) == sizeof(zf_lr_unit), "unit record layout");

struct zf_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    uint8_t *arena = nullptr;
    size_t arena_cap = 0;
    uint64_t budget = 0;
    volatile int32_t *cancel = nullptr;
    // launch accounting / optional event profiling
    uint64_t launches = 0;
    bool profiling = false;
    struct Pending {
        const char *name;
        cudaEvent_t a, b;
        uint64_t bytes;
    };
    std::vector<Pending> pending;
    std::vector<zf_kernel_time> totals;
    // pinned host staging: the batch's metadata image (descriptors, work
    // lists, unit rectangles) goes up in one copy, the decisions come back
    // in one copy
    uint8_t *h_meta = nullptr, *h_out = nullptr;
    size_t h_meta_cap = 0, h_out_cap = 0;
    // job lists of the gathered host-plane copies (pinned up, device side)
    uint8_t *h_jobs = nullptr, *d_jobs = nullptr;
    size_t h_jobs_cap = 0, d_jobs_cap = 0;
    // CUDA graph mode: one executable graph, updated from each call's capture
    bool graphs = false;
    bool capturing = false;
    bool tma = true;  // statistics kernel rows by TMA where the planes allow
    bool stats_tc = false;  // statistics of 8-bit 5-tap planes on the tensor cores (k_lr_stats_tc)
    int trial_tile = 64;    // k_lr_trial_tiles tile edge (32 or 64)
    int db_levels = 8;      // deblock level trials per launch after a climb's first two launches
    uint32_t wait_limit = 1u << 20;  // statistics kernel's TMA wait (iterations)
    int apply_group = 8;  // 64-px column tiles per restoration-apply CTA
    // search trace (zf_trace / ZF_TRACE): one text line per trial, filter
    // block and restoration unit in the reference's debug-dump formats
    FILE *trace = nullptr;
    bool trace_owned = false;
    cudaGraphExec_t gexec = nullptr;
    std::vector<uint64_t> gsig;  // node kinds, kernel functions and cluster shapes of gexec's graph
    uint64_t graph_launches = 0, graph_updates = 0, graph_instantiations = 0;
};

namespace {
// Bracket one launch: count it and, when profiling, record events on the
// context stream around it.
struct LaunchScope {
    zf_ctx *ctx;
    const char *name;
    uint64_t bytes;  // algorithmic bytes of the launch, 0 when not recorded
    cudaEvent_t a = nullptr, b = nullptr;
    LaunchScope(zf_ctx *c, const char *n, uint64_t nbytes = 0) : ctx(c), name(n), bytes(nbytes) {
        ctx->launches++;
        if (ctx->profiling && cudaEventCreate(&a) == cudaSuccess && cudaEventCreate(&b) == cudaSuccess)
            cudaEventRecord(a, ctx->stream);
    }
    ~LaunchScope() {
        if (a && b) {
            cudaEventRecord(b, ctx->stream);
            ctx->pending.push_back({name, a, b, bytes});
        }
    }
};
// Fold completed event pairs into the per-kernel totals (after a sync).
void collect_profile(zf_ctx *ctx) {
    for (auto &p : ctx->pending) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p.a, p.b);
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
        zf_kernel_time *t = nullptr;
        for (auto &k : ctx->totals)
            if (std::strncmp(k.name, p.name, sizeof(k.name)) == 0) t = &k;
        if (!t) {
            zf_kernel_time k;
            std::memset(&k, 0, sizeof(k));
            std::strncpy(k.name, p.name, sizeof(k.name) - 1);
            ctx->totals.push_back(k);
            t = &ctx->totals.back();
        }
        t->launches += 1;
        t->total_ms += ms;
        t->bytes += p.bytes;
    }
    ctx->pending.clear();
}
}  // namespace

namespace {

enum : unsigned {
    STG_DB_PICK = 1u << 0,
    STG_DB_APPLY = 1u << 1,
    STG_CDEF_SEARCH = 1u << 2,
    STG_CDEF_APPLY = 1u << 3,
    STG_LR_SEARCH = 1u << 4,
    STG_LR_APPLY = 1u << 5,
    STG_ALL = 0x3f,
};

// Where the caller's rec[] goes in, and which plane set comes back out.
enum PlaneSet { SET_A = 0, SET_B = 1, SET_C = 2 };

// zf_deblock_sse_table's request: SSE of one plane at each of n levels.
struct DbTable {
    int plane, n;
    const int32_t *levels;
    int64_t *sse;
};
// zf_cdef_search_rows' outputs (caller arrays; see the header).
struct CdefRows {
    uint64_t *mse;
    uint8_t *has_row;
    int32_t *ncand;
};

struct Run {
    unsigned stages;
    PlaneSet rec_in;
    PlaneSet rec_out;
    bool pre_cdef_in;       // zf_lr_apply: pre_cdef[] -> B
    const void *const *pre_cdef;
    bool lf_given;          // decisions provided by the caller
    bool cdef_given;
    bool lr_given;
    DbTable *table = nullptr;    // zf_deblock_sse_table: trials of the caller's levels
    CdefRows *rows = nullptr;    // zf_cdef_search_rows: the search's mse rows
};

int fail(zf_ctx *ctx, int code, const std::string &msg) {
    if (ctx) ctx->err = msg;
    return code;
}

#define CU(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return fail(ctx, ZF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));    \
    } while (0)

// ---- reference decision helpers (host scalar) ----------------------------

// kf_full_lambda_8bit_unweighted (svtav1-encoder/src/pd0.rs:218).
uint32_t lambda_8bit_unweighted(int q) {
    const double d = (double)zf_dc_qlookup_8[q];
    const int64_t rdmult = (int64_t)((3.3 + 0.0015 * d) * d * d);
    return (uint32_t)((rdmult * 150) >> 7);
}
// kf_full_lambda_bd10_unweighted (pd0.rs:330).
uint32_t lambda_bd10_unweighted(int q) {
    const double d = (double)zf_dc_qlookup_10[q];
    int64_t rdmult = (int64_t)((3.3 + 0.0015 * d) * d * d);
    rdmult = (rdmult + 8) >> 4;
    rdmult = std::max<int64_t>(rdmult, 1);
    return (uint32_t)((rdmult * 128) >> 7);
}

// pick_filter_levels_key_frame (deblock.rs:55-81).
void key_frame_levels(int q, int bd, uint8_t out[4]) {
    int fg;
    if (bd == 8) {
        const int qs = zf_ac_qlookup_8[q];
        fg = (qs * 17563 - 421574 + (1 << 17)) >> 18;
    } else {
        const int qs = zf_ac_qlookup_10[q];
        fg = ((qs * 20723 + 4060632 + (1 << 19)) >> 20) - 4;
    }
    const int fc = fg / 2;
    const uint8_t y = (uint8_t)std::min(std::max(fg, 0), 63), uv = (uint8_t)std::min(std::max(fc, 0), 63);
    out[0] = out[1] = y;
    out[2] = out[3] = uv;
}

// pick_cdef_params_key_frame (cdef.rs:151-206): f32 + roundf (intra arm) or
// f64 + truncation (screen arm). Compiled with -ffp-contract=off.
void cdef_qp_params(int q, int bd, bool screen, int out[3]) {
    const int q_raw = bd == 8 ? zf_ac_qlookup_8[q] : zf_ac_qlookup_10[q];
    const int qi = q_raw >> (bd - 8);
    int y1, y2, u1, u2;
    if (screen) {
        const double d = (double)qi;
        y1 = (int)(5.88217781e-06 * d * d + 6.10391455e-03 * d + 9.95043102e-02);
        y2 = (int)(-7.79934857e-06 * d * d + 6.58957830e-03 * d + 8.81045025e-01);
        u1 = (int)(-6.79500136e-06 * d * d + 1.02695586e-02 * d + 1.36126802e-01);
        u2 = (int)(-9.99613695e-08 * d * d - 1.79361339e-05 * d + 1.17022324e+0);
    } else {
        const float f = (float)qi;
        y1 = (int)roundf(f * f * 0.0000033731974f + f * 0.008070594f + 0.0187634f);
        y2 = (int)roundf(f * f * 0.0000029167343f + f * 0.0027798624f + 0.0079405f);
        u1 = (int)roundf(f * f * -0.0000130790995f + f * 0.012892405f - 0.00748388f);
        u2 = (int)roundf(f * f * 0.0000032651783f + f * 0.00035520183f + 0.00228092f);
    }
    auto cl = [](int v, int hi) { return std::min(std::max(v, 0), hi); };
    out[0] = 3 + (q >> 6);
    out[1] = cl(y1, 15) * 4 + cl(y2, 3);
    out[2] = cl(u1, 15) * 4 + cl(u2, 3);
}

// cdef_search_cfg_for_preset (cdef.rs:788-810).
void cdef_search_cfg(int preset, CdefParams &cp) {
    static const int PF[16] = {0, 4, 8, 12, 16, 20, 24, 28, 32, 36, 40, 44, 48, 52, 56, 60};
    std::vector<int> first, extra;
    if (preset == 0) {
        first = {0, 1, 2, 4, 5, 6, 8, 9, 10, 12, 13, 14};
        extra = {1, 2, 3};
    } else if (preset <= 3) {
        first = {0, 4, 8, 12, 15};
        extra = {1, 2, 3};
    } else if (preset <= 5) {
        first = {0, 7, 15};
        extra = {2};
    } else {
        first = {0, 15};
        extra = {2};
    }
    int n = 0;
    for (int i : first) cp.fs[n++] = PF[i];
    cp.first_pass_num = n;
    for (int i : first)
        for (int d : extra) cp.fs[n++] = PF[i] + d;
    cp.ncand = n;
    const int sub = preset >= 6 ? 4 : 1;
    cp.sub_y = std::min(sub, 4);
    cp.sub_uv = std::min(sub, 1);
}

// CDEF policy of pipeline.rs:3042-3144 for a still key frame: the RDO
// search at presets <= 6, the qp closed form above.
void cdef_policy(const zf_frame *f, CdefParams &cp) {
    if (f->preset <= 6) {
        cp.mode = 1;
        cdef_search_cfg(f->preset, cp);
        cp.damping = 3 + (f->qindex >> 6);
        cp.lambda = f->bit_depth == 8 ? lambda_8bit_unweighted(f->qindex) : lambda_bd10_unweighted(f->qindex);
    } else {
        int q[3];
        cdef_qp_params(f->qindex, f->bit_depth, f->sc_class5 != 0, q);
        cp.mode = 2;
        cp.damping = q[0];
        cp.bits = 0;
        cp.y_str[0] = (uint8_t)q[1];
        cp.uv_str[0] = (uint8_t)q[2];
    }
}

int count_units_in_tile(int unit, int size) { return std::max((size + (unit >> 1)) / unit, 1); }

// foreach_rest_unit_in_tile (svtav1-dsp/src/restoration.rs:1395-1448).
void rest_units(int pw, int ph, int ss, std::vector<UnitRect> &out) {
    const int unit = 256, ext = unit * 3 / 2;
    out.clear();
    for (int y0 = 0; y0 < ph;) {
        const int rh = ph - y0, h = rh < ext ? rh : unit;
        UnitRect r;
        r.v_start = y0;
        r.v_end = y0 + h;
        const int voff = 8 >> ss;
        r.v_start = std::max(0, r.v_start - voff);
        if (r.v_end < ph) r.v_end -= voff;
        for (int x0 = 0; x0 < pw;) {
            const int rw = pw - x0, w = rw < ext ? rw : unit;
            r.h_start = x0;
            r.h_end = x0 + w;
            out.push_back(r);
            x0 += w;
        }
        y0 += h;
    }
}

// The deblock level hill-climb of search_filter_level (deblock.rs:307-411)
// replayed over the SSEs measured so far: returns the levels that the next
// step needs (both candidates of a step are requested together), or marks
// the search done. The state where it stopped (mid level, step, direction)
// is left in the fields for speculate().
struct HillClimb {
    int64_t err[64];
    bool have[64];
    int conv_th = 0;
    bool done = false;
    int result = 0;
    int at_mid = 0, at_step = 4, at_dir = 0;
    HillClimb() {
        for (int i = 0; i < 64; ++i) {
            err[i] = 0;
            have[i] = false;
        }
    }
    int needs(int out[2]) {
        at_mid = 0;
        at_step = 4;
        at_dir = 0;
        if (!have[0]) {
            out[0] = 0;
            return 1;
        }
        int dir = 0, mid = 0, step = 4, best = 0, conv = 0;
        int64_t best_err = err[0];
        while (step > 0) {
            const int hi = std::min(mid + step, 63), lo = std::max(mid - step, 0);
            int64_t bias = (best_err >> (15 - (mid / 8))) * (int64_t)step;
            bias >>= 1;
            const bool need_lo = dir <= 0 && lo != mid, need_hi = dir >= 0 && hi != mid;
            int n = 0;
            if (need_lo && !have[lo]) out[n++] = lo;
            if (need_hi && !have[hi]) out[n++] = hi;
            if (n) {
                at_mid = mid;
                at_step = step;
                at_dir = dir;
                return n;
            }
            if (need_lo && err[lo] < best_err + bias) {
                if (err[lo] < best_err) best_err = err[lo];
                best = lo;
            }
            if (need_hi && err[hi] < best_err - bias) {
                best_err = err[hi];
                best = hi;
            }
            if (best == mid) {
                conv += 1;
                if (conv == conv_th) step = 0;
                else step /= 2;
                dir = 0;
            } else {
                dir = best < mid ? -1 : 1;
                mid = best;
            }
        }
        done = true;
        result = best;
        return 0;
    }
    // The levels the finished climb evaluated, in the order
    // search_filter_level calls try_filter_frame.
    void trial_order(std::vector<int> &out) const {
        out.clear();
        bool seen[64] = {};
        auto visit = [&](int l) {
            if (!seen[l]) out.push_back(l);
            seen[l] = true;
        };
        visit(0);
        int dir = 0, mid = 0, step = 4, best = 0, conv = 0;
        int64_t best_err = err[0];
        while (step > 0) {
            const int hi = std::min(mid + step, 63), lo = std::max(mid - step, 0);
            int64_t bias = (best_err >> (15 - (mid / 8))) * (int64_t)step;
            bias >>= 1;
            if (dir <= 0 && lo != mid) {
                visit(lo);
                if (err[lo] < best_err + bias) {
                    if (err[lo] < best_err) best_err = err[lo];
                    best = lo;
                }
            }
            if (dir >= 0 && hi != mid) {
                visit(hi);
                if (err[hi] < best_err - bias) {
                    best_err = err[hi];
                    best = hi;
                }
            }
            if (best == mid) {
                conv += 1;
                if (conv == conv_th) step = 0;
                else step /= 2;
                dir = 0;
            } else {
                dir = best < mid ? -1 : 1;
                mid = best;
            }
        }
    }
};

// Levels to evaluate in one trial launch for a climb that needs `need`:
// the needed levels, then speculatively the levels the next steps may ask
// for -- the continuation of the climb at its current step in the needed
// directions (mid +- 2 step, +- 3 step, ...) and, when the climb refines
// after converging (conv_th != 1), the half and quarter steps around the
// current mid. Only the needed levels decide anything; the others are cached
// SSEs that save a launch and a host round trip when the climb reaches them.
void speculate(const HillClimb &hc, const int *need, int m, int cap, std::vector<int> &lv) {
    lv.clear();
    bool in[64] = {};
    auto add = [&](int l) {
        if ((int)lv.size() >= cap || l < 0 || l > 63 || in[l] || hc.have[l]) return;
        in[l] = true;
        lv.push_back(l);
    };
    for (int k = 0; k < m; ++k) add(need[k]);
    const int mid = hc.at_mid, step = hc.at_step;
    bool up = false, down = false;
    for (int k = 0; k < m; ++k) {
        up = up || need[k] > mid || (need[k] == 0 && mid == 0);
        down = down || need[k] < mid;
    }
    for (int k = 1; k <= 16 && (int)lv.size() < cap; ++k) {
        if (up) add(mid + k * step);
        if (down) add(mid - k * step);
        if (hc.conv_th != 1 && k == 2) {
            add(mid + step / 2);
            add(mid - step / 2);
        }
        if (hc.conv_th != 1 && k == 3) {
            add(mid + step / 4);
            add(mid - step / 4);
        }
        if (!up && !down) break;
    }
}

// ---- per-frame plan -------------------------------------------------------

struct Plan {
    const zf_frame *in = nullptr;
    zf_decisions *out = nullptr;
    FrameDesc d;
    size_t px = 1;                    // bytes per pixel
    size_t pbytes[3] = {0, 0, 0};     // plane bytes (aligned canvas)
    int nplanes = 1;
    int nfb = 0;
    size_t off_set[3][3];             // [set A/B/C][plane]
    size_t off_src[3];
    size_t off_mi = 0, off_mse = 0, off_ids = 0, off_rows32 = 0, off_cdir = 0;
    // relative to the batch's units region (zeroed with one memset)
    size_t off_units[3];
    // relative to the rectangles part of the metadata region
    size_t off_rects[3];
    // relative to the output region (read back with one copy)
    size_t off_fbrow = 0, off_fbidx = 0, off_stats = 0, off_packed[3];
    std::vector<UnitRect> rects[3];
    int hunits[3], vunits[3];
    bool db_search = false;
    bool zero_copy = false;  // kernels read and write the caller's device planes directly
};

size_t align_up(size_t v, size_t a) { return (v + a - 1) & ~(a - 1); }

// Dynamic shared memory opted in for k_cdef_finish's compacted rows, and
// for the single-CTA form's rows, best column and partials.
constexpr size_t kFinishSmemCap = 160 * 1024;
constexpr int kFinish1SmemCap = 200 * 1024;
constexpr int kFinish1MaxFb = 1024;  // filter blocks (a 2048x2048 frame)
// k_cdef_joint launch groups: (4 or 6 candidates) x (1, 2 or 4 rows per thread)
constexpr int kJointGroups = 6;
int joint_group(int ncand, int rpt) { return (ncand == 6 ? 3 : 0) + (rpt == 4 ? 2 : rpt == 2 ? 1 : 0); }
int joint_group_ncand(int g) { return g < 3 ? 4 : 6; }
int joint_group_rpt(int g) { return 1 << (g % 3); }
// k_lr_finish: 32 B per unit plus the pair table of <= 200 units (or 32 B
// per unit alone for larger planes; 4096 units at most)
constexpr int kLrFinishSmemCap = 160 * 1024;

// Opt the kernels with large dynamic shared memory in once per device
// (a function attribute; set at context creation, not per call).
cudaError_t set_kernel_attributes() {
    cudaError_t e = cudaFuncSetAttribute(zf::k_cdef_finish1, cudaFuncAttributeMaxDynamicSharedMemorySize, kFinish1SmemCap);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(zf::k_cdef_finish, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFinishSmemCap);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(zf::k_lr_finish, cudaFuncAttributeMaxDynamicSharedMemorySize, kLrFinishSmemCap);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(zf::k_lr_stats_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)zf::lr_stats_tc_smem());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(zf::k_lr_trial, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)zf::lr_trial_smem(zf::kTrialMaxTilesHost));
    if (e == cudaSuccess) e = zf::joint_set_attributes();
    if (e == cudaSuccess) e = zf::sgr_set_attributes();
    return e;
}

int validate_frame(zf_ctx *ctx, const zf_frame *f) {
    if (!f) return fail(ctx, ZF_ERR_ARG, "frame is NULL");
    if (f->bit_depth != 8 && f->bit_depth != 10) return fail(ctx, ZF_ERR_UNSUPPORTED, "bit_depth must be 8 or 10");
    if (f->width <= 0 || f->height <= 0 || (f->width & 7) || (f->height & 7))
        return fail(ctx, ZF_ERR_INVALID_DIMS, "width/height must be positive multiples of 8");
    if (f->true_width <= 0 || f->true_height <= 0 || f->true_width > f->width || f->true_height > f->height)
        return fail(ctx, ZF_ERR_INVALID_DIMS, "true dims must be in (0, aligned dims]");
    if (f->width > 16384 || f->height > 16384) return fail(ctx, ZF_ERR_INVALID_DIMS, "frame larger than 16384");
    if (f->qindex < 0 || f->qindex > 255 || f->preset < 0 || f->preset > 13 || f->sharpness < 0 || f->sharpness > 7)
        return fail(ctx, ZF_ERR_ARG, "qindex/preset/sharpness out of range");
    if (!f->src[0] || !f->rec[0] || !f->mi) return fail(ctx, ZF_ERR_ARG, "missing plane or geometry pointer");
    if (f->chroma_420 && (!f->src[1] || !f->src[2] || !f->rec[1] || !f->rec[2]))
        return fail(ctx, ZF_ERR_ARG, "missing chroma plane");
    return ZF_OK;
}

bool lr_enabled(const zf_frame *f) {
    return f->enable_restoration && f->preset <= 6 && f->true_width >= 64 && f->true_height >= 64;
}

// Offsets: per-frame device buffers at `cursor`; the unit accumulators,
// rectangles and outputs in three batch-wide regions (ucur, rcur, ocur).
void plan_frame(Plan &p, const zf_frame *f, size_t &cursor, size_t &ucur, size_t &rcur, size_t &ocur) {
    p.in = f;
    std::memset(&p.d, 0, sizeof(p.d));
    FrameDesc &d = p.d;
    d.bd = f->bit_depth;
    d.w = f->width;
    d.h = f->height;
    d.tw = f->true_width;
    d.th = f->true_height;
    d.chroma = f->chroma_420 ? 1 : 0;
    d.preset = f->preset;
    d.qindex = f->qindex;
    d.sharpness = f->sharpness;
    d.mi_cols = f->width / 4;
    d.mi_rows = f->height / 4;
    d.nhfb = (f->width + 63) / 64;
    d.nvfb = (f->height + 63) / 64;
    p.nfb = d.nhfb * d.nvfb;
    p.px = f->bit_depth == 8 ? 1 : 2;
    p.nplanes = f->chroma_420 ? 3 : 1;
    p.pbytes[0] = (size_t)f->width * f->height * p.px;
    p.pbytes[1] = p.pbytes[2] = (size_t)(f->width / 2) * (f->height / 2) * p.px;
    auto take_in = [](size_t &c, size_t n) {
        c = align_up(c, 256);
        size_t o = c;
        c += n;
        return o;
    };
    auto take = [&](size_t n) { return take_in(cursor, n); };
    for (int s = 0; s < 3; ++s)
        for (int pl = 0; pl < 3; ++pl) p.off_set[s][pl] = pl < p.nplanes ? take(p.pbytes[pl]) : 0;
    for (int pl = 0; pl < 3; ++pl) p.off_src[pl] = pl < p.nplanes ? take(p.pbytes[pl]) : 0;
    p.off_mi = take((size_t)d.mi_cols * d.mi_rows * 4);
    p.off_mse = take((size_t)p.nfb * 2 * zf::kMaxCand * 8);
    p.off_ids = take((size_t)zf::kFinLevels * p.nfb * 4);
    p.off_rows32 = take((size_t)zf::kFinLevels * p.nfb * 2 * zf::kMaxCand * 4);
    p.off_cdir = take((size_t)p.nfb * 64);
    p.off_fbrow = take_in(ocur, p.nfb);
    p.off_fbidx = take_in(ocur, p.nfb);
    p.off_stats = take_in(ocur, 4 * 8);
    cdef_policy(f, d.cdef);
    // Loop restoration (pipeline.rs:3225-3381).
    d.lr_on = lr_enabled(f) ? 1 : 0;
    d.rdmult = f->bit_depth == 10 ? (int64_t)lambda_bd10_unweighted(f->qindex) * 16
                                  : (int64_t)lambda_8bit_unweighted(f->qindex);
    for (int pl = 0; pl < 3; ++pl) {
        const int ss = pl ? 1 : 0;
        const int pw = pl ? (f->true_width + 1) / 2 : f->true_width;
        const int ph = pl ? (f->true_height + 1) / 2 : f->true_height;
        p.hunits[pl] = count_units_in_tile(256, pw);
        p.vunits[pl] = count_units_in_tile(256, ph);
        LrPlane &L = d.lr[pl];
        L.on = d.lr_on && (pl == 0 || f->chroma_420);
        L.win = 5;  // filter_tap_lvl 2 at every enabled preset (restoration.rs:82-107)
        L.pw = pw;
        L.ph = ph;
        L.stride = pl ? f->width / 2 : f->width;
        L.hunits = p.hunits[pl];
        L.vunits = p.vunits[pl];
        L.refine = f->preset <= 3;
        rest_units(pw, ph, ss, p.rects[pl]);
        p.off_rects[pl] = take_in(rcur, p.rects[pl].size() * sizeof(UnitRect));
        p.off_units[pl] = take_in(ucur, L.on ? p.rects[pl].size() * sizeof(LrUnit) : 0);
        p.off_packed[pl] = take_in(ocur, L.on ? p.rects[pl].size() * sizeof(zf::PackedUnit) : 0);
    }
    p.db_search = f->preset <= 5;
}

void bind_pointers(Plan &p, uint8_t *base, uint8_t *units, uint8_t *rects, uint8_t *out) {
    FrameDesc &d = p.d;
    for (int pl = 0; pl < 3; ++pl) {
        const bool on = pl < p.nplanes;
        d.A[pl] = on ? base + p.off_set[0][pl] : nullptr;
        d.IN[pl] = d.A[pl];
        d.B[pl] = on ? base + p.off_set[1][pl] : nullptr;
        d.C[pl] = on ? base + p.off_set[2][pl] : nullptr;
        d.S[pl] = on ? base + p.off_src[pl] : nullptr;
        d.lr[pl].rects = (UnitRect *)(rects + p.off_rects[pl]);
        d.lr[pl].units = d.lr[pl].on ? (LrUnit *)(units + p.off_units[pl]) : nullptr;
        d.lr[pl].packed = d.lr[pl].on ? (zf::PackedUnit *)(out + p.off_packed[pl]) : nullptr;
    }
    d.mi = (const uint32_t *)(base + p.off_mi);
    d.mse = (uint64_t *)(base + p.off_mse);
    d.fb_row = out + p.off_fbrow;
    d.fb_idx = out + p.off_fbidx;
    d.cdef_ids = (int *)(base + p.off_ids);
    d.cdef_rows32 = (uint32_t *)(base + p.off_rows32);
    d.cdir = base + p.off_cdir;
    d.cdef_stats = (unsigned long long *)(out + p.off_stats);
}

// Pinned host staging buffers (grow only).
int ensure_host(zf_ctx *ctx, uint8_t *&buf, size_t &cap, size_t need) {
    if (need <= cap) return ZF_OK;
    if (buf) {
        cudaStreamSynchronize(ctx->stream);
        cudaFreeHost(buf);
        buf = nullptr;
        cap = 0;
    }
    const size_t c = align_up(need + need / 4, 1 << 16);
    if (cudaHostAlloc((void **)&buf, c, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, ZF_ERR_ALLOC, "pinned host staging allocation failed");
    }
    cap = c;
    return ZF_OK;
}

// The job buffers of the gathered copies: room for `njobs` jobs (pinned
// staging and device side), grown when a call needs more.
int ensure_jobs(zf_ctx *ctx, size_t njobs) {
    const size_t need = njobs * sizeof(zf::CopyJob);
    const int rc = ensure_host(ctx, ctx->h_jobs, ctx->h_jobs_cap, need);
    if (rc != ZF_OK) return rc;
    if (need <= ctx->d_jobs_cap) return ZF_OK;
    if (ctx->d_jobs) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(ctx->d_jobs);
        ctx->d_jobs = nullptr;
        ctx->d_jobs_cap = 0;
    }
    const size_t c = align_up(need + need / 4, 1 << 12);
    if (cudaMalloc((void **)&ctx->d_jobs, c) != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, ZF_ERR_ALLOC, "copy job list allocation failed");
    }
    ctx->d_jobs_cap = c;
    return ZF_OK;
}

int ensure_arena(zf_ctx *ctx, size_t need) {
    if (ctx->budget && need > ctx->budget)
        return fail(ctx, ZF_ERR_ALLOC, "device footprint " + std::to_string(need) + " exceeds the HBM budget");
    if (need <= ctx->arena_cap) return ZF_OK;
    if (ctx->arena) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(ctx->arena);
        ctx->arena = nullptr;
        ctx->arena_cap = 0;
    }
    size_t cap = align_up(need + need / 8, 1 << 20);
    if (cudaMalloc((void **)&ctx->arena, cap) != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, ZF_ERR_ALLOC, "cudaMalloc of the device arena failed");
    }
    ctx->arena_cap = cap;
    return ZF_OK;
}

int check_cancel(zf_ctx *ctx) {
    if (ctx->capturing) return ZF_OK;  // polled again after the graph
    if (ctx->cancel && *ctx->cancel) {
        cudaStreamSynchronize(ctx->stream);
        return fail(ctx, ZF_ERR_CANCELLED, "cancelled");
    }
    return ZF_OK;
}

// Copy a plane between caller memory (host or device) and the arena.
int copy_in(zf_ctx *ctx, void *dst, const void *src, size_t n, bool on_device) {
    CU(cudaMemcpyAsync(dst, src, n, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ctx->stream));
    return ZF_OK;
}
int copy_out(zf_ctx *ctx, void *dst, const void *src, size_t n, bool on_device) {
    CU(cudaMemcpyAsync(dst, src, n, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, ctx->stream));
    return ZF_OK;
}

// Caller host planes that the device addresses directly (page-locked and
// mapped: cudaPointerGetAttributes gives a device pointer) and that are at
// most kGatherMaxBytes go through one k_copy_list launch per direction when
// a call has at least kGatherMinCopies of them (a batch of small images is
// hundreds of copies, each with its own fixed cost: 6.2 -> 12.1 GPix/s for
// the 256-image batch through host buffers); fewer, larger planes and
// pageable memory keep a cudaMemcpyAsync each, which measured as fast or
// faster for single frames.
constexpr size_t kGatherMaxBytes = 4u << 20;
constexpr size_t kGatherMinCopies = 16;
void *mapped_host(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // an unknown pointer is pageable host memory
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}
struct HostCopies {
    struct Copy {
        void *dst;
        const void *src;
        size_t n;
        bool to_device;
        void *mapped;  // the host side's device address
    };
    std::vector<Copy> copies;
    // dst and src as cudaMemcpyAsync would take them; true when queued
    bool add(void *dst, const void *src, size_t n, bool to_device) {
        if (n == 0 || n > kGatherMaxBytes) return false;
        void *h = mapped_host(to_device ? src : dst);
        if (!h) return false;
        copies.push_back({dst, src, n, to_device, h});
        return true;
    }
};
// Issue the queued copies: one gathered launch when there are enough of
// them (the job list goes to slot `slot` of the context's job buffers,
// sized for the call beforehand), else a cudaMemcpyAsync each.
int flush_copies(zf_ctx *ctx, const HostCopies &hc, size_t slot) {
    if (hc.copies.empty()) return ZF_OK;
    if (hc.copies.size() < kGatherMinCopies) {
        for (const auto &c : hc.copies)
            CU(cudaMemcpyAsync(c.dst, c.src, c.n, c.to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost,
                               ctx->stream));
        return ZF_OK;
    }
    std::vector<zf::CopyJob> jobs;
    jobs.reserve(hc.copies.size());
    uint64_t chunks = 0;
    for (const auto &c : hc.copies) {
        zf::CopyJob j;
        j.src = c.to_device ? static_cast<const uint8_t *>(c.mapped) : static_cast<const uint8_t *>(c.src);
        j.dst = c.to_device ? static_cast<uint8_t *>(c.dst) : static_cast<uint8_t *>(c.mapped);
        j.bytes = c.n;
        j.first_chunk = chunks;
        chunks += (c.n + zf::kCopyChunk - 1) / zf::kCopyChunk;
        jobs.push_back(j);
    }
    const size_t bytes = jobs.size() * sizeof(zf::CopyJob), off = slot * sizeof(zf::CopyJob);
    std::memcpy(ctx->h_jobs + off, jobs.data(), bytes);
    CU(cudaMemcpyAsync(ctx->d_jobs + off, ctx->h_jobs + off, bytes, cudaMemcpyHostToDevice, ctx->stream));
    { LaunchScope ls_(ctx, "k_copy_list");
    CU(zf::launch_copy_list(reinterpret_cast<const zf::CopyJob *>(ctx->d_jobs + off), (int)jobs.size(), chunks,
                            ctx->stream)); }
    return ZF_OK;
}

// Work lists: one item per tile range; CTA ranges are prefix sums.
struct WorkList {
    std::vector<WorkItem> items;
    int ctas = 0;
    void add(int frame, int plane, int a, int b, int n) {
        if (n <= 0) return;
        WorkItem w;
        w.frame = frame;
        w.plane = plane;
        w.a = a;
        w.b = b;
        w.cta_begin = ctas;
        w.ctas = n;
        items.push_back(w);
        ctas += n;
    }
    // Coarse index stored after the items (find_item): entry k is the item
    // owning CTA 32 k, then a last entry nitems - 1. One-item lists have none.
    size_t coarse_count() const { return items.size() > 1 ? (size_t)(ctas + 31) / 32 + 1 : 0; }
    size_t bytes() const { return items.size() * sizeof(WorkItem) + coarse_count() * sizeof(int); }
    void write(uint8_t *dst) const {
        std::memcpy(dst, items.data(), items.size() * sizeof(WorkItem));
        const size_t nc = coarse_count();
        if (!nc) return;
        int *c = reinterpret_cast<int *>(dst + items.size() * sizeof(WorkItem));
        size_t it = 0;
        for (size_t k = 0; k + 1 < nc; ++k) {
            const int cta = (int)(k * 32);
            while (it + 1 < items.size() && items[it + 1].cta_begin <= cta) ++it;
            c[k] = (int)it;
        }
        c[nc - 1] = (int)items.size() - 1;
    }
};

int launch_check(zf_ctx *ctx, const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(ctx, ZF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return ZF_OK;
}

#define TRY(x)                  \
    do {                        \
        int r_ = (x);           \
        if (r_ != ZF_OK) return r_; \
    } while (0)

// cuTensorMapEncodeTiled from the driver (looked up once; nullptr when the
// driver does not provide it, and the kernels then stage with thread loads).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            p = nullptr;
        }
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// A 2-D tensor map of an 8-bit plane as 4-byte elements (stride / 4 per
// row, ph rows) with box_w x box_h boxes, zero fill outside. false when the
// plane does not qualify (row pitch or base not 16-byte aligned) or the
// encoder refuses it.
bool encode_plane_map(void *out128, const uint8_t *plane, int stride, int ph, int box_w, int box_h) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc || !plane || (stride & 15) || (reinterpret_cast<uintptr_t>(plane) & 15) || ph <= 0) return false;
    alignas(64) CUtensorMap m;
    const cuuint64_t dims[2] = {(cuuint64_t)stride / 4, (cuuint64_t)ph};
    const cuuint64_t strides[1] = {(cuuint64_t)stride};
    const cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_h}, estr[2] = {1, 1};
    if (enc(&m, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, const_cast<uint8_t *>(plane), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    static_assert(sizeof(CUtensorMap) == 128, "tensor map size");
    std::memcpy(out128, &m, 128);
    return true;
}

// Ends an open stream capture on every exit path (the graph is discarded).
struct CaptureGuard {
    zf_ctx *ctx;
    bool active = false;
    ~CaptureGuard() {
        if (!active) return;
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(ctx->stream, &g);
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        ctx->capturing = false;
    }
};

// Ends the capture and launches it through the context's executable graph:
// an in-place update when the captured sequence has the same shape as the
// last one, a fresh instantiation otherwise.
// The graph's shape for the update decision: per node its kind and, for a
// kernel, its function and cluster dimensions (an update may change a
// kernel's arguments, grid and shared memory, but the executable graph is
// rebuilt when a function or a cluster shape differs).
int graph_signature(zf_ctx *ctx, cudaGraph_t g, std::vector<uint64_t> &sig) {
    size_t nn = 0;
    CU(cudaGraphGetNodes(g, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    CU(cudaGraphGetNodes(g, nodes.data(), &nn));
    sig.clear();
    for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType t;
        CU(cudaGraphNodeGetType(nd, &t));
        sig.push_back((uint64_t)t);
        if (t == cudaGraphNodeTypeKernel) {
            cudaKernelNodeParams kp;
            CU(cudaGraphKernelNodeGetParams(nd, &kp));
            sig.push_back((uint64_t)(uintptr_t)kp.func);
            cudaLaunchAttributeValue v;
            std::memset(&v, 0, sizeof(v));
            if (cudaGraphKernelNodeGetAttribute(nd, cudaLaunchAttributeClusterDimension, &v) != cudaSuccess) {
                cudaGetLastError();
                std::memset(&v, 0, sizeof(v));
            }
            sig.push_back((uint64_t)v.clusterDim.x << 32 | (uint64_t)v.clusterDim.y << 16 | v.clusterDim.z);
        }
    }
    return ZF_OK;
}

int launch_captured(zf_ctx *ctx, CaptureGuard &cg) {
    cudaGraph_t g = nullptr;
    cg.active = false;
    ctx->capturing = false;
    CU(cudaStreamEndCapture(ctx->stream, &g));
    std::vector<uint64_t> sig;
    const int rc = graph_signature(ctx, g, sig);
    if (rc != ZF_OK) {
        cudaGraphDestroy(g);
        return rc;
    }
    bool ok = false;
    if (ctx->gexec && sig == ctx->gsig) {
        cudaGraphExecUpdateResultInfo info;
        if (cudaGraphExecUpdate(ctx->gexec, g, &info) == cudaSuccess) {
            ok = true;
            ctx->graph_updates++;
        } else {
            cudaGetLastError();
            cudaGraphExecDestroy(ctx->gexec);
            ctx->gexec = nullptr;
        }
    }
    if (!ok) {
        if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
        ctx->gexec = nullptr;
        ctx->gsig = sig;
        const cudaError_t e = cudaGraphInstantiate(&ctx->gexec, g, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            ctx->gexec = nullptr;
            return fail(ctx, ZF_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
        }
        ctx->graph_instantiations++;
    }
    cudaGraphDestroy(g);
    CU(cudaGraphLaunch(ctx->gexec, ctx->stream));
    ctx->graph_launches++;
    return ZF_OK;
}

// Rust {:?} of a slice: "[a, b, c]".
template <typename T> std::string list_str(const T *v, int n) {
    std::string s = "[";
    for (int i = 0; i < n; ++i) {
        if (i) s += ", ";
        s += std::to_string(v[i]);
    }
    return s + "]";
}

// After a call: the CDEF search's mse rows for zf_cdef_search_rows, and the
// search trace lines (the reference's SVTAV1_CDEF_DBG and SVTAV1_LR_DBG
// dumps, cdef.rs:1296-1322, restoration.rs:768-842) read back from the
// arena. Debug and diff aids only: they synchronise and copy.
int search_records(zf_ctx *ctx, std::vector<Plan> &plans, const FrameDesc *back, const uint8_t *ob, const Run &run,
                   std::vector<std::vector<std::string>> &p_trace) {
    const int n = (int)plans.size();
    cudaStream_t st = ctx->stream;
    for (int i = 0; i < n; ++i) {
        Plan &p = plans[i];
        const FrameDesc &b = back[i];
        const bool cdef_searched = (run.stages & STG_CDEF_SEARCH) && !run.cdef_given && p.d.cdef.mode == 1;
        const int nc = p.d.cdef.ncand;
        const uint8_t *fbrow = ob + p.off_fbrow;
        std::vector<uint64_t> mse;
        if (cdef_searched) {
            mse.resize((size_t)p.nfb * 2 * nc);
            CU(cudaMemcpyAsync(mse.data(), p.d.mse, mse.size() * 8, cudaMemcpyDeviceToHost, st));
            CU(cudaStreamSynchronize(st));
        }
        if (run.rows && i == 0) {
            *run.rows->ncand = cdef_searched ? nc : 0;
            for (int fb = 0; fb < p.nfb; ++fb) {
                const bool has = cdef_searched && fbrow[fb];
                if (run.rows->has_row) run.rows->has_row[fb] = has ? 1 : 0;
                if (run.rows->mse && has) std::memcpy(run.rows->mse + (size_t)fb * 2 * nc, &mse[(size_t)fb * 2 * nc], 2 * nc * 8);
            }
        }
        if (!ctx->trace) continue;
        std::vector<std::string> &T = p_trace[i];
        if (cdef_searched) {
            std::vector<uint64_t> ysum(nc, 0), uvsum(nc, 0);
            int sbc = 0;
            for (int fb = 0; fb < p.nfb; ++fb) {
                if (!fbrow[fb]) continue;
                const uint64_t *r = &mse[(size_t)fb * 2 * nc];
                T.push_back("RS_CDEF_FB fbr=" + std::to_string(fb / p.d.nhfb) + " fbc=" + std::to_string(fb % p.d.nhfb) +
                            " Y=" + list_str(r, nc) + " UV=" + list_str(r + nc, nc));
                for (int g = 0; g < nc; ++g) {
                    ysum[g] += r[g];
                    uvsum[g] += r[nc + g];
                }
                ++sbc;
            }
            if (sbc) {
                T.push_back("RS_CDEF_SUM sb_count=" + std::to_string(sbc) + " fs=" + list_str(p.d.cdef.fs, nc) +
                            " Ysum=" + list_str(ysum.data(), nc) + " UVsum=" + list_str(uvsum.data(), nc));
                const int bits = b.cdef.bits, nb = 1 << bits;
                int l0[8], l1[8];
                for (int k = 0; k < nb; ++k) {
                    l0[k] = b.fin_lev[bits][k];
                    l1[k] = b.fin_lev[bits][8 + k];
                }
                T.push_back("RS_CDEF_PICK bits=" + std::to_string(bits) + " lev0=" + list_str(l0, nb) +
                            " lev1=" + list_str(l1, nb));
            }
        }
        const bool lr_searched = (run.stages & STG_LR_SEARCH) && !run.lr_given;
        for (int pl = 0; lr_searched && pl < 3; ++pl) {
            const LrPlane &L = p.d.lr[pl];
            if (!L.on) continue;
            const size_t nu = p.rects[pl].size();
            std::vector<LrUnit> U(nu);
            CU(cudaMemcpyAsync(U.data(), L.units, nu * sizeof(LrUnit), cudaMemcpyDeviceToHost, st));
            CU(cudaStreamSynchronize(st));
            for (size_t u = 0; u < nu; ++u) {
                const UnitRect &r = p.rects[pl][u];
                T.push_back("LRNONE plane=" + std::to_string(pl) + " unit=" + std::to_string(u) + " lim=[" +
                            std::to_string(r.h_start) + "," + std::to_string(r.h_end) + "," + std::to_string(r.v_start) +
                            "," + std::to_string(r.v_end) + "] sse=" + std::to_string(U[u].sse_none));
            }
            for (size_t u = 0; u < nu; ++u) {
                const LrUnit &x = U[u];
                T.push_back("LRWNSCORE plane=" + std::to_string(pl) + " unit=" + std::to_string(u) +
                            " score=" + std::to_string(x.score));
                if (x.score > 0) continue;
                const int64_t sse = L.refine ? x.sse_wn
                                    : p.d.bd == 8 ? (int64_t)(x.tw_blk + x.tw_rgt + x.tw_bot)
                                                  : (int64_t)x.tw_blk + (int64_t)(uint32_t)x.tw_rgt +
                                                        (int64_t)(uint32_t)x.tw_bot;
                T.push_back("LRWNSEG plane=" + std::to_string(pl) + " unit=" + std::to_string(u) + " sse_wn=" +
                            std::to_string(sse) + " v=" + list_str(x.vf, 7) + " h=" + list_str(x.hf, 7));
            }
        }
    }
    if (ctx->trace) {
        for (int i = 0; i < n; ++i) {
            if (n > 1) std::fprintf(ctx->trace, "ZF_FRAME index=%d w=%d h=%d\n", i, plans[i].d.tw, plans[i].d.th);
            for (const std::string &l : p_trace[i]) std::fprintf(ctx->trace, "%s\n", l.c_str());
        }
        std::fflush(ctx->trace);
    }
    return ZF_OK;
}

int run_batch(zf_ctx *ctx, const zf_frame *frames, int n, zf_decisions *outs, zf_stats *stats, const Run &run) {
    if (!ctx) return ZF_ERR_ARG;
    if (n <= 0 || !frames) return fail(ctx, ZF_ERR_ARG, "empty batch");
    CU(cudaSetDevice(ctx->device));
    TRY(check_cancel(ctx));
    std::vector<Plan> plans((size_t)n);
    std::vector<std::vector<std::string>> p_trace((size_t)n);  // trace lines per frame
    size_t cursor = 0, ucur = 0, rcur = 0, ocur = 0;
    for (int i = 0; i < n; ++i) {
        TRY(validate_frame(ctx, &frames[i]));
        plan_frame(plans[i], &frames[i], cursor, ucur, rcur, ocur);
        plans[i].out = outs ? &outs[i] : nullptr;
        plans[i].d.wait_limit = ctx->wait_limit;
    }
    // Work lists (host-known shapes).
    // statistics: 5-tap 8-bit, 5-tap 10-bit (one kernel instantiation each), 7-tap
    WorkList wl_db, wl_cs, wl_ca, wl_st5, wl_st7, wl_unit, wl_apply, wl_trial, wl_tiles, wl_st5h, wl_stc;
    int trial_tiles = 1;  // k_lr_trial: the most tiles one CTA of a unit's cluster stages
    std::vector<int> cdef_small, cdef_large;  // joint search: one CTA / cluster per bit count
    std::vector<int> cdef_joint[kJointGroups];  // register-row joint search, by (candidates, rows per thread)
    for (int i = 0; i < n; ++i) {
        Plan &p = plans[i];
        for (int pl = 0; pl < p.nplanes; ++pl) {
            const int pw = pl ? p.d.w / 2 : p.d.w, ph = pl ? p.d.h / 2 : p.d.h;
            wl_db.add(i, pl, 0, 0, ((pw + 63) / 64) * ((ph + 63) / 64));
        }
        if (p.d.cdef.mode == 1 && !run.cdef_given) {
            wl_cs.add(i, 0, 0, 0, p.nfb);
            const int rpt = zf::joint_rows_per_thread(p.nfb, p.d.cdef.ncand);
            const bool small = p.nfb <= kFinish1MaxFb &&
                               zf::finish1_smem(p.nfb, p.d.cdef.ncand, kFinish1SmemCap) > 0;
            if (rpt) cdef_joint[joint_group(p.d.cdef.ncand, rpt)].push_back(i);
            else (small ? cdef_small : cdef_large).push_back(i);
        }
        wl_ca.add(i, 0, 0, 0, p.nfb);
        for (int pl = 0; pl < 3; ++pl) {
            const LrPlane &L = p.d.lr[pl];
            if (!L.on) continue;
            for (size_t u = 0; u < p.rects[pl].size(); ++u) {
                const UnitRect &r = p.rects[pl][u];
                const int uh = r.v_end - r.v_start;
                // one item per unit; the CTA offset selects the row block
                const int half = L.win / 2, srows = zf::stat_rows_host(L.win);
                if (L.win == 5 && p.d.bd == 8 && ctx->stats_tc) {
                    // tensor-core statistics: one CTA per band of output rows
                    const int tr = zf::lr_stats_tc_rows();
                    wl_stc.add(i, pl, (int)u, 0, (uh + tr - 1) / tr);
                } else {
                    (L.win == 5 ? (p.d.bd == 8 ? wl_st5 : wl_st5h) : wl_st7)
                        .add(i, pl, (int)u, 0, (uh + 2 * half + srows - 1) / srows);
                }
                wl_unit.add(i, pl, (int)u, 0, 1);
                if (L.refine) {
                    // one cluster per unit: the hill-climb is sequential, its trials are not
                    wl_trial.add(i, pl, (int)u, 0, zf::kTrialClusterHost);
                    trial_tiles = std::max(trial_tiles, zf::lr_trial_tiles_per_cta(r.h_end - r.h_start, uh));
                } else {
                    const int tl = ctx->trial_tile, uw = r.h_end - r.h_start;
                    wl_tiles.add(i, pl, (int)u, 0, ((uw + tl - 1) / tl) * ((uh + tl - 1) / tl));
                }
            }
        }
        // Wiener apply items: every (stripe, 64-px tile) of every plane's
        // aligned canvas, plus the canvas rows below the true plane (stripe
        // index nstripes); the kernel filters Wiener units and copies the rest
        for (int pl = 0; pl < p.nplanes && (run.stages & STG_LR_APPLY); ++pl) {
            const LrPlane &L = p.d.lr[pl];
            const int ss = pl ? 1 : 0, full = 64 >> ss, off = 8 >> ss;
            const int nstripes = (L.ph + off + full - 1) / full;
            const int ngroups = ((L.stride + 63) / 64 + ctx->apply_group - 1) / ctx->apply_group;
            const int canvas_h = pl ? p.d.h / 2 : p.d.h;
            // one item per stripe (CTA offset = group of ctx->apply_group
            // 64-px column tiles); a = the stripe's row of the row-major
            // hunits x vunits unit grid (-1: copy only), the kernel finds the
            // column along that row
            const std::vector<UnitRect> &R = p.rects[pl];
            const int hu = p.hunits[pl], vu = p.vunits[pl];
            for (int s = 0, r = 0; s < nstripes; ++s) {
                const int ys = std::max(0, s * full - off);
                while (r < vu && ys >= R[(size_t)r * hu].v_end) ++r;
                const bool row_ok = r < vu && ys >= R[(size_t)r * hu].v_start;
                wl_apply.add(i, pl, (L.on && row_ok) ? r : -1, s, ngroups);
            }
            if (canvas_h > L.ph) wl_apply.add(i, pl, -1, nstripes, ngroups);
        }
    }
    // finish frame ids: the joint groups in order, then the small frames,
    // then the large ones
    std::vector<int> cdef_frames;
    for (const std::vector<int> &g : cdef_joint) cdef_frames.insert(cdef_frames.end(), g.begin(), g.end());
    const int n_joint = (int)cdef_frames.size();
    cdef_frames.insert(cdef_frames.end(), cdef_small.begin(), cdef_small.end());
    cdef_frames.insert(cdef_frames.end(), cdef_large.begin(), cdef_large.end());
    const int n_small = (int)cdef_small.size();
    // Arena: per-frame buffers | unit accumulators | metadata image |
    // deblock search scratch | outputs.
    const size_t o_units = align_up(cursor, 256);
    const size_t o_meta = align_up(o_units + ucur, 256);
    size_t mcur = 0;
    auto mtake = [&mcur](size_t b) {
        mcur = align_up(mcur, 256);
        const size_t o = mcur;
        mcur += b + 16;
        return o;
    };
    const size_t desc_bytes = (size_t)n * sizeof(FrameDesc);
    const size_t m_desc = mtake(desc_bytes);
    constexpr int kLists = 11;
    const WorkList *lists[kLists] = {&wl_db,   &wl_cs,    &wl_ca,    &wl_st5,   &wl_st7,  &wl_unit,
                                     &wl_apply, &wl_trial, &wl_tiles, &wl_st5h, &wl_stc};
    size_t m_list[kLists];
    for (int k = 0; k < kLists; ++k) m_list[k] = mtake(lists[k]->bytes());
    const size_t m_cf = mtake(cdef_frames.size() * 4);
    const size_t m_rects = mtake(rcur);
    const size_t m_tm = mtake((size_t)n * 3 * 256);  // per frame and plane: post-CDEF and source tensor maps
    const size_t meta_bytes = align_up(mcur, 256);
    // deblock search scratch: up to 3 slots per frame (8 for a table of
    // all 64 levels), each of at most the largest frame's luma tiles
    // (items, then their coarse index), kDbLevels levels and SSEs per slot
    size_t max_tiles = 1;
    for (const Plan &p : plans) max_tiles = std::max(max_tiles, (size_t)((p.d.w + 63) / 64) * ((p.d.h + 63) / 64));
    size_t c2 = o_meta + meta_bytes;
    const size_t db_slots = std::max<size_t>((size_t)n * 3, (64 + zf::kDbLevels - 1) / zf::kDbLevels);
    const size_t o_dbs_items = c2;
    c2 += align_up(db_slots * sizeof(WorkItem) + (db_slots * max_tiles / 32 + 2) * sizeof(int) + 16, 256);
    const size_t o_dbs_lv = c2;
    c2 += align_up(db_slots * zf::kDbLevels * 4, 256);
    const size_t o_dbs_sse = c2;
    c2 += align_up(db_slots * zf::kDbLevels * 8, 256);
    const size_t o_out = c2;
    const size_t out_bytes = align_up(ocur, 256);
    c2 += out_bytes;
    TRY(ensure_arena(ctx, c2));
    const size_t hdesc = align_up(desc_bytes, 256);
    TRY(ensure_host(ctx, ctx->h_meta, ctx->h_meta_cap, meta_bytes + hdesc));
    TRY(ensure_host(ctx, ctx->h_out, ctx->h_out_cap, hdesc + out_bytes));
    uint8_t *base = ctx->arena;
    cudaStream_t st = ctx->stream;
    for (auto &p : plans) bind_pointers(p, base, base + o_units, base + o_meta + m_rects, base + o_out);
    FrameDesc *d_desc = (FrameDesc *)(base + o_meta + m_desc);
    const size_t o_db = o_meta + m_list[0], o_cs = o_meta + m_list[1], o_ca = o_meta + m_list[2],
                 o_st5 = o_meta + m_list[3], o_st7 = o_meta + m_list[4], o_unit = o_meta + m_list[5],
                 o_apply = o_meta + m_list[6], o_trial = o_meta + m_list[7], o_tiles = o_meta + m_list[8],
                 o_st5h = o_meta + m_list[9], o_stc = o_meta + m_list[10], o_cf = o_meta + m_cf;
    // outputs start zeroed (statistics counters, fb_idx of skipped searches)
    CU(cudaMemsetAsync(base + o_out, 0, out_bytes, st));

    // ---- inputs
    // job room for every plane copy of the call: in (rec, src, pre-CDEF per
    // plane, geometry) then out (the filtered planes)
    const size_t in_jobs = (size_t)n * 10;
    TRY(ensure_jobs(ctx, in_jobs + (size_t)n * 3));
    HostCopies hin, hout;
    auto plane_in = [&](void *dst, const void *src, size_t nb, bool dev) -> int {
        if (dev || !hin.add(dst, src, nb, true)) return copy_in(ctx, dst, src, nb, dev);
        return ZF_OK;
    };
    for (int i = 0; i < n; ++i) {
        Plan &p = plans[i];
        const zf_frame *f = p.in;
        const bool dev = f->planes_on_device != 0;
        const int set = run.rec_in;
        // Whole stage on device planes: the deblock passes read the caller's
        // recon, the Wiener apply writes every pixel of it at the end (after
        // the last read), and source and geometry are read in place.
        p.zero_copy = dev && set == SET_A && run.rec_out == SET_C && !run.pre_cdef_in &&
                      (run.stages & STG_DB_APPLY) && (run.stages & STG_LR_APPLY);
        if (p.zero_copy) {
            for (int pl = 0; pl < p.nplanes; ++pl) {
                p.d.IN[pl] = static_cast<uint8_t *>(f->rec[pl]);
                p.d.C[pl] = static_cast<uint8_t *>(f->rec[pl]);
                p.d.S[pl] = static_cast<const uint8_t *>(f->src[pl]);
            }
            p.d.mi = f->mi;
        } else {
            for (int pl = 0; pl < p.nplanes; ++pl) {
                TRY(plane_in(base + p.off_set[set][pl], f->rec[pl], p.pbytes[pl], dev));
                TRY(plane_in(base + p.off_src[pl], f->src[pl], p.pbytes[pl], dev));
                if (run.pre_cdef_in) TRY(plane_in(base + p.off_set[SET_B][pl], run.pre_cdef[pl], p.pbytes[pl], dev));
            }
            TRY(plane_in(base + p.off_mi, f->mi, (size_t)p.d.mi_cols * p.d.mi_rows * 4, dev));
        }
        for (int pl = 0; pl < 3; ++pl)
            if (!p.rects[pl].empty())
                std::memcpy(ctx->h_meta + m_rects + p.off_rects[pl], p.rects[pl].data(),
                            p.rects[pl].size() * sizeof(UnitRect));
        // The tiled Wiener trial (units without refinement) writes its
        // filtered pixels into C when this call applies the search's
        // decisions; the apply then recomputes only the rows next to
        // interior stripe boundaries of Wiener units.
        const bool trial_out = (run.stages & STG_LR_SEARCH) && !run.lr_given && (run.stages & STG_LR_APPLY);
        // The CDEF apply takes the luma directions from the search when the
        // same call searches this frame (both read the same B).
        p.d.cdir_ok = (run.stages & STG_CDEF_SEARCH) && (run.stages & STG_CDEF_APPLY) && !run.cdef_given &&
                      p.d.cdef.mode == 1;
        for (int pl = 0; pl < 3; ++pl) {
            LrPlane &L = p.d.lr[pl];
            L.trial_out = trial_out && L.on && !L.refine ? 1 : 0;
        }
        // decisions the caller provides
        const zf_decisions *dec = p.out;
        if (run.lf_given) std::memcpy(p.d.lf, dec->lf, 4);
        if (run.cdef_given) {
            CdefParams &cp = p.d.cdef;
            cp.mode = 2;
            cp.damping = dec->cdef_damping;
            cp.bits = dec->cdef_bits;
            std::memcpy(cp.y_str, dec->cdef_y, 8);
            std::memcpy(cp.uv_str, dec->cdef_uv, 8);
            if (cp.bits) {
                if (!dec->cdef_fb_idx) return fail(ctx, ZF_ERR_ARG, "cdef_bits > 0 needs cdef_fb_idx");
                CU(cudaMemcpyAsync(base + o_out + p.off_fbidx, dec->cdef_fb_idx, p.nfb, cudaMemcpyHostToDevice, st));
            }
        }
        if (run.lr_given) {
            for (int pl = 0; pl < 3; ++pl) {
                LrPlane &L = p.d.lr[pl];
                if (pl >= p.nplanes) {
                    L.on = 0;
                    continue;
                }
                L.on = dec->lr[pl].frame_rtype != ZF_RESTORE_NONE;
                L.frame_rtype = dec->lr[pl].frame_rtype;
                if (!L.on) continue;
                if (dec->lr[pl].hunits != p.hunits[pl] || dec->lr[pl].vunits != p.vunits[pl] || !dec->lr_units[pl])
                    return fail(ctx, ZF_ERR_ARG, "restoration unit grid does not match the frame");
                const size_t nu = p.rects[pl].size();
                std::vector<LrUnit> hu(nu);
                std::memset(hu.data(), 0, nu * sizeof(LrUnit));
                for (size_t u = 0; u < nu; ++u) {
                    hu[u].rtype = dec->lr_units[pl][u].rtype;
                    std::memcpy(hu[u].vf, dec->lr_units[pl][u].vfilter, 16);
                    std::memcpy(hu[u].hf, dec->lr_units[pl][u].hfilter, 16);
                }
                // units storage exists only for searched planes; reuse the
                // rects offset region sizing by re-planning is avoided by
                // requiring the plane to be LR-enabled at plan time.
                if (!p.d.lr[pl].units) return fail(ctx, ZF_ERR_UNSUPPORTED, "restoration disabled for this frame");
                CU(cudaMemcpyAsync(p.d.lr[pl].units, hu.data(), nu * sizeof(LrUnit), cudaMemcpyHostToDevice, st));
            }
        }
    }
    TRY(flush_copies(ctx, hin, 0));

    // ---- deblock level pick (presets <= 5: device SSE trials + host
    // hill-climb), or the caller's table of trial levels
    // Trials: one launch evaluates every slot (frame, plane, up to
    // kDbLevels levels) over all tiles of its plane.
    struct TrialSlot {
        int frame, plane;
        std::vector<int> levels;
        std::vector<int64_t> sse;
    };
    auto run_trials = [&](std::vector<TrialSlot> &ts) -> int {
        WorkList wl;
        std::vector<int> lv(ts.size() * zf::kDbLevels, -1);
        uint64_t nbytes = 0;  // each slot's plane and source plane, read once
        for (size_t k = 0; k < ts.size(); ++k) {
            const Plan &p = plans[ts[k].frame];
            for (size_t j = 0; j < ts[k].levels.size(); ++j) lv[k * zf::kDbLevels + j] = ts[k].levels[j];
            const int pw = ts[k].plane ? p.d.w / 2 : p.d.w, ph = ts[k].plane ? p.d.h / 2 : p.d.h;
            wl.add(ts[k].frame, ts[k].plane, (int)k, 0, ((pw + 63) / 64) * ((ph + 63) / 64));
            nbytes += 2ull * pw * ph * p.px;
        }
        if (ts.size() > db_slots) return fail(ctx, ZF_ERR_UNSUPPORTED, "too many search slots");
        std::vector<uint8_t> wl_img(wl.bytes());
        wl.write(wl_img.data());
        CU(cudaMemcpyAsync(base + o_dbs_items, wl_img.data(), wl_img.size(), cudaMemcpyHostToDevice, st));
        CU(cudaMemcpyAsync(base + o_dbs_lv, lv.data(), lv.size() * 4, cudaMemcpyHostToDevice, st));
        CU(cudaMemsetAsync(base + o_dbs_sse, 0, lv.size() * 8, st));
        { LaunchScope ls_(ctx, "k_deblock_sse", nbytes);
        zf::k_deblock_sse<<<wl.ctas, 256, 0, st>>>(d_desc, (const WorkItem *)(base + o_dbs_items),
                                                   (int)wl.items.size(), (const int *)(base + o_dbs_lv),
                                                   zf::kDbLevels, (unsigned long long *)(base + o_dbs_sse)); }
        TRY(launch_check(ctx, "k_deblock_sse"));
        std::vector<unsigned long long> sse(lv.size());
        CU(cudaMemcpyAsync(sse.data(), base + o_dbs_sse, sse.size() * 8, cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        TRY(check_cancel(ctx));
        for (size_t k = 0; k < ts.size(); ++k) {
            ts[k].sse.resize(ts[k].levels.size());
            for (size_t j = 0; j < ts[k].levels.size(); ++j)
                ts[k].sse[j] = (int64_t)sse[k * zf::kDbLevels + j];
        }
        return ZF_OK;
    };
    if ((run.stages & STG_DB_PICK) || run.table) {
        // the trial kernels read the descriptors (spare slot after the
        // metadata image; the final image goes up after the search)
        FrameDesc *hd = (FrameDesc *)(ctx->h_meta + meta_bytes);
        for (int i = 0; i < n; ++i) hd[i] = plans[i].d;
        CU(cudaMemcpyAsync(d_desc, hd, desc_bytes, cudaMemcpyHostToDevice, st));
    }
    if (run.table) {
        // zf_deblock_sse_table: the caller's levels of one plane, kDbLevels
        // per slot, one launch
        std::vector<TrialSlot> ts;
        for (int k = 0; k < run.table->n; k += zf::kDbLevels) {
            TrialSlot t{0, run.table->plane, {}, {}};
            for (int j = k; j < std::min(run.table->n, k + zf::kDbLevels); ++j) t.levels.push_back(run.table->levels[j]);
            ts.push_back(t);
        }
        TRY(run_trials(ts));
        for (size_t k = 0; k < ts.size(); ++k)
            for (size_t j = 0; j < ts[k].levels.size(); ++j) run.table->sse[k * zf::kDbLevels + j] = ts[k].sse[j];
    }
    if (run.stages & STG_DB_PICK) {
        struct Slot {
            int frame, plane;
            HillClimb hc;
            int launches = 0;
        };
        std::vector<Slot> slots;
        for (int i = 0; i < n; ++i) {
            Plan &p = plans[i];
            if (p.db_search) {
                Slot s{i, 0, HillClimb(), 0};
                s.hc.conv_th = p.in->preset <= 3 ? 0 : 1;
                slots.push_back(s);
            } else {
                key_frame_levels(p.in->qindex, p.in->bit_depth, p.d.lf);
            }
        }
        // trace lines of the climbs (try_filter_plane / search_filter_level)
        auto trace_climb = [&](const Slot &s) {
            if (!ctx->trace) return;
            const Plan &p = plans[s.frame];
            const int pw = s.plane ? p.d.w / 2 : p.d.w, ph = s.plane ? p.d.h / 2 : p.d.h;
            std::vector<int> order;
            s.hc.trial_order(order);
            char line[160];
            for (int l : order) {
                std::snprintf(line, sizeof(line), "DLF_TRY plane=%d lvl0=%d lvl1=%d w=%d h=%d sse=%lld", s.plane, l, l,
                              pw, ph, (long long)s.hc.err[l]);
                p_trace[s.frame].push_back(line);
            }
            std::snprintf(line, sizeof(line), "DLF_PICK plane=%d dir=%d level=%d sse=%lld", s.plane, s.plane ? 0 : 2,
                          s.hc.result, (long long)s.hc.err[s.hc.result]);
            p_trace[s.frame].push_back(line);
        };
        // A frame's chroma climbs (searched only when its luma level is not
        // 0) start as soon as the luma climb has left level 0, and share
        // launches with it from then on: one round trip per step of the
        // longer climb instead of the two climbs' steps in sequence. A luma
        // climb that ends at 0 after all discards them.
        const size_t nluma = slots.size();
        std::vector<int> chroma_at(n, -1);  // index of a frame's U slot (V follows)
        auto maybe_spawn = [&](size_t k) {
            const int fi = slots[k].frame;
            if (plans[fi].nplanes != 3 || chroma_at[fi] >= 0) return;
            if (!(slots[k].hc.done ? slots[k].hc.result != 0 : slots[k].hc.at_mid > 0)) return;
            const int conv = slots[k].hc.conv_th;
            chroma_at[fi] = (int)slots.size();
            for (int pl = 1; pl <= 2; ++pl) {
                Slot c{fi, pl, HillClimb(), 0};
                c.hc.conv_th = conv;
                slots.push_back(c);
            }
        };
        bool finished = false;
        for (int guard = 0; guard < 256 && !finished; ++guard) {
            std::vector<TrialSlot> ts;
            std::vector<int> owner;
            for (size_t k = 0; k < slots.size(); ++k) {  // slots may grow: chroma climbs appended
                if (slots[k].hc.done) continue;
                int need[2];
                const int m = slots[k].hc.needs(need);
                if (k < nluma) maybe_spawn(k);
                if (m == 0) continue;
                Slot &s = slots[k];
                // four levels in each of a climb's first two launches (most
                // climbs end within them), ctx->db_levels in later ones. A
                // refining climb (conv_th != 1) on a plane of >= 512 tiles
                // takes at most two levels a launch: it converges through
                // half and quarter steps, so deeper speculation is wasted as
                // often as not, and there a level costs about as much as the
                // host round trip it may save (a 4096x3072 10-bit preset-2
                // frame: 3.65 ms at two levels a launch, 4.0 ms at eight;
                // a 4K climb that only continues upwards, conv_th 1, gains
                // from eight: 1.22 against 1.45 ms).
                const Plan &sp = plans[s.frame];
                const int spw = s.plane ? sp.d.w / 2 : sp.d.w, sph = s.plane ? sp.d.h / 2 : sp.d.h;
                const bool big = ((spw + 63) / 64) * ((sph + 63) / 64) >= 512;
                int cap = s.launches < 2 ? std::min(4, ctx->db_levels) : ctx->db_levels;
                if (s.hc.conv_th != 1 && big) cap = std::min(cap, 2);
                TrialSlot t{s.frame, s.plane, {}, {}};
                speculate(s.hc, need, m, cap, t.levels);
                s.launches++;
                ts.push_back(t);
                owner.push_back((int)k);
            }
            if (owner.empty()) {
                for (auto &s : slots)
                    if (!s.hc.done) return fail(ctx, ZF_ERR_UNSUPPORTED, "deblock search stalled");
                finished = true;
                break;
            }
            TRY(run_trials(ts));
            for (size_t k = 0; k < owner.size(); ++k) {
                Slot &s = slots[owner[k]];
                for (size_t j = 0; j < ts[k].levels.size(); ++j) {
                    const int l = ts[k].levels[j];
                    s.hc.err[l] = ts[k].sse[j];
                    s.hc.have[l] = true;
                }
            }
        }
        if (!finished) return fail(ctx, ZF_ERR_UNSUPPORTED, "deblock search did not converge");
        for (size_t k = 0; k < nluma; ++k) {
            const Slot &s = slots[k];
            Plan &p = plans[s.frame];
            p.d.lf[0] = p.d.lf[1] = (uint8_t)s.hc.result;
            p.d.lf[2] = p.d.lf[3] = 0;
            trace_climb(s);
            if (s.hc.result != 0 && chroma_at[s.frame] >= 0)
                for (int pl = 1; pl <= 2; ++pl) {
                    const Slot &c = slots[chroma_at[s.frame] + pl - 1];
                    p.d.lf[1 + pl] = (uint8_t)c.hc.result;
                    trace_climb(c);
                }
        }
    }

    // ---- graph mode: everything from here to the decision readback is
    // captured and launched as one graph
    CaptureGuard cg{ctx};
    const bool use_graph = ctx->graphs && !ctx->profiling;
    if (use_graph) {
        CU(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        cg.active = true;
        ctx->capturing = true;
    }

    // ---- metadata image (descriptors, work lists, CDEF frames, unit
    // rectangles) to the device in one copy
    {
        uint8_t *hm = ctx->h_meta;
        FrameDesc *hd = (FrameDesc *)(hm + m_desc);
        // tensor maps of the 8-bit planes the 5-tap statistics read
        for (int i = 0; i < n; ++i)
            for (int pl = 0; pl < 3; ++pl) {
                LrPlane &L = plans[i].d.lr[pl];
                L.tm_a = L.tm_s = nullptr;
                if (!ctx->tma || !L.on || L.win != 5 || plans[i].d.bd != 8) continue;
                const size_t o = m_tm + ((size_t)i * 3 + pl) * 256;
                if (encode_plane_map(hm + o, plans[i].d.A[pl], L.stride, L.ph, zf::kTmaDBoxW, zf::kTmaDBoxH) &&
                    encode_plane_map(hm + o + 128, plans[i].d.S[pl], L.stride, L.ph, zf::kTmaXBoxW, zf::kTmaXBoxH)) {
                    L.tm_a = base + o_meta + o;
                    L.tm_s = base + o_meta + o + 128;
                }
            }
        for (int i = 0; i < n; ++i) hd[i] = plans[i].d;
        for (int k = 0; k < kLists; ++k)
            if (!lists[k]->items.empty()) lists[k]->write(hm + m_list[k]);
        if (!cdef_frames.empty()) std::memcpy(hm + m_cf, cdef_frames.data(), cdef_frames.size() * 4);
        CU(cudaMemcpyAsync(base + o_meta, hm, meta_bytes, cudaMemcpyHostToDevice, st));
    }

    // ---- deblock apply: A -> B
    if (run.stages & STG_DB_APPLY) {
        { LaunchScope ls_(ctx, "k_deblock_apply");
        zf::k_deblock_apply<<<wl_db.ctas, 256, 0, st>>>(d_desc, (const WorkItem *)(base + o_db),
                                                        (int)wl_db.items.size()); }
        TRY(launch_check(ctx, "k_deblock_apply"));
        TRY(check_cancel(ctx));
    }
    // ---- CDEF search + finish on B
    if ((run.stages & STG_CDEF_SEARCH) && !cdef_frames.empty()) {
        int fp = 1, ns = 1;
        for (int fi : cdef_frames) {
            const CdefParams &c = plans[fi].d.cdef;
            fp = std::max(fp, c.first_pass_num);
            ns = std::max(ns, c.ncand / c.first_pass_num);
        }
        { LaunchScope ls_(ctx, "k_cdef_search");
        CU(zf::launch_cdef_search(fp, ns, wl_cs.ctas, st, d_desc, (const WorkItem *)(base + o_cs),
                                  (int)wl_cs.items.size())); }
        TRY(launch_check(ctx, "k_cdef_search"));
        // Joint search: frames with 4 or 6 candidates and up to 2048 filter
        // blocks run k_cdef_joint, one CTA per (frame, bit count) and one
        // launch per (candidates, rows per thread) group; other frames of up
        // to kFinish1MaxFb filter blocks whose rows fit one CTA's shared
        // memory run k_cdef_finish1; larger frames a cluster per (frame, bit
        // count), which wins once the per-step row sums outweigh the cluster
        // barrier. (cdef_frames lists the joint groups, then the small
        // frames, then the large ones)
        int smem1 = 0;
        for (int k = n_joint; k < n_joint + n_small; ++k) {
            const Plan &pf = plans[cdef_frames[k]];
            smem1 = std::max(smem1, zf::finish1_smem(pf.nfb, pf.d.cdef.ncand, kFinish1SmemCap));
        }
        const std::vector<int> small_f(cdef_frames.begin() + n_joint, cdef_frames.begin() + n_joint + n_small),
            large_f(cdef_frames.begin() + n_joint + n_small, cdef_frames.end());
        { LaunchScope ls_(ctx, "k_cdef_finish");
        for (int g = 0, off = 0; g < kJointGroups; off += (int)cdef_joint[g].size(), ++g) {
            if (cdef_joint[g].empty()) continue;
            CU(zf::launch_cdef_joint(joint_group_ncand(g), joint_group_rpt(g), (int)cdef_joint[g].size(), st,
                                     d_desc, (const int *)(base + o_cf) + off));
        }
        if (!small_f.empty()) {
            zf::k_cdef_finish1<<<(int)small_f.size() * zf::kFinLevels, zf::kFin1ThreadsHost, smem1, st>>>(
                d_desc, (const int *)(base + o_cf) + n_joint);
        }
        if (!large_f.empty()) {
            // dynamic shared memory: the double-buffered pair partials (each
            // rank's inbox for the pairs it owns) and the compacted rows
            // of the largest frame, capped (frames whose rows do not fit use
            // global scratch). 16-CTA clusters where the device allows them.
            auto need = [&](int cl) {
                size_t want = 0, pairs = 0;
                for (int fi : large_f) {
                    const size_t nc = (size_t)plans[fi].d.cdef.ncand, np = nc * nc;
                    const size_t pb = zf::fin_pair_bytes((int)np, cl);
                    pairs = std::max(pairs, pb);
                    // rows (+ up to 12 padding rows per column: the padded
                    // strides) and ids
                    const size_t rows = ((size_t)plans[fi].nfb + cl - 1) / cl;
                    want = std::max(want, pb + (rows + 12) * 2 * nc * 4 + rows * 4);
                }
                return std::max(pairs, std::min<size_t>(want, kFinishSmemCap));
            };
            int cl = zf::kFinClusterMaxHost;
            size_t smem = need(cl);
            if (zf::finish_cluster_size(smem) != cl) {
                cl = zf::kFinClusterHost;
                smem = need(cl);
            }
            CU(zf::launch_cdef_finish((int)large_f.size() * zf::kFinLevels, cl, smem, st, d_desc,
                                      (const int *)(base + o_cf) + n_joint + small_f.size(), (int)smem));
        } }
        TRY(launch_check(ctx, "k_cdef_finish"));
        TRY(check_cancel(ctx));
    }
    // ---- CDEF apply: B -> A
    if (run.stages & STG_CDEF_APPLY) {
        { LaunchScope ls_(ctx, "k_cdef_apply");
        zf::k_cdef_apply<<<wl_ca.ctas, 256, 0, st>>>(d_desc, (const WorkItem *)(base + o_ca), (int)wl_ca.items.size()); }
        TRY(launch_check(ctx, "k_cdef_apply"));
        TRY(check_cancel(ctx));
    }
    // ---- Wiener search on A
    if ((run.stages & STG_LR_SEARCH) && !run.lr_given) {
        if (ucur) CU(cudaMemsetAsync(base + o_units, 0, ucur, st));
        if (wl_st5.ctas) {
            LaunchScope ls5_(ctx, "k_lr_stats5");
            CU(zf::launch_lr_stats(5, 8, wl_st5.ctas, st, d_desc, (const WorkItem *)(base + o_st5),
                                   (int)wl_st5.items.size()));
        }
        if (wl_stc.ctas) {
            LaunchScope lt_(ctx, "k_lr_stats_tc");
            zf::k_lr_stats_tc<<<wl_stc.ctas, 128, zf::lr_stats_tc_smem(), st>>>(
                d_desc, (const WorkItem *)(base + o_stc), (int)wl_stc.items.size());
            TRY(launch_check(ctx, "k_lr_stats_tc"));
        }
        if (wl_st5h.ctas) {
            LaunchScope ls5h_(ctx, "k_lr_stats5");
            CU(zf::launch_lr_stats(5, 10, wl_st5h.ctas, st, d_desc, (const WorkItem *)(base + o_st5h),
                                   (int)wl_st5h.items.size()));
        }
        if (wl_st7.ctas) {
            LaunchScope ls7_(ctx, "k_lr_stats7");
            CU(zf::launch_lr_stats(7, 0, wl_st7.ctas, st, d_desc, (const WorkItem *)(base + o_st7),
                                   (int)wl_st7.items.size()));
        }
        if (wl_unit.ctas) {
            { LaunchScope ls_(ctx, "k_lr_solve");
            zf::k_lr_solve<<<wl_unit.ctas, 128, 0, st>>>(d_desc, (const WorkItem *)(base + o_unit),
                                                        (int)wl_unit.items.size()); }
            TRY(launch_check(ctx, "k_lr_solve"));
            if (wl_trial.ctas) {
                { LaunchScope ls_(ctx, "k_lr_trial");
                if (trial_tiles > zf::kTrialMaxTilesHost)
                    return fail(ctx, ZF_ERR_UNSUPPORTED, "a restoration unit exceeds the refinement trial's tiles");
                zf::k_lr_trial<<<wl_trial.ctas, 256, zf::lr_trial_smem(trial_tiles), st>>>(
                    d_desc, (const WorkItem *)(base + o_trial), (int)wl_trial.items.size(), trial_tiles); }
                TRY(launch_check(ctx, "k_lr_trial"));
            }
            if (wl_tiles.ctas) {
                { LaunchScope ls_(ctx, "k_lr_trial_tiles");
                CU(zf::launch_lr_trial_tiles(ctx->trial_tile, wl_tiles.ctas, st, d_desc,
                                             (const WorkItem *)(base + o_tiles), (int)wl_tiles.items.size())); }
                TRY(launch_check(ctx, "k_lr_trial_tiles"));
            }
        }
        { LaunchScope ls_(ctx, "k_lr_finish");
        // dynamic shared memory: 32 B per unit, plus the (unit, reference)
        // pair table of planes with at most 200 units
        size_t smem = 32;
        for (auto &p : plans)
            for (int pl = 0; pl < 3; ++pl) {
                const size_t nu = (size_t)p.hunits[pl] * p.vunits[pl], np = nu * (nu + 1) / 2;
                smem = std::max(smem, nu * 32 + (np <= (size_t)zf::kLrPairMaxHost ? np * 4 : 0));
            }
        if (smem > (size_t)kLrFinishSmemCap) return fail(ctx, ZF_ERR_UNSUPPORTED, "restoration unit table too large");
        zf::k_lr_finish<<<n * 3, zf::kLrFinThreadsHost, smem, st>>>(d_desc, n); }
        TRY(launch_check(ctx, "k_lr_finish"));
        TRY(check_cancel(ctx));
    }
    // ---- Wiener apply: A (+ B boundary lines) -> C
    if (run.stages & STG_LR_APPLY) {
        if (wl_apply.ctas) {
            { LaunchScope ls_(ctx, "k_lr_apply");
            zf::k_lr_apply<<<wl_apply.ctas, 256, 0, st>>>(d_desc, (const WorkItem *)(base + o_apply),
                                                         (int)wl_apply.items.size(), ctx->apply_group); }
            TRY(launch_check(ctx, "k_lr_apply"));
        }
    }

    // ---- outputs: the descriptors and the output region (fb_idx, fb_row,
    // counters, unit records) in two copies, then the planes to the caller
    CU(cudaMemcpyAsync(ctx->h_out, d_desc, desc_bytes, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(ctx->h_out + hdesc, base + o_out, out_bytes, cudaMemcpyDeviceToHost, st));
    if (use_graph) TRY(launch_captured(ctx, cg));
    for (int i = 0; i < n; ++i) {
        Plan &p = plans[i];
        const zf_frame *f = p.in;
        const bool dev = f->planes_on_device != 0;
        if ((run.stages & (STG_DB_APPLY | STG_CDEF_APPLY | STG_LR_APPLY)) && !p.zero_copy)
            for (int pl = 0; pl < p.nplanes; ++pl) {
                void *dst = f->rec[pl];
                const void *src = base + p.off_set[run.rec_out][pl];
                if (dev || !hout.add(dst, src, p.pbytes[pl], false)) TRY(copy_out(ctx, dst, src, p.pbytes[pl], dev));
            }
    }
    TRY(flush_copies(ctx, hout, in_jobs));
    CU(cudaStreamSynchronize(st));
    TRY(launch_check(ctx, "stream"));
    if (use_graph) TRY(check_cancel(ctx));
    collect_profile(ctx);
    const FrameDesc *back = (const FrameDesc *)ctx->h_out;
    const uint8_t *ob = ctx->h_out + hdesc;
    for (int i = 0; i < n; ++i) {
        Plan &p = plans[i];
        const FrameDesc &b = back[i];
        const uint8_t *fbidx = ob + p.off_fbidx, *fbrow = ob + p.off_fbrow;
        const unsigned long long *cst = (const unsigned long long *)(ob + p.off_stats);
        if (cst[3] & 4)
            return fail(ctx, ZF_ERR_CUDA, "a refinement trial unit needed more tiles than its shared memory holds");
        if (cst[3]) return fail(ctx, ZF_ERR_TIMEOUT, "a statistics tile load did not arrive within its wait limit");
        const bool searched = (run.stages & STG_LR_SEARCH) && !run.lr_given;
        auto packed = [&](int pl) { return (const zf::PackedUnit *)(ob + p.off_packed[pl]); };
        zf_decisions *o = p.out;
        if (o) {
            if (run.stages & STG_DB_PICK) std::memcpy(o->lf, p.d.lf, 4);
            o->nhfb = b.nhfb;
            o->nvfb = b.nvfb;
            if ((run.stages & STG_CDEF_SEARCH) && !run.cdef_given) {
                o->cdef_damping = (uint8_t)b.cdef.damping;
                o->cdef_bits = (uint8_t)b.cdef.bits;
                std::memcpy(o->cdef_y, b.cdef.y_str, 8);
                std::memcpy(o->cdef_uv, b.cdef.uv_str, 8);
                if (o->cdef_fb_idx)
                    for (int k = 0; k < p.nfb; ++k) o->cdef_fb_idx[k] = b.cdef.bits ? fbidx[k] : 0;
            }
            if (searched) {
                for (int pl = 0; pl < 3; ++pl) {
                    o->lr[pl].frame_rtype = b.lr[pl].on ? b.lr[pl].frame_rtype : ZF_RESTORE_NONE;
                    o->lr[pl].unit_size = 256;
                    o->lr[pl].hunits = p.hunits[pl];
                    o->lr[pl].vunits = p.vunits[pl];
                    if (!o->lr_units[pl]) continue;
                    const size_t nu = (size_t)p.hunits[pl] * p.vunits[pl];
                    if (b.lr[pl].on) {
                        std::memcpy(o->lr_units[pl], packed(pl), nu * sizeof(zf_lr_unit));
                        continue;
                    }
                    static const int16_t def[8] = {3, -7, 15, -22, 15, -7, 3, 0};
                    for (size_t u = 0; u < nu; ++u) {
                        zf_lr_unit &lu = o->lr_units[pl][u];
                        std::memset(&lu, 0, sizeof(lu));
                        std::memcpy(lu.vfilter, def, 16);
                        std::memcpy(lu.hfilter, def, 16);
                    }
                }
            }
        }
        if (stats) {
            zf_stats &s = stats[i];
            std::memset(&s, 0, sizeof(s));
            s.cdef_filtered_px = cst[0];
            s.cdef_changed_px = cst[1];
            int sbc = 0;
            for (int k = 0; k < p.nfb; ++k) sbc += fbrow[k];
            s.cdef_sb_count = sbc;
            for (int pl = 0; pl < 3; ++pl) {
                s.lr_frame_rtype[pl] = b.lr[pl].on ? b.lr[pl].frame_rtype : 0;
                if (searched && b.lr[pl].on && b.lr[pl].frame_rtype) {
                    const zf::PackedUnit *pu = packed(pl);
                    for (size_t u = 0; u < p.rects[pl].size(); ++u) s.lr_wiener_units += pu[u].rtype == 1;
                }
            }
        }
    }
    if (run.rows || ctx->trace) TRY(search_records(ctx, plans, back, ob, run, p_trace));
    return ZF_OK;
}

}  // namespace

namespace zf {
// Dims and CDEF policy of a frame descriptor (no pointers), for entry points
// outside this file that build their own descriptor.
int describe_cdef_frame(const zf_frame *f, FrameDesc *d) {
    const int e = validate_frame(nullptr, f);
    if (e != ZF_OK) return e;
    std::memset(d, 0, sizeof(*d));
    d->bd = f->bit_depth;
    d->w = f->width;
    d->h = f->height;
    d->tw = f->true_width;
    d->th = f->true_height;
    d->chroma = f->chroma_420 ? 1 : 0;
    d->preset = f->preset;
    d->qindex = f->qindex;
    d->sharpness = f->sharpness;
    d->mi_cols = f->width / 4;
    d->mi_rows = f->height / 4;
    d->nhfb = (f->width + 63) / 64;
    d->nvfb = (f->height + 63) / 64;
    cdef_policy(f, d->cdef);
    return ZF_OK;
}
}  // namespace zf

namespace {
// ---- self-guided restoration entry points (zf_sgr.cu kernels) ------------
int validate_sgr_plane(zf_ctx *ctx, const zf_sgr_plane *p, int32_t nunits, int *hunits, int *vunits) {
    if (!ctx) return ZF_ERR_ARG;
    if (!p) return fail(ctx, ZF_ERR_ARG, "plane is NULL");
    if (p->bit_depth != 8 && p->bit_depth != 10) return fail(ctx, ZF_ERR_UNSUPPORTED, "bit_depth must be 8 or 10");
    if (p->width <= 0 || p->height <= 0 || p->width > 16384 || p->height > 16384)
        return fail(ctx, ZF_ERR_INVALID_DIMS, "plane dims must be in [1, 16384]");
    if (p->ss_y != 0 && p->ss_y != 1) return fail(ctx, ZF_ERR_ARG, "ss_y must be 0 or 1");
    if (!p->dgd) return fail(ctx, ZF_ERR_ARG, "missing dgd plane");
    *hunits = count_units_in_tile(256, p->width);
    *vunits = count_units_in_tile(256, p->height);
    if (nunits != *hunits * *vunits) return fail(ctx, ZF_ERR_ARG, "nunits does not match the plane's unit grid");
    return ZF_OK;
}

// The 64 x 32 tiles of every unit rectangle (search).
void sgr_search_tiles(int pw, int ph, int ss, std::vector<zf::SgrTile> &tiles) {
    std::vector<UnitRect> rects;
    rest_units(pw, ph, ss, rects);
    tiles.clear();
    for (size_t u = 0; u < rects.size(); ++u) {
        const UnitRect &r = rects[u];
        for (int y = r.v_start; y < r.v_end; y += zf::kSgrTileHHost)
            for (int x = r.h_start; x < r.h_end; x += zf::kSgrTileWHost)
                tiles.push_back(zf::SgrTile{(int)u, x, y, std::min(zf::kSgrTileWHost, r.h_end - x),
                                            std::min(zf::kSgrTileHHost, r.v_end - y), 1, 0, 0});
    }
}

// The apply's tiles: every stripe (64 >> ss rows, offset 8 >> ss) split into
// 32-row pieces, 64-column tiles inside each unit column; a tile's unit is
// the decoder's (unit row from the stripe, unit column from x).
void sgr_apply_tiles(int pw, int ph, int ss, int hunits, int vunits, std::vector<zf::SgrTile> &tiles) {
    const int full = 64 >> ss, off = 8 >> ss;
    tiles.clear();
    for (int ys = 0; ys < ph;) {
        const int stripe = (ys + off) / full, start = -off + stripe * full, end = start + full - 1;
        const int ye = std::min(ph, end + 1);
        const int urow = std::min(vunits - 1, (ys + off) / 256);
        for (int y = ys; y < ye; y += zf::kSgrTileHHost)
            for (int uc = 0; uc < hunits; ++uc) {
                const int x0 = uc * 256, x1 = uc == hunits - 1 ? pw : (uc + 1) * 256;
                for (int x = x0; x < x1; x += zf::kSgrTileWHost)
                    tiles.push_back(zf::SgrTile{urow * hunits + uc, x, y, std::min(zf::kSgrTileWHost, x1 - x),
                                                std::min(zf::kSgrTileHHost, ye - y), start, end, 0});
            }
        ys = ye;
    }
}
}  // namespace

extern "C" {

int32_t zf_abi_version(void) { return ZF_ABI_VERSION; }

int32_t zf_create(zf_ctx **out, const zf_opts *opts) {
    if (!out) return ZF_ERR_ARG;
    *out = nullptr;
    zf_ctx *c = new (std::nothrow) zf_ctx();
    if (!c) return ZF_ERR_ALLOC;
    c->device = opts ? opts->device : 0;
    c->budget = opts ? opts->hbm_budget_bytes : 0;
    c->cancel = opts ? opts->cancel_flag : nullptr;
    c->graphs = opts && (opts->flags & ZF_OPT_GRAPHS);
    c->tma = !(opts && (opts->flags & ZF_OPT_NO_TMA));
    if (cudaSetDevice(c->device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        set_kernel_attributes() != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return ZF_ERR_CUDA;
    }
    if (const char *tp = std::getenv("ZF_TRACE")) zf_trace(c, tp);
    *out = c;
    return ZF_OK;
}

void zf_destroy(zf_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->arena) cudaFree(ctx->arena);
    if (ctx->h_meta) cudaFreeHost(ctx->h_meta);
    if (ctx->h_out) cudaFreeHost(ctx->h_out);
    if (ctx->h_jobs) cudaFreeHost(ctx->h_jobs);
    if (ctx->d_jobs) cudaFree(ctx->d_jobs);
    if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->trace_owned) std::fclose(ctx->trace);
    delete ctx;
}

int32_t zf_set_wait_limit(zf_ctx *ctx, uint32_t iterations) {
    if (!ctx) return ZF_ERR_ARG;
    ctx->wait_limit = iterations ? iterations : 1u << 20;
    return ZF_OK;
}

int32_t zf_trace(zf_ctx *ctx, const char *path) {
    if (!ctx) return ZF_ERR_ARG;
    if (ctx->trace_owned) std::fclose(ctx->trace);
    ctx->trace = nullptr;
    ctx->trace_owned = false;
    if (!path || !*path) return ZF_OK;
    if (std::strcmp(path, "-") == 0) {
        ctx->trace = stderr;
        return ZF_OK;
    }
    ctx->trace = std::fopen(path, "w");
    if (!ctx->trace) return fail(ctx, ZF_ERR_ARG, std::string("cannot open trace file ") + path);
    ctx->trace_owned = true;
    return ZF_OK;
}

const char *zf_last_error(const zf_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

uint64_t zf_device_bytes(const zf_ctx *ctx) { return ctx ? (uint64_t)ctx->arena_cap : 0; }

int32_t zf_trim(zf_ctx *ctx) {
    if (!ctx) return ZF_ERR_ARG;
    CU(cudaSetDevice(ctx->device));
    CU(cudaStreamSynchronize(ctx->stream));
    if (ctx->arena) {
        CU(cudaFree(ctx->arena));
        ctx->arena = nullptr;
        ctx->arena_cap = 0;
    }
    return ZF_OK;
}

int32_t zf_reserve(zf_ctx *ctx, uint64_t device_bytes, uint64_t host_bytes) {
    if (!ctx) return ZF_ERR_ARG;
    CU(cudaSetDevice(ctx->device));
    TRY(ensure_arena(ctx, (size_t)device_bytes));
    TRY(ensure_host(ctx, ctx->h_meta, ctx->h_meta_cap, (size_t)host_bytes));
    TRY(ensure_host(ctx, ctx->h_out, ctx->h_out_cap, (size_t)host_bytes));
    // job lists for the gathered copies of up to 400 frames a call
    TRY(ensure_jobs(ctx, 400 * 13));
    return ZF_OK;
}

int32_t zf_sync(zf_ctx *ctx) {
    if (!ctx) return ZF_ERR_ARG;
    CU(cudaStreamSynchronize(ctx->stream));
    return ZF_OK;
}

int32_t zf_query_sizes(const zf_frame *f, zf_sizes *out) {
    if (!f || !out) return ZF_ERR_ARG;
    int e = validate_frame(nullptr, f);
    if (e) return e;
    Plan p;
    size_t cursor = 0, ucur = 0, rcur = 0, ocur = 0;
    plan_frame(p, f, cursor, ucur, rcur, ocur);
    // work items (upper bound): per unit its sums / statistics row blocks,
    // solve and trial items, per plane the apply (stripe, tile) items
    size_t items = 16;
    for (int pl = 0; pl < 3; ++pl) {
        const int ss = pl ? 1 : 0;
        items += p.rects[pl].size() * (384 / 16 + 1 + 392 / 12 + 1 + 1 + 1);
        items += (size_t)((p.d.lr[pl].ph + (8 >> ss)) / (64 >> ss) + 2) * ((p.d.lr[pl].pw + 63) / 64 + 1);
    }
    // coarse item indices: one int per 32 CTAs of a list (a 64x64 region
    // gives fewer than 64 CTAs over all lists) and two per list
    const size_t coarse = ((size_t)64 * p.d.nhfb * p.d.nvfb / 32 + 2 * 16) * sizeof(int);
    const size_t meta = align_up(sizeof(FrameDesc), 256) + items * sizeof(WorkItem) + coarse + 12 * 256 + rcur;
    std::memset(out, 0, sizeof(*out));
    out->nhfb = p.d.nhfb;
    out->nvfb = p.d.nvfb;
    for (int pl = 0; pl < 3; ++pl) {
        out->lr_hunits[pl] = p.hunits[pl];
        out->lr_vunits[pl] = p.vunits[pl];
    }
    out->lr_unit_size = 256;
    out->device_bytes = align_up(cursor, 256) + align_up(ucur, 256) + align_up(meta, 256) + align_up(ocur, 256) +
                        3 * 1024;  // deblock search scratch
    return ZF_OK;
}

int32_t zf_pack_geom(int32_t mi_cols, int32_t mi_rows, const uint32_t *block_id, const uint8_t *bw,
                     const uint8_t *bh, const uint8_t *tw, const uint8_t *th, const uint8_t *skip,
                     const uint8_t *skip_inter, uint32_t *out) {
    if (mi_cols <= 0 || mi_rows <= 0 || !block_id || !bw || !bh || !tw || !th || !skip || !skip_inter || !out)
        return ZF_ERR_ARG;
    auto lg = [](int v, int lo, int hi) -> int {
        if (v < lo || v > hi || (v & (v - 1))) return -1;
        int l = 0;
        while ((4 << l) < v) ++l;
        return l;
    };
    for (int r = 0; r < mi_rows; ++r)
        for (int c = 0; c < mi_cols; ++c) {
            const size_t i = (size_t)r * mi_cols + c;
            const int lbw = lg(bw[i], 4, 128), lbh = lg(bh[i], 4, 128), ltw = lg(tw[i], 4, 64), lth = lg(th[i], 4, 64);
            if (lbw < 0 || lbh < 0 || ltw < 0 || lth < 0) return ZF_ERR_GEOM;
            // Block alignment: block_id must be the aligned block origin.
            const int orow = r & ~((bh[i] >> 2) - 1), ocol = c & ~((bw[i] >> 2) - 1);
            if (block_id[i] != (uint32_t)((size_t)orow * mi_cols + ocol)) return ZF_ERR_GEOM;
            // Transform tiling: the mi at the aligned TX origin (same row /
            // column) carries the same transform dims.
            const int tr = r & ~((th[i] >> 2) - 1), tc = c & ~((tw[i] >> 2) - 1);
            const size_t ti = (size_t)tr * mi_cols + tc;
            if (tw[ti] != tw[i] || th[ti] != th[i]) return ZF_ERR_GEOM;
            out[i] = (uint32_t)lbw | ((uint32_t)lbh << 3) | ((uint32_t)ltw << 6) | ((uint32_t)lth << 9) |
                     (skip[i] ? ZF_MI_SKIP : 0u) | (skip_inter[i] ? ZF_MI_SKIP_INTER : 0u);
        }
    return ZF_OK;
}

uint64_t zf_launch_count(const zf_ctx *ctx) { return ctx ? ctx->launches : 0; }

int32_t zf_use_graphs(zf_ctx *ctx, int32_t enable) {
    if (!ctx) return ZF_ERR_ARG;
    ctx->graphs = enable != 0;
    return ZF_OK;
}

int32_t zf_get_tune(const zf_ctx *ctx, zf_tune *out) {
    if (!ctx || !out) return ZF_ERR_ARG;
    std::memset(out, 0, sizeof(*out));
    out->graphs = ctx->graphs ? 1 : 0;
    out->stats_tma = ctx->tma ? 1 : 0;
    out->apply_group = ctx->apply_group;
    out->stats_tc = ctx->stats_tc ? 1 : 0;
    out->trial_tile = ctx->trial_tile;
    out->db_levels = ctx->db_levels;
    return ZF_OK;
}

int32_t zf_set_tune(zf_ctx *ctx, const zf_tune *t) {
    if (!ctx || !t) return ZF_ERR_ARG;
    if (t->graphs < 0 || t->graphs > 1 || t->stats_tma < 0 || t->stats_tma > 1 || t->apply_group < 1 ||
        t->apply_group > zf::kApplyGroupMax || t->stats_tc < 0 || t->stats_tc > 1 ||
        (t->trial_tile != 32 && t->trial_tile != 64) || t->db_levels < 2 || t->db_levels > zf::kDbLevels)
        return fail(ctx, ZF_ERR_ARG, "tune setting out of range");
    ctx->graphs = t->graphs != 0;
    ctx->tma = t->stats_tma != 0;
    ctx->apply_group = t->apply_group;
    ctx->stats_tc = t->stats_tc != 0;
    ctx->trial_tile = t->trial_tile;
    ctx->db_levels = t->db_levels;
    return ZF_OK;
}

int32_t zf_autotune(zf_ctx *ctx, const zf_frame *frames, int32_t n, int32_t reps, zf_tune *best, zf_tune *cands,
                    int32_t max) {
    if (!ctx || !frames || n <= 0 || !best || reps < 1 || reps > 1000) return ZF_ERR_ARG;
    for (int i = 0; i < n; ++i) TRY(validate_frame(ctx, &frames[i]));
    CU(cudaSetDevice(ctx->device));
    zf_tune saved;
    zf_get_tune(ctx, &saved);
    // private recon copies: `work` is what the calls filter, `orig` restores it
    std::vector<zf_frame> fr(frames, frames + n);
    std::vector<void *> dev_bufs;
    std::vector<std::vector<uint8_t>> host_bufs;
    struct Plane {
        void *work;
        const void *orig;
        size_t bytes;
        bool dev;
    };
    std::vector<Plane> planes;
    auto cleanup = [&]() {
        for (void *p : dev_bufs) cudaFree(p);
        dev_bufs.clear();
    };
    for (int i = 0; i < n; ++i) {
        const zf_frame &f = frames[i];
        const size_t px = f.bit_depth == 8 ? 1 : 2;
        for (int pl = 0; pl < (f.chroma_420 ? 3 : 1); ++pl) {
            const size_t bytes = (pl ? (size_t)(f.width / 2) * (f.height / 2) : (size_t)f.width * f.height) * px;
            Plane P{nullptr, f.rec[pl], bytes, f.planes_on_device != 0};
            if (P.dev) {
                void *w = nullptr, *o = nullptr;
                if (cudaMalloc(&w, bytes) != cudaSuccess || cudaMalloc(&o, bytes) != cudaSuccess) {
                    if (w) cudaFree(w);
                    cudaGetLastError();
                    cleanup();
                    return fail(ctx, ZF_ERR_ALLOC, "autotune: no device memory for the frame copies");
                }
                dev_bufs.push_back(w);
                dev_bufs.push_back(o);
                if (cudaMemcpyAsync(o, f.rec[pl], bytes, cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess) {
                    cleanup();
                    return fail(ctx, ZF_ERR_CUDA, "autotune: copy of the recon failed");
                }
                P.work = w;
                P.orig = o;
            } else {
                host_bufs.emplace_back(bytes);
                P.work = host_bufs.back().data();
            }
            fr[i].rec[pl] = P.work;
            planes.push_back(P);
        }
    }
    auto restore = [&]() -> bool {
        for (const Plane &P : planes) {
            if (P.dev) {
                if (cudaMemcpyAsync(P.work, P.orig, P.bytes, cudaMemcpyDeviceToDevice, ctx->stream) != cudaSuccess)
                    return false;
            } else {
                std::memcpy(P.work, P.orig, P.bytes);
            }
        }
        return true;
    };
    std::vector<zf_decisions> outs((size_t)n);
    auto call = [&]() -> int {
        std::memset(outs.data(), 0, outs.size() * sizeof(zf_decisions));
        return n == 1 ? zf_filter_stage(ctx, fr.data(), outs.data(), nullptr)
                      : zf_submit_batch(ctx, fr.data(), n, outs.data(), nullptr);
    };
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        cleanup();
        return fail(ctx, ZF_ERR_CUDA, "autotune: event creation failed");
    }
    // Coordinate descent from the context's current setting: each knob in
    // turn takes every value with the others at the best so far -- graphs,
    // the statistics form (CUDA cores with TMA rows, CUDA cores with thread
    // staging, tensor cores), the restoration-apply column tiles per CTA, the
    // Wiener trial tile edge, the deblock trial levels per launch. A setting
    // timed once is not timed again.
    static const int kGroups[5] = {1, 2, 4, 8, 16};
    int count = 0, rc = ZF_OK;
    zf_tune win = saved;
    win.ms = -1.0;
    std::vector<zf_tune> timed;
    auto same = [](const zf_tune &a, const zf_tune &b) {
        return a.graphs == b.graphs && a.stats_tma == b.stats_tma && a.apply_group == b.apply_group &&
               a.stats_tc == b.stats_tc && a.trial_tile == b.trial_tile && a.db_levels == b.db_levels;
    };
    auto evaluate = [&](zf_tune c) -> int {
        for (const zf_tune &d : timed)
            if (same(d, c)) {
                if (win.ms < 0 || d.ms < win.ms) win = d;
                return ZF_OK;
            }
        zf_set_tune(ctx, &c);
        double total = 0.0;
        for (int r = -1; r < reps; ++r) {  // r = -1: warm-up
            if (!restore()) return fail(ctx, ZF_ERR_CUDA, "autotune: restoring the recon failed");
            cudaEventRecord(e0, ctx->stream);
            const int e = call();
            if (e != ZF_OK) return e;
            cudaEventRecord(e1, ctx->stream);
            float ms = 0.f;
            if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
                return fail(ctx, ZF_ERR_CUDA, "autotune: event timing failed");
            if (r >= 0) total += ms;
        }
        c.ms = total / reps;
        timed.push_back(c);
        if (cands && count < max) cands[count] = c;
        ++count;
        if (win.ms < 0 || c.ms < win.ms) win = c;  // strict: the earlier candidate wins ties
        return ZF_OK;
    };
    for (int knob = 0; knob < 5 && rc == ZF_OK; ++knob) {
        const zf_tune base = win;
        const int nv = knob == 0 ? 2 : knob == 1 ? 3 : knob == 2 ? 5 : knob == 3 ? 2 : 3;
        for (int v = 0; v < nv && rc == ZF_OK; ++v) {
            zf_tune c = base;
            if (knob == 0) {
                c.graphs = v;
            } else if (knob == 1) {
                c.stats_tc = v == 2 ? 1 : 0;
                c.stats_tma = v == 1 ? 0 : 1;
            } else if (knob == 2) {
                c.apply_group = kGroups[v];
            } else if (knob == 3) {
                c.trial_tile = v == 0 ? 64 : 32;
            } else {
                c.db_levels = v == 0 ? 8 : v == 1 ? 4 : 2;
            }
            rc = evaluate(c);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamSynchronize(ctx->stream);
    cleanup();
    if (rc != ZF_OK) {
        zf_set_tune(ctx, &saved);
        return rc;
    }
    zf_set_tune(ctx, &win);
    *best = win;
    return count;
}

int32_t zf_graph_stats(const zf_ctx *ctx, uint64_t out[3]) {
    if (!ctx || !out) return ZF_ERR_ARG;
    out[0] = ctx->graph_launches;
    out[1] = ctx->graph_updates;
    out[2] = ctx->graph_instantiations;
    return ZF_OK;
}

void *zf_stream(const zf_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int32_t zf_profile_enable(zf_ctx *ctx, int32_t enable) {
    if (!ctx) return ZF_ERR_ARG;
    ctx->profiling = enable != 0;
    return ZF_OK;
}

void zf_profile_reset(zf_ctx *ctx) {
    if (!ctx) return;
    cudaStreamSynchronize(ctx->stream);
    collect_profile(ctx);
    ctx->totals.clear();
}

int32_t zf_profile_read(const zf_ctx *ctx, zf_kernel_time *out, int32_t max) {
    if (!ctx) return ZF_ERR_ARG;
    const int n = (int)ctx->totals.size();
    for (int i = 0; i < n && i < max && out; ++i) out[i] = ctx->totals[i];
    return n;
}

int32_t zf_filter_stage(zf_ctx *ctx, const zf_frame *f, zf_decisions *out, zf_stats *stats) {
    if (!out) return fail(ctx, ZF_ERR_ARG, "decisions is NULL");
    Run r{STG_ALL, SET_A, SET_C, false, nullptr, false, false, false};
    return run_batch(ctx, f, 1, out, stats, r);
}

int32_t zf_submit_batch(zf_ctx *ctx, const zf_frame *frames, int32_t n, zf_decisions *outs, zf_stats *stats) {
    if (!outs) return fail(ctx, ZF_ERR_ARG, "decisions is NULL");
    Run r{STG_ALL, SET_A, SET_C, false, nullptr, false, false, false};
    return run_batch(ctx, frames, n, outs, stats, r);
}

int32_t zf_deblock_pick(zf_ctx *ctx, const zf_frame *f, uint8_t lf[4]) {
    if (!lf) return fail(ctx, ZF_ERR_ARG, "lf is NULL");
    zf_decisions d;
    std::memset(&d, 0, sizeof(d));
    Run r{STG_DB_PICK, SET_A, SET_A, false, nullptr, false, false, false};
    int e = run_batch(ctx, f, 1, &d, nullptr, r);
    if (e == ZF_OK) std::memcpy(lf, d.lf, 4);
    return e;
}

int32_t zf_deblock_sse_table(zf_ctx *ctx, const zf_frame *f, int32_t plane, const int32_t *levels, int32_t n,
                             int64_t *sse) {
    if (!ctx) return ZF_ERR_ARG;
    if (!levels || !sse || n <= 0 || n > 64) return fail(ctx, ZF_ERR_ARG, "levels: 1..64 entries required");
    for (int k = 0; k < n; ++k)
        if (levels[k] < 0 || levels[k] > 63) return fail(ctx, ZF_ERR_ARG, "level out of range 0..63");
    if (!f || plane < 0 || plane > 2 || (plane > 0 && !f->chroma_420)) return fail(ctx, ZF_ERR_ARG, "bad plane");
    DbTable t{plane, n, levels, sse};
    Run r{0, SET_A, SET_A, false, nullptr, false, false, false};
    r.table = &t;
    return run_batch(ctx, f, 1, nullptr, nullptr, r);
}

int32_t zf_deblock_apply(zf_ctx *ctx, const zf_frame *f, const uint8_t lf[4]) {
    if (!lf) return fail(ctx, ZF_ERR_ARG, "lf is NULL");
    zf_decisions d;
    std::memset(&d, 0, sizeof(d));
    std::memcpy(d.lf, lf, 4);
    Run r{STG_DB_APPLY, SET_A, SET_B, false, nullptr, true, false, false};
    return run_batch(ctx, f, 1, &d, nullptr, r);
}

int32_t zf_cdef_search(zf_ctx *ctx, const zf_frame *f, zf_decisions *out) {
    if (!out) return fail(ctx, ZF_ERR_ARG, "decisions is NULL");
    Run r{STG_CDEF_SEARCH, SET_B, SET_B, false, nullptr, false, false, false};
    return run_batch(ctx, f, 1, out, nullptr, r);
}

int32_t zf_cdef_search_rows(zf_ctx *ctx, const zf_frame *f, zf_decisions *out, uint64_t *mse, uint8_t *has_row,
                            int32_t *ncand) {
    if (!out || !ncand) return fail(ctx, ZF_ERR_ARG, "decisions or ncand is NULL");
    CdefRows rows{mse, has_row, ncand};
    Run r{STG_CDEF_SEARCH, SET_B, SET_B, false, nullptr, false, false, false};
    r.rows = &rows;
    return run_batch(ctx, f, 1, out, nullptr, r);
}

int32_t zf_cdef_apply(zf_ctx *ctx, const zf_frame *f, const zf_decisions *d, zf_stats *stats) {
    if (!d) return fail(ctx, ZF_ERR_ARG, "decisions is NULL");
    zf_decisions dd = *d;
    Run r{STG_CDEF_APPLY, SET_B, SET_A, false, nullptr, false, true, false};
    return run_batch(ctx, f, 1, &dd, stats, r);
}

int32_t zf_lr_search(zf_ctx *ctx, const zf_frame *f, zf_decisions *out) {
    if (!out) return fail(ctx, ZF_ERR_ARG, "decisions is NULL");
    Run r{STG_LR_SEARCH, SET_A, SET_A, false, nullptr, false, false, false};
    return run_batch(ctx, f, 1, out, nullptr, r);
}

int32_t zf_lr_apply(zf_ctx *ctx, const zf_frame *f, const void *const pre_cdef[3], const zf_decisions *d) {
    if (!d || !pre_cdef) return fail(ctx, ZF_ERR_ARG, "decisions or pre_cdef is NULL");
    zf_decisions dd = *d;
    Run r{STG_LR_APPLY, SET_A, SET_C, true, pre_cdef, false, false, true};
    return run_batch(ctx, f, 1, &dd, nullptr, r);
}

int32_t zf_sgr_search(zf_ctx *ctx, const zf_sgr_plane *p, uint32_t set_mask, zf_sgr_unit *units, int32_t nunits) {
    int hu, vu;
    TRY(validate_sgr_plane(ctx, p, nunits, &hu, &vu));
    if (!p->src) return fail(ctx, ZF_ERR_ARG, "missing source plane");
    if (!units) return fail(ctx, ZF_ERR_ARG, "units is NULL");
    if ((set_mask & 0xFFFFu) == 0 || (set_mask >> 16)) return fail(ctx, ZF_ERR_ARG, "set_mask must select sets 0..15");
    CU(cudaSetDevice(ctx->device));
    TRY(check_cancel(ctx));
    std::vector<int> sets;
    for (int k = 0; k < 16; ++k)
        if ((set_mask >> k) & 1) sets.push_back(k);
    const int nsets = (int)sets.size();
    std::vector<zf::SgrTile> tiles;
    sgr_search_tiles(p->width, p->height, p->ss_y, tiles);
    const size_t bps = p->bit_depth == 8 ? 1 : 2, pbytes = (size_t)p->width * p->height * bps;
    const bool dev = p->on_device != 0;
    // arena: [dgd, src copies (host planes)] | tiles | sets | acc | sse_none | out
    size_t cur = 0;
    auto take = [&cur](size_t b) {
        const size_t o = align_up(cur, 256);
        cur = o + b;
        return o;
    };
    const size_t o_dgd = dev ? 0 : take(pbytes), o_src = dev ? 0 : take(pbytes);
    const size_t o_tiles = take(tiles.size() * sizeof(zf::SgrTile)), o_sets = take(sets.size() * 4);
    const size_t o_acc = take((size_t)nunits * nsets * sizeof(zf::SgrAcc)), o_none = take((size_t)nunits * 8);
    const size_t o_out = take((size_t)nunits * sizeof(zf_sgr_unit));
    TRY(ensure_arena(ctx, cur));
    const size_t meta = align_up(tiles.size() * sizeof(zf::SgrTile), 256) + sets.size() * 4;
    TRY(ensure_host(ctx, ctx->h_meta, ctx->h_meta_cap, meta));
    TRY(ensure_host(ctx, ctx->h_out, ctx->h_out_cap, (size_t)nunits * sizeof(zf_sgr_unit)));
    uint8_t *base = ctx->arena;
    cudaStream_t st = ctx->stream;
    zf::SgrPlaneDesc P{p->bit_depth, p->width, p->height, p->ss_y, nullptr, nullptr, nullptr, nullptr};
    if (dev) {
        P.dgd = static_cast<const uint8_t *>(p->dgd);
        P.src = static_cast<const uint8_t *>(p->src);
    } else {
        TRY(copy_in(ctx, base + o_dgd, p->dgd, pbytes, false));
        TRY(copy_in(ctx, base + o_src, p->src, pbytes, false));
        P.dgd = base + o_dgd;
        P.src = base + o_src;
    }
    const size_t h_sets = align_up(tiles.size() * sizeof(zf::SgrTile), 256);
    std::memcpy(ctx->h_meta, tiles.data(), tiles.size() * sizeof(zf::SgrTile));
    std::memcpy(ctx->h_meta + h_sets, sets.data(), sets.size() * 4);
    CU(cudaMemcpyAsync(base + o_tiles, ctx->h_meta, tiles.size() * sizeof(zf::SgrTile), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(base + o_sets, ctx->h_meta + h_sets, sets.size() * 4, cudaMemcpyHostToDevice, st));
    CU(cudaMemsetAsync(base + o_acc, 0, o_out - o_acc, st));  // acc and sse_none start at zero
    const zf::SgrTile *d_tiles = (const zf::SgrTile *)(base + o_tiles);
    const int *d_sets = (const int *)(base + o_sets);
    zf::SgrAcc *d_acc = (zf::SgrAcc *)(base + o_acc);
    long long *d_none = (long long *)(base + o_none);
    zf_sgr_unit *d_out = (zf_sgr_unit *)(base + o_out);
    const size_t smem = zf::sgr_smem_bytes();
    const int ntiles = (int)tiles.size(), nacc = nunits * nsets;
    { LaunchScope ls_(ctx, "k_sgr_search");
    zf::k_sgr_search<<<ntiles, 256, smem, st>>>(P, d_tiles, d_sets, nsets, d_acc, d_none, 0); }
    TRY(launch_check(ctx, "k_sgr_search"));
    { LaunchScope ls_(ctx, "k_sgr_solve");
    zf::k_sgr_solve<<<(nacc + 127) / 128, 128, 0, st>>>(d_sets, nsets, d_acc, nacc); }
    TRY(launch_check(ctx, "k_sgr_solve"));
    { LaunchScope ls_(ctx, "k_sgr_search");
    zf::k_sgr_search<<<ntiles, 256, smem, st>>>(P, d_tiles, d_sets, nsets, d_acc, d_none, 1); }
    TRY(launch_check(ctx, "k_sgr_search"));
    { LaunchScope ls_(ctx, "k_sgr_pick");
    zf::k_sgr_pick<<<(nunits + 127) / 128, 128, 0, st>>>(d_sets, nsets, d_acc, d_none, d_out, nunits); }
    TRY(launch_check(ctx, "k_sgr_pick"));
    CU(cudaMemcpyAsync(ctx->h_out, d_out, (size_t)nunits * sizeof(zf_sgr_unit), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    TRY(launch_check(ctx, "stream"));
    collect_profile(ctx);
    std::memcpy(units, ctx->h_out, (size_t)nunits * sizeof(zf_sgr_unit));
    return ZF_OK;
}

int32_t zf_sgr_apply(zf_ctx *ctx, const zf_sgr_plane *p, const zf_sgr_unit *units, int32_t nunits, void *dst) {
    int hu, vu;
    TRY(validate_sgr_plane(ctx, p, nunits, &hu, &vu));
    if (!p->pre_cdef) return fail(ctx, ZF_ERR_ARG, "missing pre_cdef plane");
    if (!units || !dst) return fail(ctx, ZF_ERR_ARG, "units or dst is NULL");
    if (dst == p->dgd || dst == p->pre_cdef) return fail(ctx, ZF_ERR_ARG, "dst must not alias the input planes");
    for (int u = 0; u < nunits; ++u) {
        const zf_sgr_unit &x = units[u];
        if (x.set < -1 || x.set > 15) return fail(ctx, ZF_ERR_ARG, "unit set out of range");
        if (x.set >= 0 && (x.xqd[0] < -96 || x.xqd[0] > 31 || x.xqd[1] < -32 || x.xqd[1] > 95))
            return fail(ctx, ZF_ERR_ARG, "unit weights out of range");
    }
    CU(cudaSetDevice(ctx->device));
    TRY(check_cancel(ctx));
    std::vector<zf::SgrTile> tiles;
    sgr_apply_tiles(p->width, p->height, p->ss_y, hu, vu, tiles);
    const size_t bps = p->bit_depth == 8 ? 1 : 2, pbytes = (size_t)p->width * p->height * bps;
    const bool dev = p->on_device != 0;
    size_t cur = 0;
    auto take = [&cur](size_t b) {
        const size_t o = align_up(cur, 256);
        cur = o + b;
        return o;
    };
    const size_t o_dgd = dev ? 0 : take(pbytes), o_pre = dev ? 0 : take(pbytes), o_dst = dev ? 0 : take(pbytes);
    const size_t o_units = take((size_t)nunits * sizeof(zf_sgr_unit)), o_tiles = take(tiles.size() * sizeof(zf::SgrTile));
    TRY(ensure_arena(ctx, cur));
    const size_t h_tiles = align_up((size_t)nunits * sizeof(zf_sgr_unit), 256);
    TRY(ensure_host(ctx, ctx->h_meta, ctx->h_meta_cap, h_tiles + tiles.size() * sizeof(zf::SgrTile)));
    uint8_t *base = ctx->arena;
    cudaStream_t st = ctx->stream;
    zf::SgrPlaneDesc P{p->bit_depth, p->width, p->height, p->ss_y, nullptr, nullptr, nullptr, nullptr};
    if (dev) {
        P.dgd = static_cast<const uint8_t *>(p->dgd);
        P.pre = static_cast<const uint8_t *>(p->pre_cdef);
        P.dst = static_cast<uint8_t *>(dst);
    } else {
        TRY(copy_in(ctx, base + o_dgd, p->dgd, pbytes, false));
        TRY(copy_in(ctx, base + o_pre, p->pre_cdef, pbytes, false));
        P.dgd = base + o_dgd;
        P.pre = base + o_pre;
        P.dst = base + o_dst;
    }
    std::memcpy(ctx->h_meta, units, (size_t)nunits * sizeof(zf_sgr_unit));
    std::memcpy(ctx->h_meta + h_tiles, tiles.data(), tiles.size() * sizeof(zf::SgrTile));
    CU(cudaMemcpyAsync(base + o_units, ctx->h_meta, (size_t)nunits * sizeof(zf_sgr_unit), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(base + o_tiles, ctx->h_meta + h_tiles, tiles.size() * sizeof(zf::SgrTile),
                       cudaMemcpyHostToDevice, st));
    { LaunchScope ls_(ctx, "k_sgr_apply");
    zf::k_sgr_apply<<<(int)tiles.size(), 256, zf::sgr_smem_bytes(), st>>>(
        P, (const zf::SgrTile *)(base + o_tiles), (const zf_sgr_unit *)(base + o_units)); }
    TRY(launch_check(ctx, "k_sgr_apply"));
    if (!dev) TRY(copy_out(ctx, dst, base + o_dst, pbytes, false));
    CU(cudaStreamSynchronize(st));
    TRY(launch_check(ctx, "stream"));
    collect_profile(ctx);
    return ZF_OK;
}

// ---- per-superblock restoration syntax ----------------------------------

void zf_wiener_refs_reset(zf_wiener_refs *r) {
    if (!r) return;
    static const int16_t def[8] = {3, -7, 15, -22, 15, -7, 3, 0};  // WIENER_DEFAULT taps
    for (int p = 0; p < 3; ++p) {
        std::memcpy(r->vfilter[p], def, sizeof(def));
        std::memcpy(r->hfilter[p], def, sizeof(def));
    }
}

// corners_in_sb (svtav1-encoder/src/restoration.rs:1070-1106): the unit
// range whose top-left corners fall in the superblock; under superres the
// horizontal mi -> pixel mapping carries the denominator over
// SCALE_NUMERATOR = 8.
int32_t zf_lr_corners_in_sb(int32_t unit_size, int32_t is_uv, int32_t mi_row, int32_t mi_col, int32_t sb_mi,
                            int32_t frame_w, int32_t frame_h, int32_t sr_denom, int32_t out[4]) {
    if (!out || (unit_size != 32 && unit_size != 64 && unit_size != 128 && unit_size != 256) || mi_row < 0 ||
        mi_col < 0 || sb_mi <= 0 || frame_w <= 0 || frame_h <= 0 || (sr_denom != 0 && (sr_denom < 9 || sr_denom > 16)))
        return ZF_ERR_ARG;
    const int ss = is_uv ? 1 : 0;
    const int tile_w = (frame_w + ss) >> ss, tile_h = (frame_h + ss) >> ss;
    const int horz = count_units_in_tile(unit_size, tile_w), vert = count_units_in_tile(unit_size, tile_h);
    const int mi_size = 4 >> ss;
    const int mi_to_num_x = sr_denom ? mi_size * sr_denom : mi_size;
    const int denom_x = sr_denom ? unit_size * 8 : unit_size;
    const int rnd_x = denom_x - 1, rnd_y = unit_size - 1;
    const int rcol0 = (mi_col * mi_to_num_x + rnd_x) / denom_x;
    const int rrow0 = (mi_row * mi_size + rnd_y) / unit_size;
    const int rcol1 = std::min(((mi_col + sb_mi) * mi_to_num_x + rnd_x) / denom_x, horz);
    const int rrow1 = std::min(((mi_row + sb_mi) * mi_size + rnd_y) / unit_size, vert);
    if (!(rcol0 < rcol1 && rrow0 < rrow1)) return 0;
    out[0] = rcol0;
    out[1] = rcol1;
    out[2] = rrow0;
    out[3] = rrow1;
    return 1;
}

namespace {
// The bit-level steps of write_primitive_quniform / _subexpfin /
// _refsubexpfin (svtav1-entropy/src/lr.rs:40-145), emitted as elements.
struct SymOut {
    std::vector<zf_lr_sym> v;
    int plane = 0, unit = 0;
    void bits(uint32_t value, int n) {
        if (n <= 0) return;  // a zero-width literal codes nothing
        zf_lr_sym s{};
        s.kind = ZF_SYM_BITS;
        s.nbits = n;
        s.value = value;
        s.plane = (int16_t)plane;
        s.unit = unit;
        v.push_back(s);
    }
};
int msb_u32(uint32_t n) { return 31 - __builtin_clz(n); }
uint16_t recenter_nonneg_h(uint16_t r, uint16_t v) {
    if (v > (r << 1)) return v;
    if (v >= r) return (uint16_t)((v - r) << 1);
    return (uint16_t)(((r - v) << 1) - 1);
}
uint16_t recenter_finite_nonneg_h(uint16_t n, uint16_t r, uint16_t v) {
    if ((r << 1) <= n) return recenter_nonneg_h(r, v);
    return recenter_nonneg_h((uint16_t)(n - 1 - r), (uint16_t)(n - 1 - v));
}
void quniform(SymOut &o, int n, int v) {
    if (n <= 1) return;
    const int l = msb_u32((uint32_t)(n - 1)) + 1, m = (1 << l) - n;
    if (v < m) {
        o.bits((uint32_t)v, l - 1);
    } else {
        o.bits((uint32_t)(m + ((v - m) >> 1)), l - 1);
        o.bits((uint32_t)((v - m) & 1), 1);
    }
}
void subexpfin(SymOut &o, int n, int k, int v) {
    int i = 0, mk = 0;
    for (;;) {
        const int b = i ? k + i - 1 : k, a = 1 << b;
        if (n <= mk + 3 * a) {
            quniform(o, n - mk, v - mk);
            return;
        }
        const bool t = v >= mk + a;
        o.bits(t ? 1u : 0u, 1);
        if (!t) {
            o.bits((uint32_t)(v - mk), b);
            return;
        }
        ++i;
        mk += a;
    }
}
// write_wiener_filter (svtav1-entropy/src/lr.rs:154-236) against the
// plane's reference, which then becomes this filter.
void wiener_filter_syms(SymOut &o, int win, const int16_t *vf, const int16_t *hf, int16_t *rvf, int16_t *rhf) {
    static const int kMin[3] = {-5, -23, -17}, kMax[3] = {10, 8, 46}, kK[3] = {1, 2, 3};
    auto tap = [&](const int16_t *f, const int16_t *rf, int idx) {
        const int n = kMax[idx] - kMin[idx] + 1;
        subexpfin(o, n, kK[idx],
                  recenter_finite_nonneg_h((uint16_t)n, (uint16_t)(rf[idx] - kMin[idx]), (uint16_t)(f[idx] - kMin[idx])));
    };
    if (win == 7) tap(vf, rvf, 0);
    tap(vf, rvf, 1);
    tap(vf, rvf, 2);
    if (win == 7) tap(hf, rhf, 0);
    tap(hf, rhf, 1);
    tap(hf, rhf, 2);
    std::memcpy(rvf, vf, 16);
    std::memcpy(rhf, hf, 16);
}
}  // namespace

// write_lr_for_sb (svtav1-encoder/src/restoration.rs:1127-1182).
int32_t zf_lr_sb_syntax(const zf_decisions *d, int32_t mi_row, int32_t mi_col, int32_t sb_mi, int32_t frame_w,
                        int32_t frame_h, int32_t monochrome, int32_t sr_denom, zf_wiener_refs *refs,
                        zf_lr_sym *out, int32_t cap) {
    if (!d || !refs || (!out && cap > 0) || cap < 0) return ZF_ERR_ARG;
    zf_wiener_refs r = *refs;
    SymOut o;
    for (int pl = 0; pl < (monochrome ? 1 : 3); ++pl) {
        const zf_lr_plane &P = d->lr[pl];
        if (P.frame_rtype == 0) continue;  // RESTORE_NONE: corners_in_sb is None
        if (P.frame_rtype != 1 || !d->lr_units[pl]) return ZF_ERR_ARG;  // only WIENER frame types are coded here
        int32_t c[4];
        const int e = zf_lr_corners_in_sb(P.unit_size, pl > 0, mi_row, mi_col, sb_mi, frame_w, frame_h, sr_denom, c);
        if (e < 0) return e;
        if (e == 0) continue;
        if (c[1] > P.hunits || c[3] > P.vunits) return ZF_ERR_ARG;
        o.plane = pl;
        for (int rrow = c[2]; rrow < c[3]; ++rrow)
            for (int rcol = c[0]; rcol < c[1]; ++rcol) {
                const int unit = rcol + rrow * P.hunits;
                const zf_lr_unit &u = d->lr_units[pl][unit];
                const bool used = u.rtype != 0;
                o.unit = unit;
                zf_lr_sym s{};
                s.kind = ZF_SYM_WIENER_RESTORE;
                s.value = used ? 1u : 0u;
                s.plane = (int16_t)pl;
                s.unit = unit;
                o.v.push_back(s);
                if (used)
                    wiener_filter_syms(o, pl ? 5 : 7, u.vfilter, u.hfilter, r.vfilter[pl], r.hfilter[pl]);
            }
    }
    if ((int64_t)o.v.size() > cap) return ZF_ERR_ARG;
    if (!o.v.empty()) std::memcpy(out, o.v.data(), o.v.size() * sizeof(zf_lr_sym));
    *refs = r;
    return (int32_t)o.v.size();
}

// loop_filter_params / cdef_params / lr_params of write_key_frame_header
// (svtav1-entropy/src/obu.rs:1268-1377): fixed-width fields, MSB first.
int32_t zf_write_filter_params(const zf_decisions *d, const zf_header_opts *o, uint8_t *buf, int32_t cap,
                               int32_t *bit_pos) {
    if (!d || !o || !buf || !bit_pos || cap < 0 || *bit_pos < 0) return ZF_ERR_ARG;
    if (o->allow_intrabc) return ZF_OK;  // spec 5.9.11 / 5.9.19 / 5.9.20 defaults, nothing coded
    if (o->sharpness < 0 || o->sharpness > 7 || (o->sb_size != 64 && o->sb_size != 128)) return ZF_ERR_ARG;
    const bool mono = o->monochrome != 0;
    for (int k = 0; k < 4; ++k)
        if (d->lf[k] > 63) return ZF_ERR_ARG;
    if (d->cdef_damping < 3 || d->cdef_damping > 6 || d->cdef_bits > 3) return ZF_ERR_ARG;
    int pos = *bit_pos;
    bool overflow = false;
    auto put = [&](uint32_t v, int n) {
        for (int i = n - 1; i >= 0; --i) {
            if ((pos >> 3) >= cap) {
                overflow = true;
                return;
            }
            const uint8_t m = (uint8_t)(0x80u >> (pos & 7));
            buf[pos >> 3] = ((v >> i) & 1) ? (uint8_t)(buf[pos >> 3] | m) : (uint8_t)(buf[pos >> 3] & ~m);
            ++pos;
        }
    };
    // loop_filter_params()
    put(d->lf[0], 6);
    put(d->lf[1], 6);
    if (!mono && (d->lf[0] || d->lf[1])) {
        put(d->lf[2], 6);
        put(d->lf[3], 6);
    }
    put((uint32_t)o->sharpness, 3);
    put(0, 1);  // loop_filter_delta_enabled
    // cdef_params()
    put((uint32_t)(d->cdef_damping - 3), 2);
    put(d->cdef_bits, 2);
    for (int i = 0; i < (1 << d->cdef_bits); ++i) {
        if (d->cdef_y[i] > 63 || d->cdef_uv[i] > 63) return ZF_ERR_ARG;
        put(d->cdef_y[i], 6);
        if (!mono) put(d->cdef_uv[i], 6);
    }
    // lr_params()
    if (o->enable_restoration) {
        const int np = mono ? 1 : 3;
        bool all_none = true, chroma_none = true;
        for (int p = 0; p < np; ++p) {
            const int t = d->lr[p].frame_rtype;
            if (t < 0 || t > 3) return ZF_ERR_ARG;
            if (t) {
                all_none = false;
                if (p) chroma_none = false;
            }
            // lr_type pairs: NONE (0,0), WIENER (1,0), SGRPROJ (1,1), SWITCHABLE (0,1)
            put(t == 1 || t == 2, 1);
            put(t == 2 || t == 3, 1);
        }
        if (!all_none) {
            const int us = d->lr[0].unit_size;
            if ((us != 64 && us != 128 && us != 256) || us < o->sb_size) return ZF_ERR_ARG;
            if (o->sb_size == 64) put(us > 64, 1);
            if (us > 64) put(us > 128, 1);
        }
        if (!chroma_none) put(d->lr[1].unit_size != d->lr[0].unit_size, 1);
    }
    if (overflow) return ZF_ERR_ARG;
    *bit_pos = pos;
    return ZF_OK;
}

// ---- superres upscale and film grain (zf_post.cu kernels) ----------------

int32_t zf_superres_scaled_size(int32_t dim, int32_t denom) {
    // calculate_scaled_size_helper (svtav1-dsp/src/superres.rs:140)
    if (dim <= 0 || dim > 65535) return dim;
    if (denom != 8 && denom <= 16) {
        const int min_dim = std::min(16, dim);
        const int scaled = (dim * 8 + denom / 2) / denom;
        return std::max(scaled, min_dim);
    }
    return dim;
}

int32_t zf_superres_upscale(zf_ctx *ctx, const void *src, int32_t src_width, int32_t src_stride, void *dst,
                            int32_t dst_width, int32_t dst_stride, int32_t rows, int32_t bit_depth,
                            int32_t on_device) {
    if (!ctx) return ZF_ERR_ARG;
    if (!src || !dst) return fail(ctx, ZF_ERR_ARG, "src or dst is NULL");
    if (bit_depth != 8 && bit_depth != 10) return fail(ctx, ZF_ERR_UNSUPPORTED, "bit_depth must be 8 or 10");
    if (src_width <= 0 || dst_width < src_width || dst_width > 16384 || rows <= 0 || rows > 16384 ||
        src_stride < src_width || dst_stride < dst_width)
        return fail(ctx, ZF_ERR_INVALID_DIMS, "superres dims out of range");
    CU(cudaSetDevice(ctx->device));
    // upscale_convolve_step / upscale_convolve_x0 (superres.rs:117, :128)
    const int x_step = ((src_width << 14) + dst_width / 2) / dst_width;
    const int err = dst_width * x_step - (src_width << 14);
    const int x0r = (-((dst_width - src_width) << 13) + dst_width / 2) / dst_width + (1 << 7) - err / 2;
    const int x0 = (int)((uint32_t)x0r & 16383u);
    const size_t bps = bit_depth == 8 ? 1 : 2;
    const size_t sbytes = ((size_t)(rows - 1) * src_stride + src_width) * bps;
    const size_t dbytes = ((size_t)(rows - 1) * dst_stride + dst_width) * bps;
    const bool dev = on_device != 0;
    const uint8_t *d_src = static_cast<const uint8_t *>(src);
    uint8_t *d_dst = static_cast<uint8_t *>(dst);
    if (!dev) {
        TRY(ensure_arena(ctx, align_up(sbytes, 256) + dbytes));
        TRY(copy_in(ctx, ctx->arena, src, sbytes, false));
        d_src = ctx->arena;
        d_dst = ctx->arena + align_up(sbytes, 256);
    }
    cudaStream_t st = ctx->stream;
    { LaunchScope ls_(ctx, "k_superres_upscale");
    zf::k_superres_upscale<<<rows, 256, src_width * bps, st>>>(d_src, src_width, src_stride, d_dst, dst_width,
                                                                dst_stride, bit_depth, x_step, x0); }
    TRY(launch_check(ctx, "k_superres_upscale"));
    if (!dev) TRY(copy_out(ctx, dst, d_dst, dbytes, false));
    CU(cudaStreamSynchronize(st));
    TRY(launch_check(ctx, "stream"));
    collect_profile(ctx);
    return ZF_OK;
}

int32_t zf_film_grain_estimate(zf_ctx *ctx, const uint8_t *src, const uint8_t *recon, int32_t width,
                               int32_t height, int32_t stride, int32_t on_device, zf_film_grain *out) {
    if (!ctx) return ZF_ERR_ARG;
    if (!src || !recon || !out) return fail(ctx, ZF_ERR_ARG, "NULL argument");
    if (width < 0 || height < 0 || width > 65536 || height > 65536 || (height > 0 && stride < width))
        return fail(ctx, ZF_ERR_INVALID_DIMS, "film grain dims out of range");
    std::memset(out, 0, sizeof(*out));
    long long sum = 0;
    unsigned long long sq = 0;
    const long long n = (long long)width * height;
    if (n > 0) {
        CU(cudaSetDevice(ctx->device));
        const size_t bytes = (size_t)(height - 1) * stride + width;
        const bool dev = on_device != 0;
        const size_t o_sums = dev ? 0 : 2 * align_up(bytes, 256);
        TRY(ensure_arena(ctx, o_sums + 16));
        TRY(ensure_host(ctx, ctx->h_out, ctx->h_out_cap, 16));
        const uint8_t *d_src = src, *d_rec = recon;
        if (!dev) {
            TRY(copy_in(ctx, ctx->arena, src, bytes, false));
            TRY(copy_in(ctx, ctx->arena + align_up(bytes, 256), recon, bytes, false));
            d_src = ctx->arena;
            d_rec = ctx->arena + align_up(bytes, 256);
        }
        cudaStream_t st = ctx->stream;
        unsigned long long *d_sums = (unsigned long long *)(ctx->arena + o_sums);
        CU(cudaMemsetAsync(d_sums, 0, 16, st));
        // contiguous aligned planes: one flat run over a grid of 8 CTAs per SM
        // (rows_per_cta 0); otherwise row blocks
        const bool flat = stride == width && ((reinterpret_cast<uintptr_t>(d_src) | reinterpret_cast<uintptr_t>(d_rec)) & 15) == 0;
        const long long nchunk = (long long)width * height / 16;
        const int rpc = flat ? 0 : std::max(1, (int)((long long)height * width / (152LL * 4 * 16384) + 1));
        const int grid = flat ? (int)std::max(1LL, std::min(152LL * 8, (nchunk + 1023) / 1024)) : (height + rpc - 1) / rpc;
        { LaunchScope ls_(ctx, "k_grain_sums");
        zf::k_grain_sums<<<grid, 256, 0, st>>>(d_src, d_rec, width, height, stride, rpc, d_sums); }
        TRY(launch_check(ctx, "k_grain_sums"));
        CU(cudaMemcpyAsync(ctx->h_out, d_sums, 16, cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        TRY(launch_check(ctx, "stream"));
        collect_profile(ctx);
        unsigned long long h[2];
        std::memcpy(h, ctx->h_out, 16);
        sum = (long long)h[0];
        sq = h[1];
    }
    // estimate_film_grain (film_grain.rs:74-119): variance in f64, a flat
    // two-point luma scaling curve when it reaches 4
    const double var = n > 0 ? (double)sq / (double)n - ((double)sum / (double)n) * ((double)sum / (double)n) : 0.0;
    out->noise_var = var;
    if (var < 4.0) return ZF_OK;
    out->apply_grain = 1;
    out->grain_seed = 42;
    out->overlap_flag = 1;
    out->num_y_points = 2;
    const double sc = std::min(std::sqrt(var) * 2.0, 255.0);
    const uint8_t s8 = (uint8_t)sc;  // Rust `as u8` of a value in [0, 255]: truncation
    out->point_y_value[0] = 0;
    out->point_y_scaling[0] = s8;
    out->point_y_value[1] = 255;
    out->point_y_scaling[1] = s8;
    return ZF_OK;
}

int32_t zf_film_grain_synthesize(zf_ctx *ctx, uint8_t *frame, int32_t width, int32_t height, int32_t stride,
                                 int32_t on_device, const zf_film_grain *p) {
    if (!ctx) return ZF_ERR_ARG;
    if (!frame || !p) return fail(ctx, ZF_ERR_ARG, "NULL argument");
    if (width < 0 || height < 0 || width > 65536 || height > 65536 || (height > 0 && stride < width))
        return fail(ctx, ZF_ERR_INVALID_DIMS, "film grain dims out of range");
    if (!p->apply_grain || p->num_y_points == 0 || width == 0 || height == 0) return ZF_OK;
    CU(cudaSetDevice(ctx->device));
    const size_t bytes = (size_t)(height - 1) * stride + width;
    const bool dev = on_device != 0;
    uint8_t *d = frame;
    if (!dev) {
        TRY(ensure_arena(ctx, bytes));
        TRY(copy_in(ctx, ctx->arena, frame, bytes, false));
        d = ctx->arena;
    }
    cudaStream_t st = ctx->stream;
    const long long total = (long long)width * height;
    const long long threads = (total + zf::kGrainRunHost - 1) / zf::kGrainRunHost;
    { LaunchScope ls_(ctx, "k_grain_synth");
    zf::k_grain_synth<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(d, width, height, stride,
                                                                         (uint32_t)p->grain_seed,
                                                                         (int)p->point_y_scaling[0]); }
    TRY(launch_check(ctx, "k_grain_synth"));
    if (!dev) TRY(copy_out(ctx, frame, d, bytes, false));
    CU(cudaStreamSynchronize(st));
    TRY(launch_check(ctx, "stream"));
    collect_profile(ctx);
    return ZF_OK;
}

}  // extern "C"
