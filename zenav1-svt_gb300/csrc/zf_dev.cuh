// zf_dev.cuh -- device-side data layout shared by the filter-stage kernels.
//
// A launch processes a batch of frames. Every frame is described by one
// FrameDesc in device memory; every kernel walks a flat list of work items
// (frame, plane, tile) whose CTA ranges are prefix-summed on the host, so a
// single launch covers any mix of sizes and bit depths. Pixels are stored
// tight (stride = plane width) as uint8 (8-bit) or uint16 (10-bit); kernels
// branch on the frame's bit depth at load/store time only.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace zf {

constexpr int kMaxCand = 48;        // CDEF candidates at preset 0
constexpr int kMaxUnits = 4096;     // restoration units per plane (guarded on host)

// Restoration unit rectangle in plane pixels (TileLimits,
// svtav1-dsp/src/restoration.rs:1096-1101).
struct UnitRect {
    int h_start, h_end, v_start, v_end;
};

// Per-unit Wiener state, written by the stats/solve/trial/finish kernels.
struct LrUnit {
    int64_t sum_src;            // sum of src over the unit
    unsigned long long sse_blk; // sse_region parts: 16x16 blocks, right strip,
    unsigned long long sse_rgt; // bottom strip (the strips are truncated to
    unsigned long long sse_bot; // u32 at 10 bits, restoration.rs:1991-2036)
    int64_t sse_none;
    int64_t sse_wn;             // trial SSE, INT64_MAX when the score reverts
    unsigned long long tw_blk, tw_rgt, tw_bot;  // tiled trial SSE parts (no refinement)
    int64_t score;
    // Raw-sample sums (before the average correction and the bit-depth
    // divider): M, the H upper triangle (row-major win2 x win2) and the dgd
    // sums over the unit rectangle shifted by each window offset (the
    // centre one is the find_average numerator).
    int64_t m[49];
    int64_t h[2401];
    int64_t s[49];
    int32_t vd[7], hd[7];
    int16_t vf[8], hf[8];
    int32_t rtype;
    int32_t pad;
};

// Output record of a unit (the layout of zf_lr_unit in the C ABI).
struct PackedUnit {
    int16_t vf[8], hf[8];
    uint8_t rtype;
    uint8_t pad[7];
};

struct LrPlane {
    int on;              // plane searched
    int win;             // 5 or 7
    int pw, ph;          // true plane dims (chroma ceil)
    int stride;          // storage stride (aligned canvas)
    int hunits, vunits;
    int frame_rtype;
    int refine;          // finer_tile_search_wiener refinement (presets <= 3)
    int trial_out;       // the tiled trial writes its filtered pixels into C
    UnitRect *rects;     // hunits*vunits
    LrUnit *units;       // hunits*vunits
    PackedUnit *packed;  // hunits*vunits output records
    // Tensor maps (CUtensorMap, 128 B each, in the metadata image) of the
    // post-CDEF and source planes for the statistics kernel's TMA loads:
    // 4-byte elements over (stride / 4, ph), boxes of kTmaDBoxW x kTmaDBoxH
    // (post-CDEF) and kTmaXBoxW x kTmaXBoxH (source). nullptr: the kernel
    // stages with thread loads (10-bit, 7-tap, strides not a multiple of 16).
    const void *tm_a, *tm_s;
};

// Statistics kernel TMA boxes (5-tap window, 8-bit): the post-CDEF window
// of a CTA (25 rows = 17 rows + 8 halo rows) starting 16 bytes left of the
// unit (its 2-column halo at byte 14), the source rows of a CTA (17); widths
// cover a unit of up to 383 columns plus halos, in 4-byte elements. A box
// lands in shared memory with its width as the row pitch; the widths are
// 12 and 4 (mod 32) words, so eight consecutive rows start in eight
// different banks (the walks of a warp read the same column of up to a
// dozen rows; a pitch of 0 mod 32 words put every row in one bank).
constexpr int kTmaDBoxW = 108, kTmaDBoxH = 25, kTmaXBoxW = 100, kTmaXBoxH = 17;
constexpr int kTmaDLead = 14;  // byte of column -2 (the window's first) in a D row

// Restoration apply: at most this many 64-px column tiles of a stripe per
// CTA (the launch's group size is a kernel argument, 8 unless tuned).
constexpr int kApplyGroupMax = 16;

// CDEF joint strength search: bit counts 0..3, one cluster each.
constexpr int kFinLevels = 4;

struct CdefParams {
    int mode;            // 0: off (nothing signaled), 1: search, 2: fixed pick
    int damping, bits;
    int ncand, first_pass_num, sub_y, sub_uv;
    int pad;
    uint64_t lambda;
    int fs[kMaxCand];
    uint8_t y_str[8], uv_str[8];
};

struct FrameDesc {
    int bd;                 // 8 or 10
    int w, h;               // aligned canvas
    int tw, th;             // true dims
    int chroma;             // 4:2:0 planes present
    int preset, qindex, sharpness;
    int mi_cols, mi_rows;
    int nhfb, nvfb;
    uint8_t lf[4];          // deblock levels (written before the apply)
    // Planes: IN = input recon (read by the deblock passes only); B =
    // post-deblock (pre-CDEF); A = post-CDEF; C = post-LR (final); S =
    // source. IN may be A, or the caller's buffer, which may also be C.
    uint8_t *IN[3];
    uint8_t *A[3], *B[3], *C[3];
    const uint8_t *S[3];
    const uint32_t *mi;
    // CDEF
    CdefParams cdef;
    uint64_t *mse;          // nfb x 2 x ncand
    uint8_t *fb_row;        // nfb: fb has a non-skip 8x8
    uint8_t *fb_idx;        // nfb
    int *cdef_ids;          // 4 x nfb: compacted filter-block ids with rows (global fallback)
    uint32_t *cdef_rows32;  // 4 x nfb x 2 x ncand: compacted rows (global fallback)
    unsigned long long *cdef_stats;  // [filtered, changed, sb_count]
    // nfb x 64: direction | variance code << 3 of every non-skip 8x8 luma
    // block, written by the search (when not null) and read by the apply
    // when cdir_ok
    uint8_t *cdir;
    // joint strength search, one result per bit count 0..3 (zero on upload)
    unsigned long long fin_cost[4];
    uint8_t fin_lev[4][16];  // lev0[0..8) then lev1[0..8)
    int fin_done;            // clusters finished
    int cdir_ok;             // this call's search wrote cdir from the apply's B
    // LR
    LrPlane lr[3];
    int64_t rdmult;
    int lr_on;
    // iterations of the statistics kernel's bounded wait for its TMA boxes
    // (zf_set_wait_limit); a CTA that gives up sets cdef_stats[3]
    uint32_t wait_limit;
};

// k_cdef_finish (joint strength search on a cluster): bytes of the double-buffered pair partials per CTA (each
// rank owns ceil(npairs / cl) pairs and receives one partial per rank)
__host__ __device__ constexpr size_t fin_pair_bytes(int npairs, int cl) {
    return 2 * (size_t)cl * (size_t)((npairs + cl - 1) / cl) * 8;
}

// One entry of a launch work list: a tile of a frame/plane, owning CTAs
// [cta_begin, cta_begin + ctas).
struct WorkItem {
    int frame, plane;
    int a, b;               // item-specific (e.g. unit index, stripe)
    int cta_begin, ctas;
};

// The work item owning CTA `cta`. A list of more than one item is followed
// by a coarse index (written by the host): entry k is the item owning CTA
// 32 k, then a last entry n - 1; the binary search runs between two
// neighbouring entries (a few items at most), not over the whole list.
__device__ __forceinline__ int find_item(const WorkItem *items, int n, int cta) {
    if (n <= 1) return 0;
    const int *coarse = reinterpret_cast<const int *>(items + n);
    int lo = coarse[cta >> 5], hi = coarse[(cta >> 5) + 1];
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (items[mid].cta_begin <= cta) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// ---- pixel access --------------------------------------------------------
__device__ __forceinline__ int ldpx(const uint8_t *p, int64_t idx, int bd) {
    return bd == 8 ? (int)p[idx] : (int)reinterpret_cast<const uint16_t *>(p)[idx];
}
__device__ __forceinline__ void stpx(uint8_t *p, int64_t idx, int bd, int v) {
    if (bd == 8) p[idx] = (uint8_t)v; else reinterpret_cast<uint16_t *>(p)[idx] = (uint16_t)v;
}
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Row pointer (sample 0 of row y) of a plane with `stride` samples per row.
__device__ __forceinline__ const uint8_t *row_ptr(const uint8_t *plane, int64_t y, int stride, int bd) {
    return plane + y * stride * (bd == 8 ? 1 : 2);
}

// ---- word-wide access ----------------------------------------------------
// Planes are stored with rows of a multiple of 4 bytes (luma width % 8 == 0,
// chroma width % 4 == 0), so when a plane base is 4-byte aligned every word
// of 4 u8 or 2 u16 samples starting at a multiple of 4 (2) samples is one
// aligned 32-bit access.
__device__ __forceinline__ int word_samples(int bd) { return bd == 8 ? 4 : 2; }
__device__ __forceinline__ int word_sample(uint32_t v, int k, int bd) {
    return bd == 8 ? (int)((v >> (8 * k)) & 0xffu) : (int)((v >> (16 * k)) & 0xffffu);
}
__device__ __forceinline__ bool aligned4(const void *p) { return ((uintptr_t)p & 3) == 0; }
__device__ __forceinline__ int floor_div(int a, int b) { return a >= 0 ? a / b : -((b - 1 - a) / b); }

// Stage a window of a plane (all threads of the CTA call it): rows r in
// [0, nrows) read the row pointers rowp(r) (nullptr: a row of `fill`),
// columns x in [xa, xa + n). A column outside [0, pw) reads column
// clamp(x, 0, pw - 1) when clamp_x, else gives `fill`. put(r, x - xa, v)
// stores a sample. Each thread takes whole words: a word wholly inside
// [0, pw) of an aligned row is one 32-bit load, other words go per sample.
// A thread's words are taken B at a time: the B loads are issued before
// any of them is stored, so their latencies overlap (B = 1 for kernels
// whose registers are already scarce).
template <int B = 4, typename RowFn, typename PutFn>
__device__ __forceinline__ void stage_window(int bd, int pw, int nrows, int xa, int n, bool clamp_x, int fill,
                                             RowFn rowp, PutFn put) {
    const int spw = word_samples(bd);
    const int wa = floor_div(xa, spw), nw = floor_div(xa + n - 1, spw) - wa + 1;
    // flat over (row, word) pairs; the thread's row and word advance by the
    // constant quotient and remainder of blockDim.x (one division per call)
    const int step_r = blockDim.x / nw, step_w = blockDim.x - step_r * nw;
    int r = threadIdx.x / nw, w = threadIdx.x - r * nw;
    while (r < nrows) {
        int rr[B], x0s[B];
        uint32_t v[B];
        bool fast[B];
#pragma unroll
        for (int j = 0; j < B; ++j) {
            rr[j] = r < nrows ? r : -1;
            x0s[j] = (wa + w) * spw;
            fast[j] = false;
            v[j] = 0;
            if (rr[j] >= 0) {
                const uint8_t *row = rowp(r);
                const int x0 = x0s[j];
                if (row && x0 >= 0 && x0 + spw <= pw && aligned4(row)) {
                    v[j] = *reinterpret_cast<const uint32_t *>(row + (bd == 8 ? x0 : 2 * x0));
                    fast[j] = true;
                }
                r += step_r;
                w += step_w;
                if (w >= nw) {
                    w -= nw;
                    ++r;
                }
            }
        }
#pragma unroll
        for (int j = 0; j < B; ++j) {
            if (rr[j] < 0) continue;
            const int x0 = x0s[j];
            if (fast[j]) {
                for (int k = 0; k < spw; ++k) {
                    const int x = x0 + k;
                    if (x >= xa && x < xa + n) put(rr[j], x - xa, word_sample(v[j], k, bd));
                }
            } else {
                const uint8_t *row = rowp(rr[j]);
                for (int k = 0; k < spw; ++k) {
                    const int x = x0 + k;
                    if (x < xa || x >= xa + n) continue;
                    int vv = fill;
                    if (row) {
                        if (x >= 0 && x < pw) vv = ldpx(row, x, bd);
                        else if (clamp_x) vv = ldpx(row, clampi(x, 0, pw - 1), bd);
                    }
                    put(rr[j], x - xa, vv);
                }
            }
        }
    }
}

// ---- TMA and mbarrier (inline PTX) ---------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// A 4-byte asynchronous global -> shared copy (cp.async.ca): `src_bytes`
// 4 copies the word, 0 writes zeros (src is then not read, but stays a
// valid address). Completion: cp_async_wait_all() by the issuing thread,
// then a barrier for the others.
__device__ __forceinline__ void cp_async4(void *dst, const void *src, uint32_t src_bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(smem_u32(dst)), "l"(src), "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *mbar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(mbar)), "r"(parity)
        : "memory");
    return done != 0;
}
// try_wait with an explicit suspend-time hint: the thread waits at most
// about `ns` nanoseconds for the phase before the call returns false.
__device__ __forceinline__ bool mbar_try_wait_ns(uint64_t *mbar, uint32_t parity, uint32_t ns) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(mbar)), "r"(parity), "r"(ns)
        : "memory");
    return done != 0;
}
// Waits for the phase in steps of about `ns` nanoseconds, at most `limit`
// steps; false when it gave up.
__device__ __forceinline__ bool mbar_wait_timed(uint64_t *mbar, uint32_t parity, uint32_t limit, uint32_t ns) {
    for (uint32_t it = 0; it < limit; ++it)
        if (mbar_try_wait_ns(mbar, parity, ns)) return true;
    return false;
}
// Iterations of the drain wait after a timed-out wait: the copies already
// issued always complete, so this is long (seconds) but still bounded.
constexpr uint32_t kDrainWaitLimit = 1u << 26;
// Suspend-time hint of one step of the statistics kernel's first wait.
constexpr uint32_t kWaitStepNs = 100;
// Waits for the mbarrier phase with an iteration limit; false when it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *mbar, uint32_t parity, uint32_t limit) {
    for (uint32_t it = 0; it < limit; ++it)
        if (mbar_try_wait(mbar, parity)) return true;
    return false;
}
// The tensor map (written to global memory before the launch) is read
// through the tensor-map proxy.
__device__ __forceinline__ void tmap_acquire(const void *tmap) {
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(tmap) : "memory");
}
// 2-D tiled TMA load of one box at element coordinates (x, y) into shared
// memory (128-byte aligned), completing on mbar. x * element size must be a
// multiple of 16 bytes; out-of-range elements read as zero.
__device__ __forceinline__ void tma_load_2d(void *smem_dst, const void *tmap, int x, int y, uint64_t *mbar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(smem_dst)), "l"(tmap), "r"(x), "r"(y), "r"(smem_u32(mbar))
        : "memory");
}

// ---- packed geometry (zf_filter.h) --------------------------------------
__device__ __forceinline__ int mi_bw(uint32_t r) { return 4 << (r & 7); }
__device__ __forceinline__ int mi_bh(uint32_t r) { return 4 << ((r >> 3) & 7); }
__device__ __forceinline__ int mi_tw(uint32_t r) { return 4 << ((r >> 6) & 7); }
__device__ __forceinline__ int mi_th(uint32_t r) { return 4 << ((r >> 9) & 7); }
__device__ __forceinline__ bool mi_skip(uint32_t r) { return (r >> 12) & 1; }
__device__ __forceinline__ bool mi_skip_inter(uint32_t r) { return (r >> 13) & 1; }

// Error flag shared by all kernels of a context (first error wins).
struct DevStatus {
    int code;
    int where;
};

}  // namespace zf
