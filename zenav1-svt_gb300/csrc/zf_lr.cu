// zf_lr.cu -- Wiener loop restoration (search + apply) on the GPU.
//
// Reference: svtav1-dsp/src/restoration.rs (convolve :138-195 / :1820-1871,
// find_average :198, compute_stats :567-632 / :1738-1807, the tap solver
// :801-1056, stripes :1124-1385, sse_region :1666 / :1991) and
// svtav1-encoder/src/restoration.rs (search :675-924, apply :992-1052).
//
// Search data path: the reference extends the post-CDEF plane by edge
// replication (4 columns, 3 rows) before reading any window; every read
// that reaches a kept output here clamps its coordinates to the true plane,
// which is the same value. The search filters without stripe boundaries,
// where the 64-row stripe split and the 16-rounded processing-unit width
// change which call computes a pixel but not its value, so a unit is
// filtered as one separable 2-D convolution.
//
// Integer regrouping: M and H are sums of exact integer products; this file
// accumulates them in per-thread int32 partials over at most a few hundred
// pixels (products <= 1023^2, so no overflow) and folds them into int64, the
// same exact value the reference's per-pixel int64 accumulation reaches.
#include <climits>
#include <type_traits>

#include <cooperative_groups.h>

#include "zf_dev.cuh"

namespace zf {

constexpr int64_t kTapScale = 1 << 16;
constexpr int kStep = 128;  // WIENER_FILT_STEP


__device__ __forceinline__ int plane_stride(const FrameDesc &f, int p) { return p ? f.w / 2 : f.w; }

// ---------------------------------------------------------------------------
// 1. compute_stats on raw samples (restoration.rs:567-632 / :1738-1807), with
// find_average (:198) and sse_region (:1666 / :1991) folded in.
//
// M[a] = sum y_a x and H[a][b] = sum y_a y_b (b >= a) over the unit, y the
// win x win window of dgd - A in column-major order (index = col * win +
// row), x = src - A, A = find_average(dgd). With d = dgd, s = src, n the
// unit's pixel count and S_a = sum of d over the unit rectangle shifted by
// the window offset of a, the integer identities
//   H[a][b] = Hr[a][b] - A (S_a + S_b) + n A^2,
//   M[a]    = Mr[a] - A (S_a + sum s) + n A^2
// hold exactly, Hr and Mr being the same sums over the raw samples. So one
// pass accumulates Hr, Mr, S (S_centre / n is A), sum s and the three
// sse_region parts, and k_lr_solve applies the correction before the
// bit-depth divider: the same integers the reference reaches.
//
// Regrouping of Hr (exact integer sums). With window offsets s_a = (ra - h,
// ca - h) and delta = s_b - s_a = (dr, dc), Hr[a][b] = sum over the unit
// rectangle shifted by s_a of P[y][x] = d[y][x] * d[y + dr][x + dc]. For a
// fixed delta all (a, b) pairs share P and differ only in the shift, so each
// thread takes one image row y and one dr, slides along the row computing P
// for every dc at once, and gets the row sums over all shifted column
// windows [sc, sc + uw) from a running prefix; a row contributes to every
// vertical shift sr with y in [sr, sr + uh). Mr and the shift sums use the
// same walk with s (and 1) in place of the second factor. Row sums of <= 396
// products of magnitude <= 1023^2 fit int32; everything is folded into int64.
//
// 8-bit frames with the 5-tap window keep the staged rows as bytes, and the
// middle of every row walk (where no column window starts or ends) takes
// four columns per step: one 32-bit dot product of four byte products per
// dc (the partner row's bytes for dc = 1..3 are byte permutes of two
// aligned words).
//
// A CTA covers ROWS consecutive rows of the unit's vertical range extended
// by h = WIN/2 on both sides (items: a = unit, CTA offset = row block).
// Threads [0, NDR * rows) walk (row, dr) for Hr; the next WIN * (unit rows)
// walk (unit row i, ra) for Mr and the shift sums of row i + ra - h; the
// next (unit rows) take sum s and the sse parts of row i. The three kinds of
// walk take about the same time, so no warp waits long at the barrier after
// them (the sse work inside the Mr walks made those warps the slowest).
// ---------------------------------------------------------------------------
constexpr int kMaxUnitW = 384 + 8;

template <int WIN>
struct StatGeom {
    static constexpr int H = WIN / 2;
    static constexpr int NDR = 2 * WIN - 1;             // dr in [-(WIN-1), WIN-1]
    static constexpr int ROWS = 256 / (NDR + WIN + 1);  // rows per CTA (stat_rows_host)
    static constexpr int DROWS = ROWS + 2 * (WIN - 1);  // staged D rows
    static constexpr int DCOLS = kMaxUnitW + 2 * H + WIN;
    static constexpr int DSB = (DCOLS + 3) / 4 * 4;     // byte layout: row stride (a multiple of 4)
    static constexpr int XSB = (kMaxUnitW + 3) / 4 * 4;
};

__device__ __forceinline__ uint32_t ld_word(const uint8_t *p) { return *reinterpret_cast<const uint32_t *>(p); }

// Bytes k..k+3 of the little-endian byte string w0 w1 (k = 0..4).
template <int K>
__device__ __forceinline__ uint32_t bytes_at(uint32_t w0, uint32_t w1) {
    if constexpr (K == 0) return w0;
    else if constexpr (K == 4) return w1;
    else return __byte_perm(w0, w1, 0x3210 + 0x1111 * K);
}

// BD = 8 or 10: every frame of the launch has that bit depth, and only that
// path is compiled (the 8-bit byte walks or the 16-bit scalar walks; one
// kernel holding both took instruction-cache misses); BD = 0: either.
template <int WIN, int BD>
__global__ void __launch_bounds__(256, WIN == 5 ? 5 : 1) k_lr_stats(FrameDesc *frames, const WorkItem *items, int nitems) {
    using G = StatGeom<WIN>;
    constexpr int HALF = G::H, WIN2 = WIN * WIN;
    __shared__ __align__(128) int16_t D[G::DROWS * G::DCOLS];
    __shared__ __align__(128) int16_t X[G::ROWS * kMaxUnitW];
    __shared__ unsigned long long Hs[WIN2 * WIN2];
    __shared__ unsigned long long Ms[WIN2], Ss[WIN2], Es[4];  // Es: sum s, sse blocks, right, bottom
    __shared__ __align__(8) uint64_t mbar;
    // 5-tap window: each (unit row, window row) walk stores its Mr row parts
    // and shift sums, and each sse walk its four sums, in a slot of its own
    // (no shared-memory atomics, which serialised the lanes of a warp on the
    // same few words); they are summed over the rows after the walks.
    constexpr int SR = WIN == 5 ? G::ROWS : 1;
    __shared__ int Mrow[SR][WIN2];
    __shared__ unsigned Srow[SR][WIN2], Erow[SR][4];
    constexpr int kSlotSums = 2 * WIN2 + 4;  // Mr entries, shift sums, sse / source sums
    __shared__ long long slot_part[WIN == 5 ? 4 : 1][kSlotSums];
    static_assert(G::DROWS * G::DSB <= (int)sizeof(D) && G::ROWS * G::XSB <= (int)sizeof(X), "byte layout fits");
    static_assert(WIN != 5 || (kTmaDBoxH == G::DROWS && kTmaXBoxH == G::ROWS &&
                               kTmaDBoxW * 4 * kTmaDBoxH <= (int)sizeof(D) && kTmaXBoxW * 4 * kTmaXBoxH <= (int)sizeof(X) &&
                               kTmaDLead + kMaxUnitW + 2 * HALF + WIN <= kTmaDBoxW * 4 && kMaxUnitW <= kTmaXBoxW * 4 + 8),
                  "TMA boxes cover the 5-tap windows");
    const int it = find_item(items, nitems, blockIdx.x);
    const WorkItem wi = items[it];
    FrameDesc &f = frames[wi.frame];
    const LrPlane &pl = f.lr[wi.plane];
    const UnitRect r = pl.rects[wi.a];
    LrUnit &u = pl.units[wi.a];
    const int bd = BD ? BD : f.bd, stride = plane_stride(f, wi.plane);  // BD: every frame of the launch
    const int uw = r.h_end - r.h_start, uh = r.v_end - r.v_start;
    const bool packed = BD ? (WIN == 5 && BD == 8) : (WIN == 5 && bd == 8);
    uint8_t *Db = reinterpret_cast<uint8_t *>(D), *Xb = reinterpret_cast<uint8_t *>(X);
    const uint8_t *dg = f.A[wi.plane], *sr_ = f.S[wi.plane];
    // rows of this CTA in unit coordinates (extended range [-HALF, uh + HALF))
    const int y0 = -HALF + ((int)blockIdx.x - wi.cta_begin) * G::ROWS, y1 = min(uh + HALF, y0 + G::ROWS);
    // D rows [y0 - (WIN-1), y1 + (WIN-1)) clamped, columns [-HALF, uw + HALF + WIN)
    const int dy0 = y0 - (WIN - 1), dx0 = -HALF;
    const int dcols = uw + 2 * HALF + WIN;
    const int drows = (y1 - y0) + 2 * (WIN - 1);
    const int xi0 = max(y0, 0), xi1 = min(y1, uh);
    // 8-bit rows come by two TMA box loads when the plane has tensor maps:
    // D rows of kTmaDBoxW * 4 bytes from 16 bytes left of the unit (column
    // -2 at byte kTmaDLead), X rows of kTmaXBoxW * 4 bytes from the unit's
    // first column; otherwise threads stage them (row pitch DSB / XSB).
    const bool tma = packed && pl.tm_a != nullptr;
    const int dpitch = tma ? kTmaDBoxW * 4 : G::DSB, dlead = tma ? kTmaDLead : 0;
    const int xpitch = tma ? kTmaXBoxW * 4 : G::XSB;
    if (tma) {
        if (threadIdx.x == 0) {
            mbar_init(&mbar, 1);
            tmap_acquire(pl.tm_a);
            tmap_acquire(pl.tm_s);
            mbar_expect_tx(&mbar, (kTmaDBoxW * kTmaDBoxH + kTmaXBoxW * kTmaXBoxH) * 4);
            tma_load_2d(Db, pl.tm_a, (r.h_start - 16) >> 2, r.v_start + dy0, &mbar);
            tma_load_2d(Xb, pl.tm_s, r.h_start >> 2, r.v_start + xi0, &mbar);
        }
    } else {
        stage_window<1>(
            bd, pl.pw, drows, r.h_start + dx0, dcols, true, 0,
            [&](int rr) { return row_ptr(dg, clampi(r.v_start + dy0 + rr, 0, pl.ph - 1), stride, bd); },
            [&](int rr, int cc, int v) {
                if (packed) Db[rr * G::DSB + cc] = (uint8_t)v;
                else D[rr * G::DCOLS + cc] = (int16_t)v;
            });
        stage_window<1>(
            bd, pl.pw, xi1 - xi0, r.h_start, uw, true, 0,
            [&](int rr) { return row_ptr(sr_, r.v_start + xi0 + rr, stride, bd); },
            [&](int rr, int cc, int v) {
                if (packed) Xb[rr * G::XSB + cc] = (uint8_t)v;
                else X[rr * kMaxUnitW + cc] = (int16_t)v;
            });
    }
    for (int q = threadIdx.x; q < WIN2 * WIN2; q += blockDim.x) Hs[q] = 0;
    if (threadIdx.x < WIN2) Ms[threadIdx.x] = Ss[threadIdx.x] = 0;
    if (threadIdx.x < 4) Es[threadIdx.x] = 0;
    __syncthreads();
    if (tma) {
        // bounded wait for both boxes (f.wait_limit steps of about
        // kWaitStepNs nanoseconds: 2^20 steps, ~0.1 s, by default); on a
        // timeout the frame's error word is set, the copies already issued
        // are drained (they always land; the drain wait is long but bounded)
        // so that no box is still arriving in shared memory when the CTA ends
        const uint32_t lim = f.wait_limit == 0xFFFFFFFFu ? 0u : f.wait_limit;  // ZF_WAIT_GIVE_UP: a test
        const bool late = !mbar_wait_timed(&mbar, 0, lim, kWaitStepNs);
        if (__syncthreads_or(late)) {
            if (threadIdx.x == 0) atomicOr(&f.cdef_stats[3], 1ull);
            mbar_wait_bounded(&mbar, 0, kDrainWaitLimit);
            __syncthreads();
            return;
        }
        // The loads read zeros outside the tensor and the canvas padding
        // beyond the true width: clamp columns, then rows, to the plane
        // like the thread staging does.
        const int gx_lo = r.h_start + dx0, gx_hi = gx_lo + dcols;
        const int gy_lo = r.v_start + dy0, gy_hi = gy_lo + drows;
        const int cl = max(0, -gx_lo), cr = max(0, gx_hi - pl.pw);
        if (cl + cr) {
            for (int q = threadIdx.x; q < drows * (cl + cr); q += blockDim.x) {
                const int rr = q / (cl + cr), k = q - rr * (cl + cr);
                const int gy = gy_lo + rr;
                if (gy < 0 || gy >= pl.ph) continue;  // whole row copied below
                uint8_t *row = Db + rr * dpitch + dlead;  // byte c <-> column c - HALF
                if (k < cl) row[k] = row[-gx_lo];
                else row[dcols - 1 - (k - cl)] = row[pl.pw - 1 - gx_lo];
            }
            __syncthreads();
        }
        if (gy_lo < 0 || gy_hi > pl.ph) {
            for (int q = threadIdx.x; q < drows * dcols; q += blockDim.x) {
                const int rr = q / dcols, c = q - rr * dcols;
                const int gy = gy_lo + rr;
                if (gy >= 0 && gy < pl.ph) continue;
                Db[rr * dpitch + dlead + c] = Db[(clampi(gy, 0, pl.ph - 1) - gy_lo) * dpitch + dlead + c];
            }
            __syncthreads();
        }
    }
    auto Dat = [&](int y, int x) -> int {
        return packed ? (int)Db[(y - dy0) * dpitch + (x - dx0) + dlead] : (int)D[(y - dy0) * G::DCOLS + (x - dx0)];
    };

    const int nh = G::NDR * (y1 - y0);
    const int t = threadIdx.x;
    // Every row's sums go through the cross-row reduction; rows with every
    // vertical shift valid (HALF <= y < uh - HALF) add to all of them.
    const bool all_interior = y0 >= HALF && y1 <= uh - HALF;
    int rs[WIN][WIN];  // rs[dc][sc + HALF]
    bool keep = false;
#pragma unroll
    for (int k = 0; k < WIN; ++k)
#pragma unroll
        for (int j = 0; j < WIN; ++j) rs[k][j] = 0;
    if (t < nh) {
        // ---- Hr: one (row y, dr) per thread; every such thread keeps its
        // row sums (zeros when the partner row is outside the range)
        keep = true;
        const int dr = t % G::NDR - (WIN - 1);
        const int y = y0 + t / G::NDR;
        // the row and its partner must lie in the extended range
        if (y + dr >= -HALF && y + dr < uh + HALF) {
            int pre[WIN];
#pragma unroll
            for (int k = 0; k < WIN; ++k) pre[k] = 0;
            int win[WIN];  // d[y + dr][x + dc], dc = 0..WIN-1
#pragma unroll
            for (int k = 0; k < WIN - 1; ++k) win[k + 1] = Dat(y + dr, -HALF + k);
            // x runs over [-HALF, uw + HALF); prefix bookkeeping at the
            // column-window starts (x = sc) and ends (x = sc + uw), which
            // all lie outside the middle range [HALF + 1, uw - HALF).
            auto step = [&](int x) {  // one column: window slide, products
#pragma unroll
                for (int k = 0; k < WIN - 1; ++k) win[k] = win[k + 1];
                win[WIN - 1] = Dat(y + dr, x + WIN - 1);
                const int a = Dat(y, x);
#pragma unroll
                for (int dc = 0; dc < WIN; ++dc) pre[dc] += a * win[dc];
            };
            const int xm0 = HALF + 1, xm1 = max(xm0, uw - HALF);
            int x = -HALF;
            if (uw >= 16) {
                // head: x = sc starts the windows of sc (unrolled, so the
                // bookkeeping is resolved at compile time)
#pragma unroll
                for (int k = 0; k < WIN; ++k) {
#pragma unroll
                    for (int dc = 0; dc < WIN; ++dc)
                        if (k + dc <= WIN - 1) rs[dc][k] -= pre[dc];
                    step(k - HALF);
                }
                x = xm0;
                if (packed) {
                    if constexpr (WIN == 5) {
                        // plain steps up to a word boundary of the byte rows
                        // (x + HALF + row lead = 0 mod 4), then four columns per step
                        const int xs = HALF + 1 + ((4 - ((2 * HALF + 1 + dlead) & 3)) & 3);
                        for (; x < xs; ++x) step(x);
                        const uint8_t *ra_ = Db + (y - dy0) * dpitch + dlead + HALF,
                                      *rb_ = Db + (y + dr - dy0) * dpitch + dlead + HALF;
                        if (x + 4 <= xm1) {
                            uint32_t w0 = ld_word(rb_ + x);
                            // four steps per iteration: the next steps' loads
                            // issue before this step's products need theirs
#pragma unroll 4
                            for (; x + 4 <= xm1; x += 4) {
                                const uint32_t a4 = ld_word(ra_ + x), w1 = ld_word(rb_ + x + 4);
                                pre[0] = (int)__dp4a(a4, w0, (uint32_t)pre[0]);
                                pre[1] = (int)__dp4a(a4, bytes_at<1>(w0, w1), (uint32_t)pre[1]);
                                pre[2] = (int)__dp4a(a4, bytes_at<2>(w0, w1), (uint32_t)pre[2]);
                                pre[3] = (int)__dp4a(a4, bytes_at<3>(w0, w1), (uint32_t)pre[3]);
                                pre[4] = (int)__dp4a(a4, w1, (uint32_t)pre[4]);
                                w0 = w1;
                            }
                            // the step's window: win[k + 1] = d[y + dr][x + k]
#pragma unroll
                            for (int k = 0; k < WIN - 1; ++k) win[k + 1] = Dat(y + dr, x + k);
                        }
                    }
                } else {
                    // middle: the window rotates through registers (slot
                    // (u + dc) % WIN holds d[y + dr][x + u + dc]), no moves
                    int w[WIN];
#pragma unroll
                    for (int k = 0; k < WIN - 1; ++k) w[k] = win[k + 1];
                    for (; x + WIN <= xm1; x += WIN) {
#pragma unroll
                        for (int u = 0; u < WIN; ++u) {
                            w[(u + WIN - 1) % WIN] = Dat(y + dr, x + u + WIN - 1);
                            const int a = Dat(y, x + u);
#pragma unroll
                            for (int dc = 0; dc < WIN; ++dc) pre[dc] += a * w[(u + dc) % WIN];
                        }
                    }
#pragma unroll
                    for (int k = 0; k < WIN - 1; ++k) win[k + 1] = w[k];
                }
                for (; x < uw - HALF; ++x) step(x);
                // tail: x = sc + uw ends the windows of sc; the last end
                // (sc = HALF) is at x = uw + HALF, past the walk
#pragma unroll
                for (int k = 0; k < WIN; ++k) {
#pragma unroll
                    for (int dc = 0; dc < WIN; ++dc)
                        if (k + dc <= WIN - 1) rs[dc][k] += pre[dc];
                    if (k < WIN - 1) step(uw - HALF + k);
                }
            } else {
                // narrow unit: starts and ends may interleave
                for (; x < uw + HALF; ++x) {
#pragma unroll
                    for (int dc = 0; dc < WIN; ++dc)
#pragma unroll
                        for (int sc = -HALF; sc <= HALF; ++sc) {
                            if (sc + HALF + dc > WIN - 1) continue;  // cb = ca + dc < WIN
                            if (x == sc) rs[dc][sc + HALF] -= pre[dc];
                            if (x == sc + uw) rs[dc][sc + HALF] += pre[dc];
                        }
                    step(x);
                }
#pragma unroll
                for (int dc = 0; dc < WIN; ++dc)
                    if (HALF + HALF + dc <= WIN - 1) rs[dc][2 * HALF] += pre[dc];
            }
            // rs goes to the cross-row reduction after the walks, which adds
            // it to Hr[a][b], a = (ca, ra), b = (ca + dc, ra + dr) (dc = 0 of
            // a negative dr mirrors a positive dr and is dropped there)
        }
    } else if (t < nh + WIN * (xi1 - xi0)) {
        // ---- Mr and shift sums: one (unit row i, ra) per thread
        const int q = t - nh;
        const int ra = q % WIN, i = xi0 + q / WIN;
        const int yy = i + ra - HALF;
        int acc[WIN];  // Mr[ca][ra] row parts
#pragma unroll
        for (int k = 0; k < WIN; ++k) acc[k] = 0;
        // c0 = sum of d[yy][j - HALF], j in [0, uw) (the ca = 0 column window)
        unsigned c0 = 0;
        int j = 0;
        if (packed) {
            if constexpr (WIN == 5) {
                const uint8_t *rd = Db + (yy - dy0) * dpitch + dlead;  // byte j + ca is d[yy][j + ca - HALF]
                const uint8_t *rx = Xb + (i - xi0) * xpitch;
                const int uw4 = uw & ~3;
                // four columns per step: the ca windows are bytes ca + sh .. ca + sh + 3
                // of the aligned words from rd - sh (sh = 0 for thread-staged rows,
                // 2 for the TMA rows whose column -2 sits at byte 14)
                auto mwalk = [&](auto shc) {
                    constexpr int SH = decltype(shc)::value;
                    const uint8_t *ra = rd - SH;
                    uint32_t w0 = ld_word(ra), w1 = ld_word(ra + 4);
#pragma unroll 4
                    for (; j < uw4; j += 4) {
                        const uint32_t w2 = ld_word(ra + j + 8), xv = ld_word(rx + j);
                        const uint32_t e0 = bytes_at<SH>(w0, w1), e1 = bytes_at<SH + 1>(w0, w1);
                        const uint32_t d2 = SH == 2 ? w1 : bytes_at<(SH + 2) & 3>(w0, w1);
                        const uint32_t e3 = SH == 2 ? bytes_at<1>(w1, w2) : bytes_at<SH + 3>(w0, w1);
                        const uint32_t e4 = SH == 2 ? bytes_at<2>(w1, w2) : w1;
                        acc[0] = (int)__dp4a(e0, xv, (uint32_t)acc[0]);
                        acc[1] = (int)__dp4a(e1, xv, (uint32_t)acc[1]);
                        acc[2] = (int)__dp4a(d2, xv, (uint32_t)acc[2]);
                        acc[3] = (int)__dp4a(e3, xv, (uint32_t)acc[3]);
                        acc[4] = (int)__dp4a(e4, xv, (uint32_t)acc[4]);
                        c0 = __dp4a(e0, 0x01010101u, c0);
                        w0 = w1;
                        w1 = w2;
                    }
                };
                if (dlead & 3) mwalk(std::integral_constant<int, 2>());
                else mwalk(std::integral_constant<int, 0>());
                for (; j < uw; ++j) {
                    const int xv = rx[j];
#pragma unroll
                    for (int ca = 0; ca < WIN; ++ca) acc[ca] += (int)rd[j + ca] * xv;
                    c0 += rd[j];
                }
            }
        } else {
            int win[WIN];  // d[yy][j + ca - HALF], ca = 0..WIN-1
#pragma unroll
            for (int k = 0; k < WIN - 1; ++k) win[k + 1] = Dat(yy, -HALF + k);
            const int16_t *xr = X + (i - xi0) * kMaxUnitW;
            {
                // rotating window: slot (u + ca) % WIN holds d[yy][j + u + ca - HALF]
                int w[WIN];
#pragma unroll
                for (int k = 0; k < WIN - 1; ++k) w[k] = win[k + 1];
                for (; j + WIN <= uw; j += WIN) {
#pragma unroll
                    for (int u = 0; u < WIN; ++u) {
                        w[(u + WIN - 1) % WIN] = Dat(yy, j + u + HALF);
                        const int xv = xr[j + u];
#pragma unroll
                        for (int ca = 0; ca < WIN; ++ca) acc[ca] += w[(u + ca) % WIN] * xv;
                        c0 += w[u % WIN];
                    }
                }
#pragma unroll
                for (int k = 0; k < WIN - 1; ++k) win[k + 1] = w[k];
            }
            for (; j < uw; ++j) {
#pragma unroll
                for (int k = 0; k < WIN - 1; ++k) win[k] = win[k + 1];
                win[WIN - 1] = Dat(yy, j + HALF);
                const int xv = xr[j];
#pragma unroll
                for (int ca = 0; ca < WIN; ++ca) acc[ca] += win[ca] * xv;
                c0 += win[0];
            }
        }
        // column windows ca = 1..WIN-1 slide the ca = 0 one
        if constexpr (WIN == 5) {
            const int rr = i - xi0;
            unsigned cw = c0;
            Srow[rr][ra] = cw;
#pragma unroll
            for (int ca = 0; ca < WIN; ++ca) {
                Mrow[rr][ca * WIN + ra] = acc[ca];
                if (ca) {
                    cw = cw - (unsigned)Dat(yy, ca - 1 - HALF) + (unsigned)Dat(yy, ca - 1 - HALF + uw);
                    Srow[rr][ca * WIN + ra] = cw;
                }
            }
        } else {
#pragma unroll
            for (int ca = 0; ca < WIN; ++ca) atomicAdd(&Ms[ca * WIN + ra], (unsigned long long)(long long)acc[ca]);
            unsigned long long cw = c0;
            atomicAdd(&Ss[ra], cw);
#pragma unroll
            for (int ca = 1; ca < WIN; ++ca) {
                cw = cw - (unsigned)Dat(yy, ca - 1 - HALF) + (unsigned)Dat(yy, ca - 1 - HALF + uw);
                atomicAdd(&Ss[ca * WIN + ra], cw);
            }
        }
    } else if (t < nh + (WIN + 1) * (xi1 - xi0)) {
        // ---- sum s and the sse_region parts of unit row i: one row per
        // thread (d row i against the source row)
        const int i = xi0 + (t - nh - WIN * (xi1 - xi0));
        const int jr = uw - uw % 16;  // the right strip of sse_region
        unsigned sx = 0, e_in = 0, e_rgt = 0;
        int j = 0;
        if (packed) {
            const uint8_t *rd = Db + (i - dy0) * dpitch + dlead + HALF;  // byte j is d[i][j]
            const uint8_t *rx = Xb + (i - xi0) * xpitch;
            const int uw4 = uw & ~3;
            // four columns per step (j and jr are multiples of 4, so a step
            // lies on one side of the right strip); d words start on a word
            // boundary for the TMA rows, two bytes into one otherwise
            auto ewalk = [&](uint32_t xv, uint32_t dv) {
                sx = __dp4a(xv, 0x01010101u, sx);
                const uint32_t e = __vabsdiffu4(xv, dv);
                if (j >= jr) e_rgt = __dp4a(e, e, e_rgt);
                else e_in = __dp4a(e, e, e_in);
            };
            if (((dlead + HALF) & 3) == 0) {
#pragma unroll 4
                for (; j < uw4; j += 4) ewalk(ld_word(rx + j), ld_word(rd + j));
            } else {
                const uint8_t *ra = rd - 2;
                uint32_t w0 = ld_word(ra);
#pragma unroll 4
                for (; j < uw4; j += 4) {
                    const uint32_t w1 = ld_word(ra + j + 4);
                    ewalk(ld_word(rx + j), bytes_at<2>(w0, w1));
                    w0 = w1;
                }
            }
            for (; j < uw; ++j) {
                const int xv = rx[j], e = xv - (int)rd[j];
                sx += xv;
                if (j >= jr) e_rgt += e * e;
                else e_in += e * e;
            }
        } else {
            const int16_t *xr = X + (i - xi0) * kMaxUnitW;
            for (; j < uw; ++j) {
                const int xv = xr[j], e = xv - Dat(i, j);
                sx += xv;
                if (j >= jr) e_rgt += e * e;
                else e_in += e * e;
            }
        }
        if constexpr (WIN == 5) {
            const bool bottom = i >= uh - uh % 16;
            Erow[i - xi0][0] = sx;
            Erow[i - xi0][1] = bottom ? 0u : e_in;
            Erow[i - xi0][2] = e_rgt;
            Erow[i - xi0][3] = bottom ? e_in : 0u;
        } else {
            atomicAdd(&Es[0], (unsigned long long)sx);
            atomicAdd(&Es[i >= uh - uh % 16 ? 3 : 1], (unsigned long long)e_in);
            atomicAdd(&Es[2], (unsigned long long)e_rgt);
        }
    }
    __syncthreads();
    // The row sums of each (dr, dc, ca) are added over the CTA's rows in
    // shared memory (D is no longer read), then one atomic per H entry (per
    // vertical shift when some row of the CTA lies within HALF of the unit's
    // top or bottom, where a row reaches only some shifts).
    // RS[(row * NDR + dr index) * NE + e], e enumerating (dc, ca) with
    // ca + dc < WIN.
    {
        constexpr int NE = WIN * (WIN + 1) / 2;
        static_assert(G::ROWS * G::NDR * NE * 4 <= G::DROWS * G::DCOLS * 2, "row-sum buffer fits in D");
        int *RS = reinterpret_cast<int *>(D);
        if (keep) {
            int e = 0;
#pragma unroll
            for (int dc = 0; dc < WIN; ++dc)
#pragma unroll
                for (int ca = 0; ca + dc < WIN; ++ca) RS[t * NE + e++] = rs[dc][ca];
        }
        if constexpr (WIN == 5) {
            // the row slots of the (row, window row) and sse walks: 25 Mr
            // entries, 25 shift sums, 4 sse / source sums, over the unit rows
            // of this CTA, in four interleaved parts of the rows (short
            // chains of loads and adds on many threads), added after the
            // barrier (each entry of Ms / Ss / Es is written there only)
            const int nr = xi1 - xi0;
            if (t < 4 * kSlotSums) {
                const int part = t / kSlotSums, q = t - part * kSlotSums;
                long long a = 0;
                for (int r = part; r < nr; r += 4)
                    a += q < WIN2 ? (long long)Mrow[r][q] : q < 2 * WIN2 ? (long long)Srow[r][q - WIN2]
                                                                         : (long long)Erow[r][q - 2 * WIN2];
                slot_part[part][q] = a;
            }
        }
        __syncthreads();
        if constexpr (WIN == 5) {
            if (t < kSlotSums) {
                const unsigned long long a = (unsigned long long)(slot_part[0][t] + slot_part[1][t] + slot_part[2][t] +
                                                                  slot_part[3][t]);
                if (t < WIN2) Ms[t] = a;
                else if (t < 2 * WIN2) Ss[t - WIN2] = a;
                else Es[t - 2 * WIN2] = a;
            }
        }
        // every (dr, dc, ca) and window row ra below is a distinct H entry
        // (ia, ib) -- (ca, ra) and (ca + dc, ra + dr) give back all four --
        // so each entry of Hs has one writer here and takes a plain add
        for (int q = t; q < G::NDR * NE; q += blockDim.x) {
            const int dri = q / NE, dr = dri - (WIN - 1);
            int e = q - dri * NE, dc = 0;
            while (e >= WIN - dc) {
                e -= WIN - dc;
                ++dc;
            }
            const int ca = e;
            if (dr < 0 && dc == 0) continue;
            const int ra0 = max(0, -dr), ra1 = min(WIN, WIN - dr);
            if (all_interior) {  // every vertical shift holds every row
                long long acc = 0;
                for (int r = 0; r < y1 - y0; ++r) acc += RS[(r * G::NDR + dri) * NE + (q - dri * NE)];
                if (acc == 0) continue;
                for (int ra = ra0; ra < ra1; ++ra) {
                    const int ia = ca * WIN + ra, ib = (ca + dc) * WIN + ra + dr;
                    Hs[ia * WIN2 + ib] += (unsigned long long)acc;
                }
            } else {  // a row adds to the vertical shifts sr = ra - HALF whose window [sr, sr + uh) holds it
                long long acc[WIN];
#pragma unroll
                for (int k = 0; k < WIN; ++k) acc[k] = 0;
                for (int r = 0; r < y1 - y0; ++r) {
                    const long long v = RS[(r * G::NDR + dri) * NE + (q - dri * NE)];
                    const int y = y0 + r;
#pragma unroll
                    for (int ra = 0; ra < WIN; ++ra)
                        if (ra >= ra0 && ra < ra1 && y >= ra - HALF && y < ra - HALF + uh) acc[ra] += v;
                }
#pragma unroll
                for (int ra = 0; ra < WIN; ++ra) {
                    if (ra < ra0 || ra >= ra1 || acc[ra] == 0) continue;
                    const int ia = ca * WIN + ra, ib = (ca + dc) * WIN + ra + dr;
                    Hs[ia * WIN2 + ib] += (unsigned long long)acc[ra];
                }
            }
        }
    }
    __syncthreads();
    for (int q = threadIdx.x; q < WIN2 * WIN2; q += blockDim.x) {
        const int ia = q / WIN2, ib = q - ia * WIN2;
        if (ib >= ia && Hs[q]) atomicAdd((unsigned long long *)&u.h[q], Hs[q]);
    }
    if (threadIdx.x < WIN2) {
        if (Ms[threadIdx.x]) atomicAdd((unsigned long long *)&u.m[threadIdx.x], Ms[threadIdx.x]);
        if (Ss[threadIdx.x]) atomicAdd((unsigned long long *)&u.s[threadIdx.x], Ss[threadIdx.x]);
    }
    if (threadIdx.x < 4 && Es[threadIdx.x]) {
        unsigned long long *dst = threadIdx.x == 0 ? (unsigned long long *)&u.sum_src
                                : threadIdx.x == 1 ? &u.sse_blk : threadIdx.x == 2 ? &u.sse_rgt : &u.sse_bot;
        atomicAdd(dst, Es[threadIdx.x]);
    }
}

// ---------------------------------------------------------------------------
// 2. Solve: wiener_decompose_sep_sym + finalize_sym_filter + compute_score
// (restoration.rs:801-1056), one CTA per unit. The update_{a,b} sums are
// sums of independently truncated terms, so threads split the terms and the
// bins are reduced exactly.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int wrap_index(int i, int win) {
    const int h1 = (win >> 1) + 1;
    return i >= h1 ? win - 1 - i : i;
}

// linsolve_wiener (restoration.rs:801-846) for N unknowns in registers
// (N = 2 for the 5-tap window, 3 for the 7-tap one): the same pivoting and
// the same truncating divisions in the same order; independent divisions
// of one elimination step interleave in the instruction stream.
template <int N>
__device__ __forceinline__ bool linsolve_reg(int64_t (&a)[N][N], int64_t (&b)[N], int32_t (&x)[N]) {
#pragma unroll
    for (int k = 0; k < N - 1; ++k) {
#pragma unroll
        for (int i = N - 1; i >= k + 1; --i) {
            const int64_t u = a[i - 1][k], v = a[i][k];
            if ((u < 0 ? -u : u) < (v < 0 ? -v : v)) {
#pragma unroll
                for (int j = 0; j < N; ++j) {
                    const int64_t t = a[i][j];
                    a[i][j] = a[i - 1][j];
                    a[i - 1][j] = t;
                }
                const int64_t t = b[i];
                b[i] = b[i - 1];
                b[i - 1] = t;
            }
        }
        const int64_t cd = a[k][k];
        if (cd == 0) return false;
#pragma unroll
        for (int i = k; i < N - 1; ++i) {
            const int64_t c = a[i + 1][k];
#pragma unroll
            for (int j = 0; j < N; ++j) a[i + 1][j] -= c / 256 * a[k][j] / cd * 256;
            b[i + 1] -= c * b[k] / cd;
        }
    }
#pragma unroll
    for (int i = N - 1; i >= 0; --i) {
        if (a[i][i] == 0) return false;
        int64_t c = 0;
#pragma unroll
        for (int j = i + 1; j < N; ++j) c += a[i][j] * (int64_t)x[j] / kTapScale;
        x[i] = (int32_t)(kTapScale * (b[i] - c) / a[i][i]);
    }
    return true;
}

// normalize_and_solve (restoration.rs:913-941) in registers, one thread;
// `out` (WIN taps) is written only when the system solves.
template <int WIN>
__device__ __forceinline__ void normalize_and_solve_reg(int64_t (&av)[WIN / 2 + 1], int64_t (&bv)[WIN / 2 + 1][WIN / 2 + 1],
                                                        int32_t *out) {
    constexpr int H1 = WIN / 2 + 1, N = H1 - 1;
    const int64_t ah = av[H1 - 1], bc = bv[H1 - 1][H1 - 1];
    int64_t a[N][N], b[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
        b[i] = av[i] - (ah * 2 + bv[i][H1 - 1] - 2 * bc);
#pragma unroll
        for (int j = 0; j < N; ++j) a[i][j] = bv[i][j] - 2 * (bv[i][H1 - 1] + bv[H1 - 1][j] - 2 * bc);
    }
    int32_t x[N];
#pragma unroll
    for (int i = 0; i < N; ++i) x[i] = 0;
    if (!linsolve_reg<N>(a, b, x)) return;
    int32_t sv[WIN];
#pragma unroll
    for (int i = 0; i < N; ++i) sv[i] = x[i];
    sv[H1 - 1] = (int32_t)kTapScale;
#pragma unroll
    for (int i = H1; i < WIN; ++i) {
        sv[i] = sv[WIN - 1 - i];
        sv[H1 - 1] -= 2 * sv[i];
    }
#pragma unroll
    for (int i = 0; i < WIN; ++i) out[i] = sv[i];
}

// Block-wide int64 sum of `n` per-thread bins into out[] (thread 0 valid).
template <int NB>
__device__ void reduce_bins(int64_t (&bins)[NB], int n, int64_t *out) {
    __shared__ unsigned long long sb[NB];
    for (int k = threadIdx.x; k < n; k += blockDim.x) sb[k] = 0;
    __syncthreads();
    for (int k = 0; k < n; ++k) {
        unsigned long long v = (unsigned long long)bins[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&sb[k], v);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += blockDim.x) out[k] = (int64_t)sb[k];
    __syncthreads();
}

// One update_{a,b}_sep_sym (restoration.rs:849-909) for a WIN-tap window
// on a 128-thread CTA. `upd_a` selects which factor is solved; `fix` is the
// other one. Every bin is a sum of independently truncated terms, so the
// order of the sum is free: a thread owns one bin pair q (the (k, l) of
// update_a, the (i, j) of update_b) and a slice of the other pair index and
// leaves its partial in `part` (plus one partial per av term); lanes of warp
// 0 add the partials of one bin each (binq lists the pairs of a bin; no
// atomics) and lane 0 solves in registers.
template <int WIN>
__device__ __forceinline__ void update_sep_sym(bool upd_a, const int64_t *M, const int64_t *H, const int32_t *fix,
                                               int32_t *outv, int64_t *part, int64_t *binv,
                                               const int8_t (*binq)[4]) {
    constexpr int W2 = WIN * WIN, H1 = WIN / 2 + 1, R = 128 / W2, NPP = (W2 + R - 1) / R;
    const int t = threadIdx.x;
    if (t < R * W2) {
        const int q = t % W2, sl = t / W2;
        const int qa = q / WIN, qb = q - qa * WIN;
        int64_t acc = 0;
#pragma unroll
        for (int k = 0; k < NPP; ++k) {
            const int pp = sl + k * R;
            if (pp < W2) {
                const int pa = pp / WIN, pb = pp - pa * WIN;
                // update_a: (i, j) = (pa, pb), (k, l) = (qa, qb); update_b:
                // (i, j) = (qa, qb), (k, l) = (pa, pb); factors from `fix`
                const int64_t hv = upd_a ? H[pb * WIN * W2 + pa * WIN + qa * W2 + qb]
                                         : H[qa * WIN * W2 + qb * WIN + pa * W2 + pb];
                acc += hv * (int64_t)fix[pa] / kTapScale * (int64_t)fix[pb] / kTapScale;
            }
        }
        part[t] = acc;
    }
    if (t < WIN) {  // av terms: t is j (update_a) or i (update_b)
        int64_t acc = 0;
#pragma unroll
        for (int o = 0; o < WIN; ++o)
            acc += (upd_a ? M[o * WIN + t] : M[t * WIN + o]) * (int64_t)fix[o] / kTapScale;
        part[R * W2 + t] = acc;
    }
    __syncthreads();
    if (t < 32) {
        // lane t < H1^2: matrix bin t (wrap(qb) = t / H1, wrap(qa) = t % H1);
        // lane H1^2 + a: vector bin a (wrap(term) = a)
        if (t < H1 * H1 + H1) {
            const bool vec = t >= H1 * H1;
            const int row = vec ? 16 + t - H1 * H1 : t;
            int64_t sum = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int q = binq[row][k];
                if (q < 0) continue;
                if (vec) sum += part[R * W2 + q];
                else
#pragma unroll
                    for (int sl = 0; sl < R; ++sl) sum += part[sl * W2 + q];
            }
            binv[t] = sum;
        }
        __syncwarp();
        if (t == 0) {
            int64_t av[H1], bv[H1][H1];
#pragma unroll
            for (int i = 0; i < H1; ++i) {
                av[i] = binv[H1 * H1 + i];
#pragma unroll
                for (int j = 0; j < H1; ++j) bv[i][j] = binv[i * H1 + j];
            }
            normalize_and_solve_reg<WIN>(av, bv, outv);
        }
    }
    __syncthreads();
}

__device__ void finalize_sym(int win, const int32_t *f, int16_t *fi) {
    const int half = win >> 1;
    for (int i = 0; i < half; ++i) {
        const int64_t d = (int64_t)f[i] * kStep, q = kTapScale;
        fi[i] = (int16_t)(d < 0 ? (d - q / 2) / q : (d + q / 2) / q);
    }
    if (win == 7) {
        fi[0] = (int16_t)clampi(fi[0], -5, 10);
        fi[1] = (int16_t)clampi(fi[1], -23, 8);
        fi[2] = (int16_t)clampi(fi[2], -17, 46);
    } else {
        fi[2] = (int16_t)clampi(fi[1], -17, 46);
        fi[1] = (int16_t)clampi(fi[0], -23, 8);
        fi[0] = 0;
    }
    fi[6] = fi[0];
    fi[5] = fi[1];
    fi[4] = fi[2];
    fi[3] = (int16_t)(-2 * (fi[0] + fi[1] + fi[2]));
    fi[7] = 0;
}

// One unit's solve (the WIN-tap window), 128 threads.
template <int WIN>
__device__ __forceinline__ void solve_unit(const FrameDesc &f, const LrPlane &pl, int unit) {
    constexpr int W2 = WIN * WIN, H1 = WIN / 2 + 1, R = 128 / W2;
    __shared__ int64_t H[W2 * W2];
    __shared__ int64_t M[W2], Sv[W2];
    __shared__ int32_t a[WIN], b[WIN];
    __shared__ int64_t spart[128 + 8];
    __shared__ int64_t binv[H1 * H1 + H1];
    __shared__ int8_t binq[20][4];
    __shared__ int16_t vf[8], hf[8];
    __shared__ int32_t ab[W2];
    static_assert(R * W2 + WIN <= 128 + 8, "partials fit");
    LrUnit &u = pl.units[unit];
    const int t = threadIdx.x;
    // The raw-sample sums corrected by the unit average A = find_average
    // (restoration.rs:198: the centre shift sum over the pixel count), then
    // the bit-depth divider on M and the upper triangle (truncating division
    // by 4 at 10 bits, written as a shift with the sign correction), then
    // mirrored (compute_stats_hbd, restoration.rs:1799-1806).
    const bool hbd = f.bd == 10;
    auto divd = [hbd](int64_t v) { return hbd ? (v + ((v >> 63) & 3)) >> 2 : v; };
    const UnitRect rc = pl.rects[unit];
    const int64_t n = (int64_t)(rc.h_end - rc.h_start) * (rc.v_end - rc.v_start);
    constexpr int ctr = (WIN / 2) * WIN + WIN / 2;
    const int64_t A = (int64_t)((unsigned long long)u.s[ctr] / (unsigned long long)n), nAA = n * A * A;
    if (t < W2) {
        Sv[t] = u.s[t];
        M[t] = divd(u.m[t] - A * (u.s[t] + u.sum_src) + nAA);
    }
    // bins of update_sep_sym: matrix bin a * H1 + b holds the pairs q =
    // qa * WIN + qb with wrap(qb) = a, wrap(qa) = b (at most 4); vector bin a
    // (row 16 + a) the terms o with wrap(o) = a (at most 2)
    if (t < 20) {
        int nq = 0;
        int8_t lst[4] = {-1, -1, -1, -1};
        if (t < H1 * H1) {
            const int ra = t / H1, rb = t - ra * H1;
            for (int qa = 0; qa < WIN; ++qa)
                for (int qb = 0; qb < WIN; ++qb)
                    if (wrap_index(qb, WIN) == ra && wrap_index(qa, WIN) == rb && nq < 4)
                        lst[nq++] = (int8_t)(qa * WIN + qb);
        } else if (t >= 16 && t < 16 + H1) {
            for (int o = 0; o < WIN; ++o)
                if (wrap_index(o, WIN) == t - 16 && nq < 4) lst[nq++] = (int8_t)o;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) binq[t][k] = lst[k];
    }
    if (t == 0) {
        if (f.bd == 8) u.sse_none = (int64_t)(u.sse_blk + u.sse_rgt + u.sse_bot);
        else u.sse_none = (int64_t)u.sse_blk + (int64_t)(uint32_t)u.sse_rgt + (int64_t)(uint32_t)u.sse_bot;
        constexpr int off = (7 - WIN) >> 1;
        const int init[7] = {3, -7, 15, kStep - 2 * (3 - 7 + 15), 15, -7, 3};
#pragma unroll
        for (int i = 0; i < WIN; ++i) {
            a[i] = (int32_t)(kTapScale / kStep) * init[i + off];
            b[i] = a[i];
        }
    }
    __syncthreads();
    // H in chunks of five entries per thread, the loads issued first
    for (int t0 = 0; t0 < W2 * W2; t0 += 5 * 128) {
        int64_t hv[5];
#pragma unroll
        for (int c = 0; c < 5; ++c) {
            const int q = t0 + c * 128 + t;
            hv[c] = q < W2 * W2 ? u.h[q] : 0;
        }
#pragma unroll
        for (int c = 0; c < 5; ++c) {
            const int q = t0 + c * 128 + t;
            if (q >= W2 * W2) break;
            const int k = q / W2, l = q - k * W2;
            if (l >= k) {
                const int64_t v = divd(hv[c] - A * (Sv[k] + Sv[l]) + nAA);
                H[q] = v;
                H[l * W2 + k] = v;
            }
        }
    }
    __syncthreads();
    for (int round = 1; round < 5; ++round) {
        update_sep_sym<WIN>(true, M, H, b, a, spart, binv, binq);
        update_sep_sym<WIN>(false, M, H, a, b, spart, binv, binq);
    }
    if (t == 0) {
        for (int i = 0; i < 8; ++i) {
            vf[i] = 0;
            hf[i] = 0;
        }
        finalize_sym(WIN, a, vf);
        finalize_sym(WIN, b, hf);
        for (int i = 0; i < 7; ++i) {
            u.vd[i] = i < WIN ? a[i] : 0;
            u.hd[i] = i < WIN ? b[i] : 0;
        }
        for (int i = 0; i < 8; ++i) {
            u.vf[i] = vf[i];
            u.hf[i] = hf[i];
        }
    }
    __syncthreads();
    // compute_score (restoration.rs:1009-1056): ab[k * WIN + l] = av[l + off]
    // * bv[k + off], av / bv the symmetric 7-tap filters of vf / hf (centre
    // 128 - 2 * the others).
    if (t < W2) {
        constexpr int off = (7 - WIN) >> 1;
        auto tap7 = [](const int16_t *fl, int i) -> int32_t {
            return i == 3 ? (int16_t)(kStep - 2 * (fl[0] + fl[1] + fl[2])) : fl[i < 3 ? i : 6 - i];
        };
        const int k = t / WIN, l = t - k * WIN;
        ab[t] = tap7(vf, l + off) * tap7(hf, k + off);
    }
    __syncthreads();
    int64_t bins[2] = {0, 0};
    if (t < W2) bins[0] = (int64_t)ab[t] * M[t] / kStep / kStep;
    for (int q = t; q < W2 * W2; q += 128) {
        const int k = q / W2, l = q - k * W2;
        bins[1] += (int64_t)ab[k] * H[q] * (int64_t)ab[l] / kStep / kStep / kStep / kStep;
    }
    __shared__ int64_t pq[2];
    reduce_bins<2>(bins, 2, pq);
    if (t == 0) {
        const int64_t score = pq[1] - 2 * pq[0];
        const int64_t ip = M[W2 >> 1], iq = H[(W2 >> 1) * W2 + (W2 >> 1)];
        u.score = score - (iq - 2 * ip);
    }
}

// items: a = unit. One CTA (128 threads) per unit.
__global__ void __launch_bounds__(128) k_lr_solve(FrameDesc *frames, const WorkItem *items, int nitems) {
    const WorkItem wi = items[blockIdx.x];
    const FrameDesc &f = frames[wi.frame];
    const LrPlane &pl = f.lr[wi.plane];
    if (pl.win == 5) solve_unit<5>(f, pl, wi.a);
    else solve_unit<7>(f, pl, wi.a);
}

// ---------------------------------------------------------------------------
// 3. Trial filter + SSE (try_restoration_unit, restoration.rs:472-507) and
// the refinement hill-climb (finer_tile_search_wiener, :513-636). One CTA
// per unit.
// ---------------------------------------------------------------------------
constexpr int TT_W = 64, TT_H = 32;

struct Taps {
    int16_t v[8], h[8];
};

// Horizontal then vertical pass of wiener_convolve_add_src[_hbd] for one
// output pixel column tile; `row_src(r)` yields the data row pointer
// (already clamped / substituted) in plane coordinates.
__device__ __forceinline__ int wiener_h(const int *px, const int16_t *hf, int bd) {
    int sum = (px[3] << 7) + (1 << (bd + 7 - 1));
#pragma unroll
    for (int k = 0; k < 8; ++k) sum += px[k] * hf[k];
    const int lim = (1 << (bd + 1 + 7 - 3)) - 1;
    return clampi((sum + 4) >> 3, 0, lim);
}
__device__ __forceinline__ int wiener_v(const int *tp, const int16_t *vf, int bd) {
    int sum = (tp[3] << 7) - (1 << (bd + 11 - 1));
#pragma unroll
    for (int k = 0; k < 8; ++k) sum += tp[k] * vf[k];
    return clampi((sum + (1 << 10)) >> 11, 0, (1 << bd) - 1);
}

// SSE of the unit filtered with `t` against the source; three parts as in
// sse_region_hbd. Returns the combined value (every thread gets it).
// The refinement trial runs on a cluster of kTrialCluster CTAs per unit:
// CTA `rank` owns tiles rank, rank + CL, ... of the unit. It stages their
// dgd windows and source tiles in shared memory once, before the first
// trial (the samples do not change between trials, only the taps), so a
// trial is the two filter passes over shared memory: the horizontal pass of
// tile k and the vertical pass of tile k - 1 share one barrier (two
// horizontal-pass buffers). The partial SSE parts are pushed into every
// rank's inbox (double-buffered) before one cluster barrier, and every CTA
// forms the same total, so the hill-climb decisions stay identical across
// the cluster.
constexpr int kTrialCluster = 8;
constexpr int TRIAL_SW = TT_W + 8, TRIAL_SH = TT_H + 7;  // staged window rows 8-byte aligned
constexpr int TRIAL_WIN = TRIAL_SH * TRIAL_SW, TRIAL_SRC = TT_H * TT_W, TRIAL_TMP = TRIAL_SH * TT_W;

// With at most kTrialCacheTiles tiles per CTA every tile keeps its own
// horizontal-pass buffer: the trials of the vertical taps (the second
// refinement pass) leave the horizontal taps alone, so they reuse it and run
// only the vertical pass. Above that the CTA keeps two buffers, alternating.
constexpr int kTrialCacheTiles = 5;
struct TrialTiles {
    const uint16_t *win, *src;  // [n][TRIAL_WIN], [n][TRIAL_SRC]
    uint16_t *tmp;              // [n][TRIAL_TMP] when cached, else [2][TRIAL_TMP]
    int n, ntx, rank, CL;
    bool cached;
};

// do_h: run the horizontal pass (always when the buffers are not cached;
// when they are, a trial whose horizontal taps equal those of the buffers'
// last pass may skip it).
__device__ int64_t trial_sse(const FrameDesc &f, const UnitRect &r, const Taps &t, const TrialTiles &T,
                             unsigned long long *red, unsigned long long (*inbox)[kTrialCluster][3], int &buf,
                             bool do_h = true) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const int bd = f.bd;
    const int uw = r.h_end - r.h_start, uh = r.v_end - r.v_start;
    const int dw = uw % 16, dh = uh % 16;
    // The taps are symmetric (f[6 - k] = f[k], f[7] = 0: the solve and every
    // refinement step keep them so), so each pass is four multiplies per
    // output on pair sums, the centre tap carrying the 128 of
    // wiener_convolve_add_src; a thread takes four outputs per pass. With
    // both outer taps 0 (every 5-tap window: the refinement starts at tap 1)
    // the outer pair is dropped.
    int hf[4], vf[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        hf[k] = t.h[k];
        vf[k] = t.v[k];
    }
    const bool t5 = hf[0] == 0 && vf[0] == 0;  // uniform over the cluster
    const int hc3 = 128 + hf[3], hoff = 1 << (bd + 6), hlim = (1 << (bd + 5)) - 1;
    const int vc3 = 128 + vf[3], voff = -(1 << (bd + 10)), vmax = (1 << bd) - 1;
    uint32_t blk = 0, rgt = 0, bot = 0;  // a thread's parts of one trial: <= 9 tiles x 8 pixels of e^2 <= 1023^2
    // cached buffers: every tile's horizontal pass (unless skipped), one
    // barrier, then every tile's vertical pass; else the horizontal pass of
    // tile k and the vertical pass of tile k - 1 share a barrier
    const int hk = T.cached ? T.n : 1;  // tiles per phase
    const int nphase = T.cached ? (do_h ? 2 : 1) : T.n + 1;
    for (int ph = 0; ph < nphase; ++ph) {
        const int kh0 = T.cached ? (do_h && ph == 0 ? 0 : T.n) : ph;        // horizontal tiles [kh0, kh0 + hk)
        const int kv0 = T.cached ? (do_h && ph == 0 ? T.n : 0) : ph - 1;    // vertical tiles [kv0, kv0 + hk)
        for (int k = kh0; k < min(kh0 + hk, T.n); ++k) {
            // horizontal pass of tile k: every staged row x 16 runs of four columns
            const int tile = T.rank + k * T.CL;
            const int tw = min(TT_W, uw - (tile % T.ntx) * TT_W);
            const uint16_t *stage = T.win + k * TRIAL_WIN;
            uint16_t *tmp = T.tmp + (T.cached ? k : (k & 1)) * TRIAL_TMP;
            for (int q = threadIdx.x; q < TRIAL_SH * (TT_W / 4); q += blockDim.x) {
                const int rr = q >> 4, c0 = (q & 15) * 4;
                if (c0 >= tw) continue;
                const uint2 *sp = reinterpret_cast<const uint2 *>(stage + rr * TRIAL_SW + c0);
                int p[12];
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    const uint2 w = sp[j];
                    p[4 * j] = (int)(w.x & 0xffffu);
                    p[4 * j + 1] = (int)(w.x >> 16);
                    p[4 * j + 2] = (int)(w.y & 0xffffu);
                    p[4 * j + 3] = (int)(w.y >> 16);
                }
                uint32_t o[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    int sum = p[j + 3] * hc3 + hf[1] * (p[j + 1] + p[j + 5]) + hf[2] * (p[j + 2] + p[j + 4]) + hoff;
                    if (!t5) sum += hf[0] * (p[j] + p[j + 6]);
                    o[j] = (uint32_t)clampi((sum + 4) >> 3, 0, hlim);
                }
                *reinterpret_cast<uint2 *>(tmp + rr * TT_W + c0) = make_uint2(o[0] | o[1] << 16, o[2] | o[3] << 16);
            }
        }
        for (int k = max(kv0, 0); k < min(kv0 + hk, T.n); ++k) {
            // vertical pass of tile k: four columns of one row per thread,
            // packed pair sums (tmp values are < 2^15), the SSE parts
            // against the staged source
            const int tile = T.rank + k * T.CL;
            const int ty = (tile / T.ntx) * TT_H, tx = (tile % T.ntx) * TT_W;
            const int th = min(TT_H, uh - ty), tw = min(TT_W, uw - tx);
            const uint16_t *tmp = T.tmp + (T.cached ? k : (k & 1)) * TRIAL_TMP;
            const uint16_t *srct = T.src + k * TRIAL_SRC;
            for (int q = threadIdx.x; q < th * (TT_W / 4); q += blockDim.x) {
                const int rr = q >> 4, c0 = (q & 15) * 4;
                if (c0 >= tw) continue;
                uint2 v[7];
#pragma unroll
                for (int j = 0; j < 7; ++j)
                    v[j] = (t5 && (j == 0 || j == 6)) ? make_uint2(0, 0)
                                                      : *reinterpret_cast<const uint2 *>(tmp + (rr + j) * TT_W + c0);
                const uint32_t p1x = v[1].x + v[5].x, p1y = v[1].y + v[5].y;
                const uint32_t p2x = v[2].x + v[4].x, p2y = v[2].y + v[4].y;
                const uint32_t p0x = v[0].x + v[6].x, p0y = v[0].y + v[6].y;
                auto lo = [](uint32_t w) { return (int)(w & 0xffffu); };
                auto hi = [](uint32_t w) { return (int)(w >> 16); };
                auto out = [&](int c, int a1, int a2, int a0) {
                    const int sum = c * vc3 + vf[1] * a1 + vf[2] * a2 + vf[0] * a0 + voff;
                    return clampi((sum + (1 << 10)) >> 11, 0, vmax);
                };
                const int y[4] = {out(lo(v[3].x), lo(p1x), lo(p2x), lo(p0x)),
                                  out(hi(v[3].x), hi(p1x), hi(p2x), hi(p0x)),
                                  out(lo(v[3].y), lo(p1y), lo(p2y), lo(p0y)),
                                  out(hi(v[3].y), hi(p1y), hi(p2y), hi(p0y))};
                const uint2 sv = *reinterpret_cast<const uint2 *>(srct + rr * TT_W + c0);
                const int sx[4] = {lo(sv.x), hi(sv.x), lo(sv.y), hi(sv.y)};
                const int i = ty + rr, nq = min(4, tw - c0);
                // the four columns share their sse_region part unless the
                // right strip starts inside them (a unit width not a
                // multiple of 4)
                const int xc = tx + c0, xr = uw - dw;
                uint32_t e2s = 0;
                if (xc + nq <= xr || xc >= xr) {
#pragma unroll
                    for (int jj = 0; jj < 4; ++jj) {
                        const int e = sx[jj] - y[jj];
                        e2s += jj < nq ? (uint32_t)(e * e) : 0u;
                    }
                    if (xc >= xr) rgt += e2s;
                    else if (i >= uh - dh) bot += e2s;
                    else blk += e2s;
                } else {
#pragma unroll
                    for (int jj = 0; jj < 4; ++jj) {
                        if (jj >= nq) break;
                        const int e = sx[jj] - y[jj];
                        const uint32_t e2 = (uint32_t)(e * e);
                        if (xc + jj >= xr) rgt += e2;
                        else if (i >= uh - dh) bot += e2;
                        else blk += e2;
                    }
                }
            }
        }
        __syncthreads();
    }
    unsigned long long v[3] = {blk, rgt, bot};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
        if ((threadIdx.x & 31) == 0) red[k * 8 + (threadIdx.x >> 5)] = v[k];
    }
    __syncthreads();
    __shared__ unsigned long long mine[3];
    if (threadIdx.x < 3) {
        unsigned long long s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[threadIdx.x * 8 + w];
        mine[threadIdx.x] = s;
    }
    __syncthreads();
    if (threadIdx.x < T.CL)  // this CTA's parts into rank threadIdx.x's inbox
        for (int k = 0; k < 3; ++k) *cl.map_shared_rank(&inbox[buf][T.rank][k], (int)threadIdx.x) = mine[k];
    cl.sync();
    unsigned long long sp[3] = {0, 0, 0};
    for (int q = 0; q < T.CL; ++q)
        for (int k = 0; k < 3; ++k) sp[k] += inbox[buf][q][k];
    buf ^= 1;
    return bd == 8 ? (int64_t)(sp[0] + sp[1] + sp[2])
                   : (int64_t)sp[0] + (int64_t)(uint32_t)sp[1] + (int64_t)(uint32_t)sp[2];
}

size_t lr_trial_smem(int max_tiles) {
    const int tmps = max_tiles <= kTrialCacheTiles ? max_tiles : 2;
    return ((size_t)max_tiles * (TRIAL_WIN + TRIAL_SRC) + (size_t)tmps * TRIAL_TMP) * 2;
}
__host__ __device__ int lr_trial_tiles_per_cta(int uw, int uh) {
    return (((uw + TT_W - 1) / TT_W) * ((uh + TT_H - 1) / TT_H) + kTrialCluster - 1) / kTrialCluster;
}

// max_tiles: the tiles per CTA the dynamic shared memory holds
// (lr_trial_smem); a unit needing more sets cdef_stats[3] bit 2 and is
// skipped by its whole cluster.
__global__ void __cluster_dims__(kTrialCluster, 1, 1) __launch_bounds__(256, 3)
    k_lr_trial(FrameDesc *frames, const WorkItem *items, int nitems, int max_tiles) {
    extern __shared__ __align__(16) uint16_t trial_dyn[];
    __shared__ unsigned long long red[24];
    __shared__ unsigned long long inbox[2][kTrialCluster][3];
    __shared__ Taps t;
    int buf = 0;
    const WorkItem wi = items[find_item(items, nitems, blockIdx.x)];
    FrameDesc &f = frames[wi.frame];
    const LrPlane &pl = f.lr[wi.plane];
    LrUnit &u = pl.units[wi.a];
    const UnitRect r = pl.rects[wi.a];
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const bool lead = cl.block_rank() == 0;
    if (u.score > 0) {  // uniform over the cluster (one unit)
        if (lead && threadIdx.x == 0) u.sse_wn = INT64_MAX;
        return;
    }
    const int uw = r.h_end - r.h_start, uh = r.v_end - r.v_start;
    if (lr_trial_tiles_per_cta(uw, uh) > max_tiles) {  // uniform over the cluster
        if (lead && threadIdx.x == 0) atomicOr(&f.cdef_stats[3], 4ull);
        return;
    }
    TrialTiles T;
    T.rank = (int)cl.block_rank();
    T.CL = (int)cl.num_blocks();
    T.ntx = (uw + TT_W - 1) / TT_W;
    const int ntiles = T.ntx * ((uh + TT_H - 1) / TT_H);
    T.n = T.rank < ntiles ? (ntiles - T.rank + T.CL - 1) / T.CL : 0;
    T.win = trial_dyn;
    T.src = trial_dyn + max_tiles * TRIAL_WIN;
    T.tmp = trial_dyn + max_tiles * (TRIAL_WIN + TRIAL_SRC);
    T.cached = max_tiles <= kTrialCacheTiles;  // uniform over the launch
    {
        const int bd = f.bd, stride = plane_stride(f, wi.plane);
        const uint8_t *dg = f.A[wi.plane], *sr = f.S[wi.plane];
        for (int k = 0; k < T.n; ++k) {
            const int tile = T.rank + k * T.CL;
            const int ty = (tile / T.ntx) * TT_H, tx = (tile % T.ntx) * TT_W;
            const int y0 = r.v_start + ty, x0 = r.h_start + tx;
            const int th = min(TT_H, uh - ty), tw = min(TT_W, uw - tx);
            uint16_t *stage = trial_dyn + k * TRIAL_WIN, *srct = trial_dyn + max_tiles * TRIAL_WIN + k * TRIAL_SRC;
            stage_window<4>(
                bd, pl.pw, TRIAL_SH, x0 - 3, TT_W + 7, true, 0,
                [&](int rr) { return row_ptr(dg, clampi(y0 - 3 + rr, 0, pl.ph - 1), stride, bd); },
                [&](int rr, int cc, int v) { stage[rr * TRIAL_SW + cc] = (uint16_t)v; });
            stage_window<4>(
                bd, pl.pw, th, x0, tw, true, 0, [&](int rr) { return row_ptr(sr, y0 + rr, stride, bd); },
                [&](int rr, int cc, int v) { srct[rr * TT_W + cc] = (uint16_t)v; });
        }
    }
    if (threadIdx.x < 8) {
        t.v[threadIdx.x] = u.vf[threadIdx.x];
        t.h[threadIdx.x] = u.hf[threadIdx.x];
    }
    __syncthreads();
    int64_t err = trial_sse(f, r, t, T, red, inbox, buf);
    if (pl.refine) {
        // use_refinement with max_one_refinement_step: one step size (4).
        const int plane_off = (7 - pl.win) >> 1;
        const int tap_min[3] = {-5, -23, -17}, tap_max[3] = {10, 8, 46};
        const int s = 4;
        for (int pass = 0; pass < 2; ++pass) {
            // the second pass changes vertical taps only: with cached
            // buffers its first trial runs the horizontal pass with the
            // horizontal taps the first pass settled on, the rest reuse it
            bool h_ready = false;
            for (int p = plane_off; p < 3; ++p) {
                bool skip = false;
                // minus direction
                int16_t *fp = pass == 0 ? t.h : t.v;
                if (fp[p] - s >= tap_min[p]) {
                    __syncthreads();
                    if (threadIdx.x == 0) {
                        fp[p] -= s;
                        fp[6 - p] -= s;
                        fp[3] += 2 * s;
                    }
                    __syncthreads();
                    const int64_t e2 = trial_sse(f, r, t, T, red, inbox, buf, !(T.cached && pass == 1 && h_ready));
                    h_ready = h_ready || pass == 1;
                    if (e2 > err) {
                        __syncthreads();
                        if (threadIdx.x == 0) {
                            fp[p] += s;
                            fp[6 - p] += s;
                            fp[3] -= 2 * s;
                        }
                        __syncthreads();
                    } else {
                        err = e2;
                        skip = true;
                    }
                }
                if (skip) break;
                // plus direction
                if (fp[p] + s <= tap_max[p]) {
                    __syncthreads();
                    if (threadIdx.x == 0) {
                        fp[p] += s;
                        fp[6 - p] += s;
                        fp[3] -= 2 * s;
                    }
                    __syncthreads();
                    const int64_t e2 = trial_sse(f, r, t, T, red, inbox, buf, !(T.cached && pass == 1 && h_ready));
                    h_ready = h_ready || pass == 1;
                    if (e2 > err) {
                        __syncthreads();
                        if (threadIdx.x == 0) {
                            fp[p] -= s;
                            fp[6 - p] -= s;
                            fp[3] += 2 * s;
                        }
                        __syncthreads();
                    } else {
                        err = e2;
                    }
                }
            }
        }
    }
    __syncthreads();
    if (lead && threadIdx.x == 0) {
        u.sse_wn = err;
        for (int i = 0; i < 8; ++i) {
            u.vf[i] = t.v[i];
            u.hf[i] = t.h[i];
        }
    }
}

// Trial SSE without refinement (presets >= 4), split over the unit's 64x64
// tiles so that every unit's filter runs on many SMs at once: one CTA per
// tile (items: a = unit, one item per unit, CTA offset = tile index in
// raster order), the three sse_region parts accumulate into the unit and
// k_lr_finish combines them.
//
// When the plane's trial output is kept (trial_out), the tile also writes
// the apply's pixels (apply_restoration_frame, restoration.rs:992-1052)
// into C. They equal the trial's except within 3 rows of an interior stripe
// edge b (stripes of 64 rows, the first 8 shorter, halved for chroma), where
// the apply reads the post-deblock lines that save_lr_boundaries keeps: the
// upper stripe's rows b-3..b-1 take B[b] and B[min(b+1, ph-1)] in place of
// rows >= b, the lower stripe's rows b..b+2 take B[b-1] and B[b-2] in place
// of rows < b. Those four B rows per edge are staged and filtered with the
// tile's rows, so C ends final for a Wiener unit.
constexpr int kTileEdges = 3;  // stripe edges whose rows can meet a tile of <= 64 rows (stripes >= 32 rows)

// TL: tile edge (32 or 64), a launch setting (zf_tune.trial_tile).
template <int TL>
__global__ void __launch_bounds__(256) k_lr_trial_tiles(FrameDesc *frames, const WorkItem *items, int nitems) {
    constexpr int QPR = TL / 4, LQ = TL == 64 ? 4 : 3;  // four-sample runs per row, log2
    // staged rows of TL + 7 samples at a pitch of TL + 8 (8-byte aligned
    // rows: the horizontal pass reads each run with three 8-byte loads)
    constexpr int SW = TL + 8, SR = TL + 7 + 4 * kTileEdges;
    __shared__ __align__(16) uint16_t stage[SR * SW];
    __shared__ __align__(16) uint16_t tmp[SR * TL];
    __shared__ __align__(16) uint16_t srct[TL * TL];
    __shared__ unsigned long long red[24];
    const int it = find_item(items, nitems, blockIdx.x);
    const WorkItem wi = items[it];
    const FrameDesc &f = frames[wi.frame];
    const LrPlane &pl = f.lr[wi.plane];
    LrUnit &u = pl.units[wi.a];
    if (u.score > 0) return;  // the unit reverts to NONE: no trial
    const UnitRect r = pl.rects[wi.a];
    const int bd = f.bd, stride = plane_stride(f, wi.plane);
    const int uw = r.h_end - r.h_start, uh = r.v_end - r.v_start;
    const int dw = uw % 16, dh = uh % 16;
    const int ntx = (uw + TL - 1) / TL;
    const int tile = blockIdx.x - wi.cta_begin;
    const int ty = (tile / ntx) * TL, tx = (tile % ntx) * TL;
    const int th = min(TL, uh - ty), tw = min(TL, uw - tx);
    const int y0 = r.v_start + ty, x0 = r.h_start + tx;
    int16_t hf[8], vf[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        hf[k] = u.hf[k];
        vf[k] = u.vf[k];
    }
    const uint8_t *dg = f.A[wi.plane], *sr = f.S[wi.plane], *pre = f.B[wi.plane];
    const bool tout = pl.trial_out != 0;
    uint8_t *outp = f.C[wi.plane];
    const int ph = pl.ph;
    // interior stripe edges whose rows b - 3 .. b + 2 meet the tile
    int eb[kTileEdges], ne = 0;
#pragma unroll
    for (int e = 0; e < kTileEdges; ++e) eb[e] = INT_MIN / 2;
    if (tout) {
        const int ssh = wi.plane ? 1 : 0, full = 64 >> ssh, soff = 8 >> ssh;
        for (int si = max(1, (y0 - 3 + soff) / full); ne < kTileEdges; ++si) {
            const int b = si * full - soff;
            if (b >= ph || b - 3 >= y0 + th) break;
            if (b + 3 <= y0) continue;
#pragma unroll
            for (int e = 0; e < kTileEdges; ++e)
                if (e == ne) eb[e] = b;
            ++ne;
        }
    }
    const int na = th + 7, rows = na + 4 * ne;  // A rows, then per edge B[b-2], B[b-1], B[b], B[min(b+1, ph-1)]
    // the staging compiled once with the bit depth a constant for 8-bit
    // planes (samples per word resolved at compile time), once for others
    auto stage_all = [&](const int bdc) {
        stage_window(
            bdc, pl.pw, rows, x0 - 3, tw + 7, true, 0,
            [&](int rr) {
                if (rr < na) return row_ptr(dg, clampi(y0 - 3 + rr, 0, ph - 1), stride, bdc);
                const int e = (rr - na) >> 2, k = (rr - na) & 3;
                const int b = e == 0 ? eb[0] : e == 1 ? eb[1] : eb[2];
                return row_ptr(pre, k < 3 ? b - 2 + k : min(b + 1, ph - 1), stride, bdc);
            },
            [&](int rr, int cc, int v) { stage[rr * SW + cc] = (uint16_t)v; });
        stage_window(
            bdc, pl.pw, th, x0, tw, true, 0, [&](int rr) { return row_ptr(sr, y0 + rr, stride, bdc); },
            [&](int rr, int cc, int v) { srct[rr * TL + cc] = (uint16_t)v; });
    };
    if (bd == 8) stage_all(8);
    else stage_all(bd);
    __syncthreads();
    const bool t5 = hf[0] == 0 && vf[0] == 0;  // uniform over the CTA
    // The solver's taps are symmetric (f[6 - k] = f[k], f[7] = 0), so each
    // pass is 4 multiplies per output on pair sums, the centre tap carrying
    // the 128 of wiener_convolve_add_src; a thread takes four outputs along
    // the pass from 11 staged samples.
    // horizontal: every staged row x 16 runs of four columns
    {
        // T5: the 5-tap window's outer taps are 0 (finalize_sym), so the
        // four outputs need samples 1..8 of the 11 and no outer pair
        const int c3 = 128 + hf[3], off = 1 << (bd + 6), lim = (1 << (bd + 5)) - 1;
        auto hpass = [&](auto t5c) {
            constexpr bool T5 = decltype(t5c)::value;
            for (int q = threadIdx.x; q < rows * (TL / 4); q += blockDim.x) {
                const int rr = q >> LQ, c0 = (q & (QPR - 1)) * 4;
                if (c0 >= tw) continue;
                const uint2 *sp = reinterpret_cast<const uint2 *>(stage + rr * SW + c0);
                int p[12];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const uint2 w = sp[k];
                    p[4 * k] = (int)(w.x & 0xffffu);
                    p[4 * k + 1] = (int)(w.x >> 16);
                    p[4 * k + 2] = (int)(w.y & 0xffffu);
                    p[4 * k + 3] = (int)(w.y >> 16);
                }
                uint32_t o[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    int sum = p[j + 3] * c3 + hf[1] * (p[j + 1] + p[j + 5]) + hf[2] * (p[j + 2] + p[j + 4]) + off;
                    if (!T5) sum += hf[0] * (p[j] + p[j + 6]);
                    o[j] = (uint32_t)clampi((sum + 4) >> 3, 0, lim);
                }
                *reinterpret_cast<uint2 *>(tmp + rr * TL + c0) = make_uint2(o[0] | o[1] << 16, o[2] | o[3] << 16);
            }
        };
        if (t5) hpass(std::true_type());
        else hpass(std::false_type());
    }
    // Rows of the tile the vertical pass writes (tout, not within 3 rows of
    // a stripe edge) and rows in the unit's bottom strip, as bit masks over
    // the tile's <= 64 rows (one ballot per 32 rows).
    __shared__ uint32_t s_rows[4];
    if (threadIdx.x < 64) {
        const int rr = threadIdx.x;
        bool near_edge = false;
#pragma unroll
        for (int e = 0; e < kTileEdges; ++e) near_edge |= y0 + rr >= eb[e] - 3 && y0 + rr < eb[e] + 3;
        const unsigned mw = __ballot_sync(0xffffffffu, rr < th && tout && !near_edge);
        const unsigned mb = __ballot_sync(0xffffffffu, rr < th && ty + rr >= uh - dh);
        if ((threadIdx.x & 31) == 0) {
            s_rows[threadIdx.x >> 5] = mw;
            s_rows[2 + (threadIdx.x >> 5)] = mb;
        }
    }
    __syncthreads();
    const int c3 = 128 + vf[3], voff = -(1 << (bd + 10)), vmax = (1 << bd) - 1;
    auto vert = [&](const int *p) {
        const int sum = p[3] * c3 + vf[0] * (p[0] + p[6]) + vf[1] * (p[1] + p[5]) + vf[2] * (p[2] + p[4]) + voff;
        return clampi((sum + (1 << 10)) >> 11, 0, vmax);
    };
    const uint64_t write_rows = s_rows[0] | ((uint64_t)s_rows[1] << 32);
    const uint64_t bottom_rows = s_rows[2] | ((uint64_t)s_rows[3] << 32);
    // vertical: each thread takes four adjacent columns of one row (seven
    // 8-byte loads of tmp, pair sums of two columns per 32-bit add), its
    // SSE parts and one packed store of the trial output. A thread takes at
    // most 16 pixels of a tile, each e^2 <= 1023^2, so its SSE parts fit
    // u32. tmp values are < 2^15, so two packed 16-bit lanes add without
    // carrying into each other.
    uint32_t blk32 = 0, rgt32 = 0, bot32 = 0;
    // plane rows and tile columns keep 4-sample groups word aligned when
    // the plane base is (an arena plane always is; a caller's may not be)
    const bool out_aligned = ((uintptr_t)outp & (bd == 8 ? 3u : 7u)) == 0;
    auto vpass = [&](auto t5c) {
        constexpr bool T5 = decltype(t5c)::value;
        for (int q = threadIdx.x; q < th * (TL / 4); q += blockDim.x) {
            const int rr = q >> LQ, c0 = (q & (QPR - 1)) * 4;
            if (c0 >= tw) continue;
            uint2 v[7];
#pragma unroll
            for (int k = T5 ? 1 : 0; k < (T5 ? 6 : 7); ++k)
                v[k] = *reinterpret_cast<const uint2 *>(tmp + (rr + k) * TL + c0);
            // packed pair sums (columns c0, c0 + 1 in .x; c0 + 2, c0 + 3 in .y)
            const uint32_t p1x = v[1].x + v[5].x, p1y = v[1].y + v[5].y;
            const uint32_t p2x = v[2].x + v[4].x, p2y = v[2].y + v[4].y;
            uint32_t p0x = 0, p0y = 0;
            if (!T5) {
                p0x = v[0].x + v[6].x;
                p0y = v[0].y + v[6].y;
            }
            auto lo = [](uint32_t w) { return (int)(w & 0xffffu); };
            auto hi = [](uint32_t w) { return (int)(w >> 16); };
            auto out = [&](int c, int p1, int p2, int p0) {
                int sum = c * c3 + vf[1] * p1 + vf[2] * p2 + voff;
                if (!T5) sum += vf[0] * p0;
                return clampi((sum + (1 << 10)) >> 11, 0, vmax);
            };
            int y[4];
            y[0] = out(lo(v[3].x), lo(p1x), lo(p2x), lo(p0x));
            y[1] = out(hi(v[3].x), hi(p1x), hi(p2x), hi(p0x));
            y[2] = out(lo(v[3].y), lo(p1y), lo(p2y), lo(p0y));
            y[3] = out(hi(v[3].y), hi(p1y), hi(p2y), hi(p0y));
            const int nq = min(4, tw - c0);
            if ((write_rows >> rr) & 1) {
                const int64_t o = (int64_t)(y0 + rr) * stride + x0 + c0;
                if (nq == 4 && !out_aligned) {
                    for (int j = 0; j < 4; ++j) stpx(outp, o + j, bd, y[j]);
                } else if (nq == 4 && bd == 8) {
                    *reinterpret_cast<uint32_t *>(outp + o) =
                        (uint32_t)y[0] | (uint32_t)y[1] << 8 | (uint32_t)y[2] << 16 | (uint32_t)y[3] << 24;
                } else if (nq == 4) {
                    *reinterpret_cast<uint2 *>(outp + o * 2) =
                        make_uint2((uint32_t)y[0] | (uint32_t)y[1] << 16, (uint32_t)y[2] | (uint32_t)y[3] << 16);
                } else {
                    for (int j = 0; j < nq; ++j) stpx(outp, o + j, bd, y[j]);
                }
            }
            const uint2 sv = *reinterpret_cast<const uint2 *>(srct + rr * TL + c0);
            const int sx[4] = {lo(sv.x), hi(sv.x), lo(sv.y), hi(sv.y)};
            const bool bottom = (bottom_rows >> rr) & 1;
            // the four columns share their sse_region part unless the right
            // strip starts inside them (a unit width not a multiple of 4)
            const int xc = tx + c0, xr = uw - dw;
            if (xc + nq <= xr || xc >= xr) {
                uint32_t e2s = 0;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int e = sx[j] - y[j];
                    e2s += j < nq ? (uint32_t)(e * e) : 0u;
                }
                if (xc >= xr) rgt32 += e2s;
                else if (bottom) bot32 += e2s;
                else blk32 += e2s;
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (j >= nq) break;
                    const int e = sx[j] - y[j];
                    const uint32_t e2 = (uint32_t)(e * e);
                    if (xc + j >= xr) rgt32 += e2;
                    else if (bottom) bot32 += e2;
                    else blk32 += e2;
                }
            }
        }
    };
    if (t5) vpass(std::true_type());
    else vpass(std::false_type());
    unsigned long long blk = blk32, rgt = rgt32, bot = bot32;
    // the apply's rows at the stripe edges: tmp rows of A (index y - y0 + 3)
    // or of the edge's B rows (index na + 4 e + k)
    for (int q = threadIdx.x; q < ne * 6 * TL; q += blockDim.x) {
        const int e = q / (6 * TL), k6 = (q / TL) % 6, cc = q & (TL - 1);
        const int b = e == 0 ? eb[0] : e == 1 ? eb[1] : eb[2];
        const int y = b - 3 + k6;
        if (cc >= tw || y < y0 || y >= y0 + th) continue;
        const int bb = na + 4 * e;
        int tp[7];
#pragma unroll
        for (int k = 0; k < 7; ++k) {
            const int t = y - 3 + k;
            int row;
            if (y < b) row = t < b ? t - y0 + 3 : bb + (t == b ? 2 : 3);
            else row = t < b ? bb + (t == b - 1 ? 1 : 0) : t - y0 + 3;
            tp[k] = tmp[row * TL + cc];
        }
        stpx(outp, (int64_t)y * stride + x0 + cc, bd, vert(tp));
    }
    unsigned long long v[3] = {blk, rgt, bot};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
        if ((threadIdx.x & 31) == 0) red[k * 8 + (threadIdx.x >> 5)] = v[k];
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        unsigned long long s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[threadIdx.x * 8 + w];
        if (s) atomicAdd(threadIdx.x == 0 ? &u.tw_blk : threadIdx.x == 1 ? &u.tw_rgt : &u.tw_bot, s);
    }
}

// ---------------------------------------------------------------------------
// 4. Frame RD (search_restoration_still_bd finish, restoration.rs:847-897):
// one thread per (frame, plane); reference-chained count_wiener_bits and
// RDCOST_DBL in IEEE double without contraction.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int d_msb(unsigned v) { return 31 - __clz(v); }
__device__ int recenter_nonneg(int r, int v) {
    if (v > (r << 1)) return v;
    if (v >= r) return (v - r) << 1;
    return ((r - v) << 1) - 1;
}
__device__ int recenter_finite_nonneg(int n, int r, int v) {
    if ((r << 1) <= n) return recenter_nonneg(r, v);
    return recenter_nonneg(n - 1 - r, n - 1 - v);
}
__device__ int count_quniform(int n, int v) {
    if (n <= 1) return 0;
    const int l = d_msb((unsigned)(n - 1)) + 1;
    const int m = (1 << l) - n;
    return v < m ? l - 1 : l;
}
__device__ int count_subexpfin(int n, int k, int v) {
    int count = 0, i = 0, mk = 0;
    for (;;) {
        const int b = i ? k + i - 1 : k;
        const int a = 1 << b;
        if (n <= mk + 3 * a) {
            count += count_quniform(n - mk, v - mk);
            break;
        }
        count += 1;
        if (v >= mk + a) {
            i += 1;
            mk += a;
        } else {
            count += b;
            break;
        }
    }
    return count;
}
__device__ int count_wiener_bits(int win, const int16_t *vf, const int16_t *hf, const int16_t *rvf,
                                 const int16_t *rhf) {
    auto tap = [](const int16_t *f, const int16_t *rf, int idx, int minv, int maxv, int k) {
        return count_subexpfin(maxv - minv + 1, k, recenter_finite_nonneg(maxv - minv + 1, rf[idx] - minv, f[idx] - minv));
    };
    int bits = 0;
    if (win == 7) bits += tap(vf, rvf, 0, -5, 10, 1);
    bits += tap(vf, rvf, 1, -23, 8, 2);
    bits += tap(vf, rvf, 2, -17, 46, 3);
    if (win == 7) bits += tap(hf, rhf, 0, -5, 10, 1);
    bits += tap(hf, rhf, 1, -23, 8, 2);
    bits += tap(hf, rhf, 2, -17, 46, 3);
    return bits;
}
__device__ __forceinline__ double rdcost_dbl(int64_t rdmult, int64_t rate, int64_t dist) {
    // the reference divides by 512.0: scaling by 2^-9 is exact, so the
    // multiplication gives the same double
    return __dadd_rn(__dmul_rn(__dmul_rn((double)rate, (double)rdmult), 1.0 / 512.0), __dmul_rn((double)dist, 128.0));
}

// Per-unit RD inputs staged in shared memory (count_wiener_bits reads taps
// 0..2 of each filter only).
struct RdUnit {
    int64_t sse_none, sse_wn;
    int16_t v[3], h[3];
    int16_t pick;
    int16_t thr;  // WIENER beats NONE iff the tap bits <= thr (-1: never); after the walk, the WIENER bits
};


// Frame RD of one (frame, plane) per CTA (search_restoration_still,
// restoration.rs:838-924). The unit walk is sequential only through the
// reference filter of count_wiener_bits: the last unit chosen WIENER (or the
// default taps). So every (unit k, reference j) pair -- j = -1 for the
// default, else a unit before k -- is evaluated in parallel first: the bits
// of k's taps against j's taps and whether WIENER beats NONE for k under
// that reference. The walk then only looks pairs up. Planes with more units
// than the pair table holds walk with the full evaluation per unit.
constexpr int kLrFinThreads = 1024;
constexpr int kLrPairMax = 20100;  // units <= 200 (pair table of int32 in shared memory)
constexpr int kLrPairUnits = 200;

// Bits of one tap as a table over (reference, value) for the three tap
// positions (ranges [-5, 10], [-23, 8], [-17, 46]; finalize_sym_filter and the
// refinement keep taps inside them): count_wiener_bits becomes six lookups.
constexpr int kTb0 = 16, kTb1 = 32, kTb2 = 64;
struct TapBits {
    uint8_t t0[kTb0 * kTb0], t1[kTb1 * kTb1], t2[kTb2 * kTb2];
};
__device__ void fill_tap_bits(TapBits &tb) {
    for (int q = threadIdx.x; q < kTb0 * kTb0 + kTb1 * kTb1 + kTb2 * kTb2; q += blockDim.x) {
        // entry [r * n + v]: reference tap r + minv, tap v + minv
        int n, k, rel = q;
        uint8_t *dst;
        if (rel < kTb0 * kTb0) {
            n = kTb0, k = 1, dst = tb.t0;
        } else if ((rel -= kTb0 * kTb0) < kTb1 * kTb1) {
            n = kTb1, k = 2, dst = tb.t1;
        } else {
            rel -= kTb1 * kTb1;
            n = kTb2, k = 3, dst = tb.t2;
        }
        const int r = rel / n, v = rel - r * n;
        dst[rel] = (uint8_t)count_subexpfin(n, k, recenter_finite_nonneg(n, r, v));
    }
}
__device__ __forceinline__ int count_bits_tab(const TapBits &tb, int win, const int16_t *v, const int16_t *h,
                                              const int16_t *rv, const int16_t *rh) {
    int bits = tb.t1[(rv[1] + 23) * kTb1 + v[1] + 23] + tb.t2[(rv[2] + 17) * kTb2 + v[2] + 17] +
               tb.t1[(rh[1] + 23) * kTb1 + h[1] + 23] + tb.t2[(rh[2] + 17) * kTb2 + h[2] + 17];
    if (win == 7) bits += tb.t0[(rv[0] + 5) * kTb0 + v[0] + 5] + tb.t0[(rh[0] + 5) * kTb0 + h[0] + 5];
    return bits;
}

__device__ __forceinline__ void unit_rd(const FrameDesc &f, const LrPlane &pl, const RdUnit &u,
                                        const int16_t *rv, const int16_t *rh, const TapBits &tb, int64_t &bits_wn,
                                        bool &pick) {
    const int64_t cnt = count_bits_tab(tb, pl.win, u.v, u.h, rv, rh);
    bits_wn = 320 + (cnt << 9);
    const int64_t bits_none = 768;
    const double cn = rdcost_dbl(f.rdmult, bits_none >> 4, u.sse_none);
    const double cw = rdcost_dbl(f.rdmult, bits_wn >> 4, u.sse_wn);
    pick = cw < cn;
}

__global__ void __launch_bounds__(kLrFinThreads) k_lr_finish(FrameDesc *frames, int nframes) {
    extern __shared__ unsigned char lr_dyn[];
    __shared__ int frame_rtype;
    __shared__ int64_t red[kLrFinThreads / 32];
    __shared__ TapBits tb;
    const int id = blockIdx.x;
    if (id >= nframes * 3) return;
    FrameDesc &f = frames[id / 3];
    LrPlane &pl = f.lr[id % 3];
    const int t = threadIdx.x;
    if (!pl.on) {
        if (t == 0) pl.frame_rtype = 0;
        return;
    }
    const int n = pl.hunits * pl.vunits;
    const int npairs = n * (n + 1) / 2;
    const bool table = npairs <= kLrPairMax;
    fill_tap_bits(tb);
    RdUnit *U = reinterpret_cast<RdUnit *>(lr_dyn);
    int32_t *PT = reinterpret_cast<int32_t *>(lr_dyn + (size_t)n * sizeof(RdUnit));
    int64_t part = 0;
    for (int k = t; k < n; k += blockDim.x) {
        const LrUnit &u = pl.units[k];
        RdUnit r;
        r.sse_none = u.sse_none;
        if (pl.refine) {
            r.sse_wn = u.sse_wn;
        } else {  // k_lr_trial_tiles parts, combined as sse_region_hbd does
            r.sse_wn = u.score > 0 ? INT64_MAX
                       : f.bd == 8 ? (int64_t)(u.tw_blk + u.tw_rgt + u.tw_bot)
                                   : (int64_t)u.tw_blk + (int64_t)(uint32_t)u.tw_rgt + (int64_t)(uint32_t)u.tw_bot;
        }
        for (int i = 0; i < 3; ++i) {
            r.v[i] = u.vf[i];
            r.h[i] = u.hf[i];
        }
        r.pick = 0;
        // The WIENER cost grows with the tap bits and NONE's does not depend
        // on them, so the pick is "bits <= thr": thr by bisection on the
        // reference's own double comparison.
        r.thr = -1;
        if (r.sse_wn != INT64_MAX) {
            const double cn = rdcost_dbl(f.rdmult, 768 >> 4, r.sse_none);
            int lo = -1, hi = 64;  // pick(lo) holds (or lo = -1), pick(hi) does not
            if (rdcost_dbl(f.rdmult, (320 + ((int64_t)hi << 9)) >> 4, r.sse_wn) < cn) {
                lo = hi;  // beyond any count the taps can reach
            } else {
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (rdcost_dbl(f.rdmult, (320 + ((int64_t)mid << 9)) >> 4, r.sse_wn) < cn) lo = mid;
                    else hi = mid;
                }
            }
            r.thr = (int16_t)lo;
        }
        U[k] = r;
        part += u.sse_none;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
    if ((t & 31) == 0) red[t >> 5] = part;
    __syncthreads();
    // units with a trial (bit k of vmask), and each unit's taps packed for
    // the pair table: bytes v1 + 23, v2 + 17, h1 + 23, h2 + 17, then v0 + 5,
    // h0 + 5 (the tap tables' row / column offsets)
    __shared__ unsigned vmask[(kLrPairUnits + 31) / 32];
    __shared__ unsigned long long ptap[kLrPairUnits + 1];
    if (table) {
        if (t < kLrPairUnits + 1) {
            const int16_t dv[3] = {3, -7, 15};
            const int16_t *v = t < n ? U[t].v : dv, *h = t < n ? U[t].h : dv;  // entry n: the default reference
            ptap[t] = (unsigned long long)((v[1] + 23) | (v[2] + 17) << 8 | (h[1] + 23) << 16 | (h[2] + 17) << 24) |
                      (unsigned long long)((v[0] + 5) | (h[0] + 5) << 8) << 32;
        }
        if (t < ((kLrPairUnits + 31) / 32) * 32) {
            const unsigned m = __ballot_sync(0xffffffffu, t < n && U[t].sse_wn != INT64_MAX);
            if ((t & 31) == 0) vmask[t >> 5] = m;
        }
        __syncthreads();
        // pair (k, j), j in [-1, k): index k (k + 1) / 2 + j + 1; entry =
        // bits_wn | pick << 30 (bits_wn < 2^16). A warp per row k, lanes
        // over j (the unit's taps broadcast, the references' consecutive).
        const int lane = t & 31, warp = t >> 5, nw = blockDim.x >> 5;
        for (int k = warp; k < n; k += nw) {
            const int base = k * (k + 1) / 2 + 1;
            if (!((vmask[k >> 5] >> (k & 31)) & 1)) {
                for (int j = lane - 1; j < k; j += 32) PT[base + j] = 0;
                continue;
            }
            const unsigned long long pk = ptap[k];
            const int thr = U[k].thr;
            for (int j = lane - 1; j < k; j += 32) {
                const unsigned long long pj = ptap[j < 0 ? n : j];
                const unsigned a = (unsigned)pk, r = (unsigned)pj;
                int cnt = tb.t1[(r & 0xff) * kTb1 + (a & 0xff)] + tb.t2[((r >> 8) & 0xff) * kTb2 + ((a >> 8) & 0xff)] +
                          tb.t1[((r >> 16) & 0xff) * kTb1 + ((a >> 16) & 0xff)] + tb.t2[(r >> 24) * kTb2 + (a >> 24)];
                if (pl.win == 7) {
                    const unsigned a0 = (unsigned)(pk >> 32), r0 = (unsigned)(pj >> 32);
                    cnt += tb.t0[(r0 & 0xff) * kTb0 + (a0 & 0xff)] + tb.t0[(r0 >> 8) * kTb0 + (a0 >> 8)];
                }
                PT[base + j] = (320 + (cnt << 9)) | (cnt <= thr ? 1 << 30 : 0);
            }
        }
        __syncthreads();
    }
    // The walk (count_wiener_bits chained through the last WIENER unit's
    // taps): with the pair table its only serial step is the lookup of
    // (unit, last WIENER unit); each unit's pick and WIENER bits are recorded
    // and the frame's bits and SSE are summed by all threads afterwards.
    __shared__ int64_t fsum[2];
    if (t == 0) {
        if (table) {
            int last = -1;
            unsigned vm = 0;
            for (int k = 0; k < n; ++k) {
                if ((k & 31) == 0) vm = vmask[k >> 5];
                if (!((vm >> (k & 31)) & 1)) continue;  // no trial: pick stays 0
                const int32_t e = PT[k * (k + 1) / 2 + last + 1];
                const bool pick = (e >> 30) & 1;
                U[k].pick = pick ? 1 : 0;
                U[k].thr = (int16_t)(e & 0xffff);  // the WIENER bits, read back below
                last = pick ? k : last;
            }
        } else {
            int16_t rv[3] = {3, -7, 15}, rh[3] = {3, -7, 15};
            for (int k = 0; k < n; ++k) {
                RdUnit &u = U[k];
                if (u.sse_wn == INT64_MAX) continue;
                int64_t bits_wn;
                bool pick;
                unit_rd(f, pl, u, rv, rh, tb, bits_wn, pick);
                u.pick = pick ? 1 : 0;
                u.thr = (int16_t)bits_wn;
                if (pick)
                    for (int i = 0; i < 3; ++i) {
                        rv[i] = u.v[i];
                        rh[i] = u.h[i];
                    }
            }
        }
    }
    __syncthreads();
    {
        int64_t bsum = 0, ssum = 0;
        for (int k = t; k < n; k += blockDim.x) {
            const RdUnit &u = U[k];
            if (u.pick) {
                bsum += (uint16_t)u.thr;
                ssum += u.sse_wn;
            } else {
                bsum += 768;
                ssum += u.sse_none;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            bsum += __shfl_down_sync(0xffffffffu, bsum, o);
            ssum += __shfl_down_sync(0xffffffffu, ssum, o);
        }
        if (t < 2) fsum[t] = 0;
        __syncthreads();
        if ((t & 31) == 0) {
            atomicAdd((unsigned long long *)&fsum[0], (unsigned long long)bsum);
            atomicAdd((unsigned long long *)&fsum[1], (unsigned long long)ssum);
        }
        __syncthreads();
    }
    if (t == 0) {
        int64_t total = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) total += red[w];
        const double cost_none_frame = rdcost_dbl(f.rdmult, 0, total);
        const double cost_wn_frame = rdcost_dbl(f.rdmult, fsum[0] >> 4, fsum[1]);
        frame_rtype = cost_wn_frame < cost_none_frame ? 1 : 0;
        pl.frame_rtype = frame_rtype;
    }
    __syncthreads();
    for (int k = t; k < n; k += blockDim.x) {
        const int rt = frame_rtype ? U[k].pick : 0;
        pl.units[k].rtype = rt;
        PackedUnit o;
        for (int i = 0; i < 8; ++i) {
            o.vf[i] = pl.units[k].vf[i];
            o.hf[i] = pl.units[k].hf[i];
        }
        o.rtype = (uint8_t)rt;
        for (int i = 0; i < 7; ++i) o.pad[i] = 0;
        pl.packed[k] = o;
    }
}

// ---------------------------------------------------------------------------
// 5. Apply (apply_restoration_frame, restoration.rs:992-1052) with the
// stripe boundaries of save_lr_boundaries, writing every pixel of C: one CTA
// per (plane, stripe, group of `group` <= kApplyGroupMax 64-px column tiles) over the
// aligned canvas. Tiles of Wiener units are filtered within the true plane
// and copied from A beyond it; every other tile (unit NONE, frame NONE,
// plane not searched, and the rows below the true plane: stripe index
// nstripes) is copied from A. Rows above / below a stripe come from the
// post-deblock (pre-CDEF) plane B at interior stripe edges (the only lines
// the single-tile apply reads) and from the edge-replicated post-CDEF plane
// at the frame top / bottom. items: a = unit row (-1: copy only), b = stripe.
// A CTA looks its tiles' units up at once and copies every copied part
// before it filters (planes the tiled trial did not write), so a copy-only
// group pays one barrier.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_lr_apply(FrameDesc *frames, const WorkItem *items, int nitems, int group) {
    constexpr int SW = TT_W + 7;
    constexpr int MAXH = 64 + 7;
    __shared__ __align__(16) uint16_t stage[MAXH * SW];
    __shared__ __align__(16) uint16_t tmp[MAXH * TT_W];
    __shared__ int s_unit[kApplyGroupMax], s_filter[kApplyGroupMax];
    const WorkItem wi = items[find_item(items, nitems, blockIdx.x)];
    const FrameDesc &f = frames[wi.frame];
    const LrPlane &pl = f.lr[wi.plane];
    const int ss = wi.plane ? 1 : 0;
    const int full = 64 >> ss, off = 8 >> ss;
    const int s = wi.b;
    const int bd = f.bd, stride = plane_stride(f, wi.plane);
    const int canvas_h = wi.plane ? f.h / 2 : f.h;
    const int nstripes = (pl.ph + off + full - 1) / full;
    // rows of this item: a stripe of the true plane, or the canvas rows below it
    const int ys = s < nstripes ? max(0, s * full - off) : pl.ph;
    const int ye = s < nstripes ? min(pl.ph, (s + 1) * full - off) : canvas_h;
    const int ntiles = (stride + TT_W - 1) / TT_W;
    const int g0 = (blockIdx.x - wi.cta_begin) * group;
    const int ntl = min(group, ntiles - g0);
    const uint8_t *post = f.A[wi.plane], *pre = f.B[wi.plane];
    uint8_t *out = f.C[wi.plane];
    // the unit of each tile: wi.a is its row of the unit grid (-1: copy
    // only), the column is looked up along that row, one thread per tile
    if ((int)threadIdx.x < ntl) {
        const int x0 = (g0 + (int)threadIdx.x) * TT_W;
        int unit = -1;
        if (wi.a >= 0 && pl.on) {
            const UnitRect *urow = pl.rects + wi.a * pl.hunits;
            for (int c = 0; c < pl.hunits; ++c)
                if (x0 >= urow[c].h_start && x0 < urow[c].h_end) {
                    unit = wi.a * pl.hunits + c;
                    break;
                }
        }
        s_unit[threadIdx.x] = unit;
        s_filter[threadIdx.x] = s < nstripes && unit >= 0 && pl.frame_rtype != 0 && pl.units[unit].rtype == 1;
    }
    __syncthreads();
    const int spw = word_samples(bd);
    const bool words = aligned4(post) && aligned4(out);
    // copied columns of each tile: all of them, or those beyond the true width
    for (int k = 0; k < ntl; ++k) {
        const int x0 = (g0 + k) * TT_W, tw = min(TT_W, stride - x0);
        const int cx = s_filter[k] ? min(tw, pl.pw - x0) : 0;
        if (cx == 0 && words) {  // whole tile: word copies (tw is a multiple of 4, as plane widths are)
            const int nwr = tw / spw;
            for (int q = threadIdx.x; q < (ye - ys) * nwr; q += blockDim.x) {
                const int rr = q / nwr, wx = q - rr * nwr;
                const int64_t o = ((int64_t)(ys + rr) * stride + x0) * (bd == 8 ? 1 : 2) + wx * 4;
                *reinterpret_cast<uint32_t *>(out + o) = *reinterpret_cast<const uint32_t *>(post + o);
            }
        } else if (cx < tw) {
            for (int q = threadIdx.x; q < (ye - ys) * (tw - cx); q += blockDim.x) {
                const int rr = q / (tw - cx), cc = cx + (q - rr * (tw - cx));
                const int64_t o = (int64_t)(ys + rr) * stride + x0 + cc;
                stpx(out, o, bd, ldpx(post, o, bd));
            }
        }
    }
    // a tiled-trial plane: the trial wrote its units' final pixels
    if (pl.trial_out) return;
    const bool copy_above = s > 0, copy_below = ye < pl.ph;
    for (int k = 0; k < ntl; ++k) {
        if (!s_filter[k]) continue;  // uniform over the CTA
        const int x0 = (g0 + k) * TT_W, tw = min(TT_W, stride - x0);
        const int ncol = min(tw, pl.pw - x0);
        const LrUnit &u = pl.units[s_unit[k]];
        int16_t hf[8], vf[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            hf[j] = u.hf[j];
            vf[j] = u.vf[j];
        }
        // Output rows [rb, re) of the stripe: stage rows rb - 3 .. re + 3
        // with the stripe's boundary substitution, horizontal pass, vertical
        // pass.
        const int rb = ys, re = ye;
        const int nrow = re - rb, rows = nrow + 7;
        auto row_of = [&](int rr) {
            const int y = rb - 3 + rr;
            const uint8_t *src = post;
            int yy;
            if (y < ys) {
                if (copy_above) {
                    src = pre;
                    yy = y == ys - 1 ? ys - 1 : ys - 2;
                } else {
                    yy = clampi(y, 0, pl.ph - 1);
                }
            } else if (y >= ye) {
                if (copy_below) {
                    src = pre;
                    yy = y == ye ? ye : min(ye + 1, pl.ph - 1);
                } else {
                    yy = clampi(y, 0, pl.ph - 1);
                }
            } else {
                yy = y;
            }
            return row_ptr(src, yy, stride, bd);
        };
        __syncthreads();  // the previous tile's reads of stage / tmp are done
        stage_window(bd, pl.pw, rows, x0 - 3, SW, true, 0, row_of,
                     [&](int rr, int cc, int v) { stage[rr * SW + cc] = (uint16_t)v; });
        __syncthreads();
        // four outputs per thread along each pass from 11 staged samples
        for (int q = threadIdx.x; q < rows * (TT_W / 4); q += blockDim.x) {
            const int rr = q >> 4, c0 = (q & 15) * 4;
            int p[11];
#pragma unroll
            for (int j = 0; j < 11; ++j) p[j] = stage[rr * SW + c0 + j];
            uint32_t o[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) o[j] = (uint32_t)wiener_h(p + j, hf, bd);
            *reinterpret_cast<uint2 *>(tmp + rr * TT_W + c0) = make_uint2(o[0] | o[1] << 16, o[2] | o[3] << 16);
        }
        __syncthreads();
        for (int q = threadIdx.x; q < ((nrow + 3) >> 2) * TT_W; q += blockDim.x) {
            const int r0 = (q >> 6) * 4, cc = q & (TT_W - 1);
            if (cc >= ncol) continue;
            int p[11];
#pragma unroll
            for (int j = 0; j < 11; ++j) p[j] = tmp[(r0 + j) * TT_W + cc];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (r0 + j >= nrow) break;
                stpx(out, (int64_t)(rb + r0 + j) * stride + x0 + cc, bd, wiener_v(p + j, vf, bd));
            }
        }
    }
}

}  // namespace zf

namespace zf {
// Host-side launcher: the templated kernel is instantiated and launched in
// this translation unit (whole-program compilation cannot launch a template
// instantiation owned by another unit).
cudaError_t launch_lr_trial_tiles(int tl, int ctas, cudaStream_t st, FrameDesc *frames, const WorkItem *items,
                                  int nitems) {
    if (tl == 32) k_lr_trial_tiles<32><<<ctas, 256, 0, st>>>(frames, items, nitems);
    else if (tl == 64) k_lr_trial_tiles<64><<<ctas, 256, 0, st>>>(frames, items, nitems);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_lr_stats(int win, int bd, int ctas, cudaStream_t st, FrameDesc *frames, const WorkItem *items,
                            int nitems) {
    if (win == 5 && bd == 8) k_lr_stats<5, 8><<<ctas, 256, 0, st>>>(frames, items, nitems);
    else if (win == 5 && bd == 10) k_lr_stats<5, 10><<<ctas, 256, 0, st>>>(frames, items, nitems);
    else if (win == 5) return cudaErrorInvalidValue;  // bit depths are 8 or 10
    else k_lr_stats<7, 0><<<ctas, 256, 0, st>>>(frames, items, nitems);
    return cudaGetLastError();
}
}  // namespace zf
