// zf_cdef.cu -- CDEF strength search and apply on the GPU.
//
// Reference: svtav1-dsp/src/cdef.rs (find_dir :143-198, constrain :113,
// adjust_strength :125, the scalar block filter :931-1034 and its dst16
// twin hbd.rs:1765-1850) and svtav1-encoder/src/cdef.rs (search
// :1166-1568, finish :812-944, apply :343-708).
//
// The CDEF working buffer of the reference is a per-64x64 copy of the
// post-deblock plane with CDEF_VERY_LARGE (0x7f7f) outside the aligned
// canvas. Here a CTA owns one 64x64 filter block and stages exactly that
// (plus the 2-pixel reach of the taps) in shared memory, so every pixel of
// every candidate reads the same values as the reference's build_src.
#include <algorithm>
#include <mutex>

#include <cuda.h>

#include <cooperative_groups.h>

#include "zf_dev.cuh"

namespace zf {

constexpr uint16_t kVeryLarge = 0x7f7f;
constexpr int CR = 68;  // luma region edge: 64 + 2 * 2 halo
constexpr int CRC = 36; // chroma region edge: 32 + 2 * 2
// Row pitches in 2-byte samples. At presets <= 5 a warp reads 4 rows x 8
// columns of one luma 8x8 block, every lane at the same tap offset: with
// 38 words per row those rows start 6 banks apart, so the 4-word row
// segments (5 words at an odd offset) of the 32 lanes fall in distinct
// banks (the region's own 34 words put the rows 2 banks apart: a 2-way
// conflict on every tap read). At preset 6 (every fourth row) a warp reads
// rows 0 and 4 of two adjacent blocks, 24 banks apart at this pitch. The
// direction search's 8 rows x 4 blocks of a warp stay 2-way, as before.
// The source tiles read one sample per lane: 36 words per row (64 samples
// were 32 words, every row in the same banks: 4-way); the chroma windows
// keep 18 words per row, their source tiles take the same.
constexpr int CRP = 76;
constexpr int SRCP = 72;
constexpr int SRCCP = 36;

// Cdef_Directions (AV1 spec 7.15.3) as (dy, dx).
__constant__ int8_t kDir[8][2][2] = {
    {{-1, 1}, {-2, 2}}, {{0, 1}, {-1, 2}}, {{0, 1}, {0, 2}}, {{0, 1}, {1, 2}},
    {{1, 1}, {2, 2}},   {{1, 0}, {2, 1}},  {{1, 0}, {2, 0}}, {{1, 0}, {2, -1}},
};

__device__ __forceinline__ int msb(unsigned v) { return 31 - __clz(v); }

// adjust_strength (cdef.rs:125-136).
__device__ __forceinline__ int adjust_strength(int strength, int var) {
    int i = (var >> 6) != 0 ? min(msb((unsigned)(var >> 6)), 12) : 0;
    return var != 0 ? (strength * (4 + i) + 8) >> 4 : 0;
}

// The search stores each block's variance as a code (0: var == 0, else
// 1 + i with i the adjust_strength exponent) beside its direction; the
// apply rebuilds the adjusted strength from it.
__device__ __forceinline__ int var_code(int var) {
    return var != 0 ? 1 + ((var >> 6) != 0 ? min(msb((unsigned)(var >> 6)), 12) : 0) : 0;
}
__device__ __forceinline__ int adjust_strength_code(int strength, int code) {
    return code != 0 ? (strength * (3 + code) + 8) >> 4 : 0;
}

// cdef_find_dir (cdef.rs:143-198), split by direction pairs so that four
// threads share one 8x8 block: pair 0 = directions (0, 4), 1 = (2, 6),
// 2 = (1, 5), 3 = (3, 7). Each pass keeps at most 30 partial sums live.
__host__ __device__ constexpr int kDiv(int n) { return n ? 840 / n : 0; }  // 840 / n

template <int PAIR>
__device__ __forceinline__ void dir_cost_pair(const uint16_t *img, int rs, int cs, int &ca, int &cb) {
    constexpr int NB = (PAIR == 0) ? 15 : (PAIR == 1 ? 8 : 11);
    int pa[NB], pb[NB];
#pragma unroll
    for (int k = 0; k < NB; ++k) pa[k] = pb[k] = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int x = ((int)img[i * rs + j] >> cs) - 128;
            if (PAIR == 0) {
                pa[i + j] += x;
                pb[7 + i - j] += x;
            } else if (PAIR == 1) {
                pa[i] += x;
                pb[j] += x;
            } else if (PAIR == 2) {
                pa[i + j / 2] += x;
                pb[3 - i / 2 + j] += x;
            } else {
                pa[3 + i - j / 2] += x;
                pb[i / 2 + j] += x;
            }
        }
    auto cost = [&](const int *p) {
        int c = 0;
        if (PAIR == 0) {
#pragma unroll
            for (int i = 0; i < 7; ++i) c += (p[i] * p[i] + p[14 - i] * p[14 - i]) * kDiv(i + 1);
            c += p[7] * p[7] * kDiv(8);
        } else if (PAIR == 1) {
#pragma unroll
            for (int i = 0; i < 8; ++i) c += p[i] * p[i];
            c *= kDiv(8);
        } else {
#pragma unroll
            for (int j = 0; j < 5; ++j) c += p[3 + j] * p[3 + j];
            c *= kDiv(8);
#pragma unroll
            for (int j = 0; j < 3; ++j) c += (p[j] * p[j] + p[10 - j] * p[10 - j]) * kDiv(2 * j + 2);
        }
        return c;
    };
    ca = cost(pa);
    cb = cost(pb);
}

// Directions and variances of the blocks blist[0..nblk) of a region (block
// b at region row (b >> 3) * 8 + 2, column (b & 7) * 8 + 2): four threads
// per block (a 256-thread CTA: thread t takes pair t >> 6, block t & 63, so
// each warp runs one pair), the per-direction costs meet in `cost`, then
// one thread per block picks the best direction (strictly greater wins, the
// lowest index on ties) and var = (best - cost of the orthogonal) >> 10.
// Every thread of the CTA calls this.
__device__ void find_dirs(const uint16_t *reg, int rs, int cs, const int *blist, int nblk, int (*cost)[8],
                          int *sdir, int *svar) {
    const int t = threadIdx.x, pair = t >> 6, k = t & 63;
    if (k < nblk) {
        const int b = blist[k];
        const uint16_t *img = reg + ((b >> 3) * 8 + 2) * rs + (b & 7) * 8 + 2;
        int ca, cb;
        if (pair == 0) {
            dir_cost_pair<0>(img, rs, cs, ca, cb);
            cost[b][0] = ca;
            cost[b][4] = cb;
        } else if (pair == 1) {
            dir_cost_pair<1>(img, rs, cs, ca, cb);
            cost[b][2] = ca;
            cost[b][6] = cb;
        } else if (pair == 2) {
            dir_cost_pair<2>(img, rs, cs, ca, cb);
            cost[b][1] = ca;
            cost[b][5] = cb;
        } else {
            dir_cost_pair<3>(img, rs, cs, ca, cb);
            cost[b][3] = ca;
            cost[b][7] = cb;
        }
    }
    __syncthreads();
    if (t < nblk) {
        const int b = blist[t];
        int best_cost = 0, best_dir = 0;
#pragma unroll
        for (int i = 0; i < 8; ++i)
            if (cost[b][i] > best_cost) {
                best_cost = cost[b][i];
                best_dir = i;
            }
        sdir[b] = best_dir;
        svar[b] = (best_cost - cost[b][(best_dir + 4) & 7]) >> 10;
    }
    __syncthreads();
}

// Stage a plane window [y0-2, y0+n+2) x [x0-2, x0+n+2) with the sentinel
// outside the aligned plane (build_src, cdef.rs:517-544).
__device__ __noinline__ void load_region(const uint8_t *plane, int bd, int pw, int ph, int x0, int y0, int n,
                                         uint16_t *reg, int pitch) {
    const int rs = n + 4;
    auto rowf = [&](int ry) {
        const int y = y0 - 2 + ry;
        return (y >= 0 && y < ph) ? row_ptr(plane, y, pw, bd) : (const uint8_t *)nullptr;
    };
    auto putf = [&](int ry, int rx, int v) { reg[ry * pitch + rx] = (uint16_t)v; };
    // the staging loop once with the bit depth a constant (8-bit rows: four
    // samples a word and their extraction resolved at compile time, 8 % off
    // the CDEF search on 8-bit frames), once for other depths
    if (bd == 8) stage_window<1>(8, pw, rs, x0 - 2, rs, false, kVeryLarge, rowf, putf);
    else stage_window<1>(bd, pw, rs, x0 - 2, rs, false, kVeryLarge, rowf, putf);
}

// Stage the n x n source tile at (x0, y0), 0 outside the canvas.
__device__ __noinline__ void load_src(const uint8_t *plane, int bd, int pw, int ph, int x0, int y0, int n,
                                      uint16_t *src, int pitch) {
    auto rowf = [&](int ry) { return y0 + ry < ph ? row_ptr(plane, y0 + ry, pw, bd) : (const uint8_t *)nullptr; };
    auto putf = [&](int ry, int rx, int v) { src[ry * pitch + rx] = (uint16_t)v; };
    if (bd == 8) stage_window<1>(8, pw, n, x0, n, false, 0, rowf, putf);  // as in load_region
    else stage_window<1>(bd, pw, n, x0, n, false, 0, rowf, putf);
}

// Non-skip 8x8 blocks of one filter block (the dlist, cdef.rs:1203-1213):
// bit (by*8+bx) of the returned mask; blocks past a partial fb are 0.
// Threads 0..63 test one block each, warp ballots meet in `part` (two
// words); every thread of the CTA calls this and gets the mask.
__device__ uint64_t fb_dlist(const FrameDesc &f, int fbr, int fbc, unsigned *part) {
    const int vsize = min(64, f.h - fbr * 64), hsize = min(64, f.w - fbc * 64);
    const int t = threadIdx.x;
    bool nonskip = false;
    if (t < 64) {
        const int by = t >> 3, bx = t & 7;
        if (by < vsize / 8 && bx < hsize / 8) {
            const int r = fbr * 16 + by * 2, c = fbc * 16 + bx * 2;
            bool all = true;
            for (int rr = r; rr < min(r + 2, f.mi_rows); ++rr)
                for (int cc = c; cc < min(c + 2, f.mi_cols); ++cc)
                    all = all && mi_skip(f.mi[(int64_t)rr * f.mi_cols + cc]);
            nonskip = !all;
        }
    }
    const unsigned m = __ballot_sync(0xffffffffu, nonskip);
    if (t < 64 && (t & 31) == 0) part[t >> 5] = m;
    __syncthreads();
    return (uint64_t)part[0] | ((uint64_t)part[1] << 32);
}

__device__ __forceinline__ unsigned long long block_sum_u64(unsigned long long v, unsigned long long *scratch) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) scratch[threadIdx.x >> 5] = v;
    __syncthreads();
    unsigned long long s = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += scratch[w];
    return s;  // valid in thread 0
}

// constrain with the damping shift precomputed: shift = max(0, damping -
// msb(threshold)) (cdef.rs:113-120); threshold 0 gives 0 for any shift.
// sign(d) * min(|d|, m) with m = max(0, thr - (|d| >> shift)) >= 0 is d
// clamped to [-m, m].
//
// Computed as sign(d) * max(0, min(|d|, thr - (|d| >> shift))) -- the same
// value, since |d| >= 0 -- whose clamp is one three-operand min-with-zero
// (a DPX instruction) instead of three two-operand min/max.
__device__ __forceinline__ int constrain_s(int d, int thr, int shift) {
    const int a = abs(d);
    const int r = __vimin_s32_relu(a, thr - (a >> shift));
    return d < 0 ? -r : r;
}
__device__ __forceinline__ int damp_shift(int thr, int damping) {
    return thr ? max(0, damping - msb((unsigned)thr)) : 0;
}

// Region offsets of the taps of direction `dir` (row stride rs): primary
// k = 0, 1, then the secondary directions dir + 2 and dir + 6, k = 0, 1.
__device__ __forceinline__ void dir_offsets(int dir, int rs, int *o) {
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        o[k] = kDir[dir][k][0] * rs + kDir[dir][k][1];
        o[2 + k] = kDir[(dir + 2) & 7][k][0] * rs + kDir[(dir + 2) & 7][k][1];
        o[4 + k] = kDir[(dir + 6) & 7][k][0] * rs + kDir[(dir + 6) & 7][k][1];
    }
}

// The 12 taps of one pixel as differences to x (read as int16, so the
// sentinel is a large positive value), and the clamp range: min over x and
// all taps, max over x and the taps that are not the sentinel.
// d[0..3]: primary +k0, -k0, +k1, -k1; d[4..7]: secondary k0 (+2, -2, +6,
// -6); d[8..11]: secondary k1.
// EDGE = false: the region holds no sentinel (the filter block and its
// 2-pixel reach lie inside the canvas), so the max needs no test.
template <bool EDGE = true>
__device__ __forceinline__ void load_taps(const uint16_t *reg, int pos, const int *o, int x, int *d, int &mx,
                                          int &mn) {
    mx = x;
    mn = x;
    int q[12];
    q[0] = pos + o[0]; q[1] = pos - o[0]; q[2] = pos + o[1]; q[3] = pos - o[1];
    q[4] = pos + o[2]; q[5] = pos - o[2]; q[6] = pos + o[4]; q[7] = pos - o[4];
    q[8] = pos + o[3]; q[9] = pos - o[3]; q[10] = pos + o[5]; q[11] = pos - o[5];
    if constexpr (EDGE) {
#pragma unroll
        for (int t = 0; t < 12; ++t) {
            const uint16_t r = reg[q[t]];
            const int v = (int16_t)r;
            if (r != kVeryLarge) mx = max(mx, v);
            mn = min(mn, v);
            d[t] = v - x;
        }
    } else {
        // no sentinel: the 13 values' max and min by three-operand DPX
        // min/max, two taps per instruction
        int v[12];
#pragma unroll
        for (int t = 0; t < 12; ++t) {
            v[t] = (int16_t)reg[q[t]];
            d[t] = v[t] - x;
        }
#pragma unroll
        for (int t = 0; t < 12; t += 2) {
            mx = __vimax3_s32(mx, v[t], v[t + 1]);
            mn = __vimin3_s32(mn, v[t], v[t + 1]);
        }
    }
}

// load_taps with the sentinel test only where the region can hold one
// (a CTA-uniform branch).
__device__ __forceinline__ void load_taps_at(bool edge, const uint16_t *reg, int pos, const int *o, int x, int *d,
                                             int &mx, int &mn) {
    if (edge) load_taps<true>(reg, pos, o, x, d, mx, mn);
    else load_taps<false>(reg, pos, o, x, d, mx, mn);
}

// Primary and secondary parts of the tap sum. The reference sums in
// wrapping int16 (cdef.rs:965-1023); |sum| <= 2*(4+2)*60 + 12*16 = 912 for
// every strength at 8 and 10 bits, so plain int sums are identical, and the
// sum splits exactly into a primary part (per primary strength) and a
// secondary part (per secondary strength).
__device__ __forceinline__ int prim_sum(const int *d, int t, int shift, int cs) {
    const int odd = (t >> cs) & 1;
    const int w0 = odd ? 3 : 4, w1 = odd ? 3 : 2;
    return w0 * (constrain_s(d[0], t, shift) + constrain_s(d[1], t, shift)) +
           w1 * (constrain_s(d[2], t, shift) + constrain_s(d[3], t, shift));
}
__device__ __forceinline__ int sec_sum(const int *d, int s, int shift) {
    return 2 * (constrain_s(d[4], s, shift) + constrain_s(d[5], s, shift) + constrain_s(d[6], s, shift) +
                constrain_s(d[7], s, shift)) +
           (constrain_s(d[8], s, shift) + constrain_s(d[9], s, shift) + constrain_s(d[10], s, shift) +
            constrain_s(d[11], s, shift));
}
__device__ __forceinline__ int cdef_round(int x, int sum, int mn, int mx) {
    return min(max(x + ((8 + sum - (sum < 0)) >> 4), mn), mx);
}

// Search: one CTA per filter block. Writes the fb's luma and joint-chroma
// mse rows (cdef_search_still[_hbd], cdef.rs:1166-1568) and whether the fb
// has a row.
//
// The candidate list of every preset is a grid: fp first-pass strengths
// (primary p_i, secondary 0) followed by p_i x each of ns - 1 extra
// secondary strengths (cdef_search_cfg_for_preset, cdef.rs:788-810). Per
// pixel the kernel loads the taps once per direction set (the block's
// direction for p_i != 0, direction 0 for p_i == 0), computes the primary
// part once per p_i and the secondary part once per secondary strength, and
// forms every candidate from the two parts. FPM x NSM bounds fp x ns.
template <int FPM, int NSM>
__global__ void __launch_bounds__(256) k_cdef_search(const FrameDesc *frames, const WorkItem *items, int nitems) {
    constexpr int NCM = FPM * NSM;
    __shared__ uint16_t reg[CR * CRP];
    __shared__ uint16_t src[64 * SRCP];
    __shared__ int sdir[64], svar[64];
    __shared__ int dcost[64][8];
    __shared__ int boff[64][6], boffc[64][6];
    __shared__ int bpri[64][FPM];  // adjusted primary strength | damping shift << 16
    __shared__ int blist[64];
    __shared__ int nblk;
    __shared__ uint16_t regc[2][CRC * CRC];
    __shared__ uint16_t srcc[2][32 * SRCCP];
    __shared__ uint32_t part[8][NCM + 2 * FPM];
    const int it = find_item(items, nitems, blockIdx.x);
    const WorkItem wi = items[it];
    const FrameDesc &f = frames[wi.frame];
    const CdefParams &cp = f.cdef;
    const int fb = blockIdx.x - wi.cta_begin;
    const int fbr = fb / f.nhfb, fbc = fb - fbr * f.nhfb;
    const int bd = f.bd, cs = bd - 8;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ unsigned dl_part[2];
    const uint64_t dl = fb_dlist(f, fbr, fbc, dl_part);
    if (threadIdx.x == 0) {
        f.fb_row[fb] = dl != 0;
        int n = 0;
        for (int b = 0; b < 64; ++b)
            if ((dl >> b) & 1) blist[n++] = b;
        nblk = n;
    }
    if (dl == 0) return;
    const int n_cand = cp.ncand, fp = cp.first_pass_num, ns = n_cand / fp;
    uint64_t *row = f.mse + (int64_t)fb * 2 * n_cand;
    const int dmp = cp.damping + cs;
    int pri[FPM], sec[NSM], ssh[NSM];
    bool any_zero = false;
#pragma unroll
    for (int i = 0; i < FPM; ++i) {
        pri[i] = i < fp ? (cp.fs[i] / 4) << cs : 0;
        any_zero = any_zero || (i < fp && pri[i] == 0);
    }
    sec[0] = 0;
    ssh[0] = 0;
#pragma unroll
    for (int j = 1; j < NSM; ++j) {
        const int s = j < ns ? cp.fs[fp + j - 1] % 4 : 0;
        sec[j] = (s + (s == 3)) << cs;
        ssh[j] = damp_shift(sec[j], dmp);
    }
    // ---- every plane's window staged at once (luma, then U and V)
    const int x0 = fbc * 64, y0 = fbr * 64;
    const int cw = f.w / 2, ch = f.h / 2, cx0 = fbc * 32, cy0 = fbr * 32;
    load_region(f.B[0], bd, f.w, f.h, x0, y0, 64, reg, CRP);
    load_src(f.S[0], bd, f.w, f.h, x0, y0, 64, src, SRCP);
    if (f.chroma)
#pragma unroll 1
        for (int p = 0; p < 2; ++p) {
            load_region(f.B[p + 1], bd, cw, ch, cx0, cy0, 32, regc[p], CRC);
            load_src(f.S[p + 1], bd, cw, ch, cx0, cy0, 32, srcc[p], SRCCP);
        }
    __syncthreads();
    find_dirs(reg, CRP, cs, blist, nblk, dcost, sdir, svar);
    for (int k = threadIdx.x; k < nblk; k += blockDim.x) {
        const int b = blist[k];
        const int dir = sdir[b], var = svar[b];
        if (f.cdir) f.cdir[(int64_t)fb * 64 + b] = (uint8_t)(dir | (var_code(var) << 3));
        dir_offsets(dir, CRP, boff[b]);
        dir_offsets(dir, CRC, boffc[b]);
#pragma unroll
        for (int i = 0; i < FPM; ++i) {
            const int t = adjust_strength(pri[i], var);
            bpri[b][i] = t | (damp_shift(t, dmp) << 16);
        }
    }
    __syncthreads();
    const int sub = cp.sub_y;
    const int lgs = 6 - (__ffs(sub) - 1);  // sampled slots per 8x8 block: 64 / sub
    const int slots = nblk << lgs;
    // the 2-pixel reach of the filter block inside the canvas: no sentinel
    const bool edge_y = !(x0 >= 2 && y0 >= 2 && x0 + 66 <= f.w && y0 + 66 <= f.h);
    const bool edge_uv = !(x0 >= 4 && y0 >= 4 && x0 / 2 + 34 <= f.w / 2 && y0 / 2 + 34 <= f.h / 2);
    uint32_t acc[NCM];
#pragma unroll
    for (int c = 0; c < NCM; ++c) acc[c] = 0;
    for (int q = threadIdx.x; q < slots; q += blockDim.x) {
        const int k = q >> lgs, rem = q & ((1 << lgs) - 1);
        const int b = blist[k];
        const int py = (b >> 3) * 8 + (rem >> 3) * sub, px = (b & 7) * 8 + (rem & 7);
        const int pos = (py + 2) * CRP + px + 2;
        const int x = (int16_t)reg[pos], sv = src[py * SRCP + px];
        int d[12], mx, mn, S[NSM];
        {  // block direction: candidates with p_i != 0
            load_taps_at(edge_y, reg, pos, boff[b], x, d, mx, mn);
            S[0] = 0;
#pragma unroll
            for (int j = 1; j < NSM; ++j) S[j] = j < ns ? sec_sum(d, sec[j], ssh[j]) : 0;
#pragma unroll
            for (int i = 0; i < FPM; ++i) {
                if (i >= fp || pri[i] == 0) continue;
                const int tp = bpri[b][i];
                const int P = prim_sum(d, tp & 0xffff, tp >> 16, cs);
#pragma unroll
                for (int j = 0; j < NSM; ++j) {
                    if (j >= ns) continue;
                    const int e = sv - cdef_round(x, P + S[j], mn, mx);
                    acc[i * NSM + j] += (uint32_t)(e * e);
                }
            }
        }
        if (any_zero) {  // direction 0: candidates with p_i == 0
            const int o0[6] = {-1 * CRP + 1, -2 * CRP + 2, 0 * CRP + 1, 0 * CRP + 2, 1 * CRP + 0, 2 * CRP + 0};
            load_taps_at(edge_y, reg, pos, o0, x, d, mx, mn);
#pragma unroll
            for (int j = 1; j < NSM; ++j) S[j] = j < ns ? sec_sum(d, sec[j], ssh[j]) : 0;
#pragma unroll
            for (int i = 0; i < FPM; ++i) {
                if (i >= fp || pri[i] != 0) continue;
#pragma unroll
                for (int j = 0; j < NSM; ++j) {
                    if (j >= ns) continue;
                    const int e = sv - cdef_round(x, S[j], mn, mx);
                    acc[i * NSM + j] += (uint32_t)(e * e);
                }
            }
        }
    }
    // per-warp partials (a lane holds <= 16 pixels of e^2 <= 1023^2: the
    // warp total fits u32), then the fb total in u64
#pragma unroll
    for (int c = 0; c < NCM; ++c) {
        uint32_t v = acc[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) part[warp][c] = v;
    }
    // ---- chroma: U and V accumulate into the joint row (first-pass
    // strengths only: secondary 0, primary not adjusted, damping - 1)
    if (f.chroma) {
        const int cdmp = dmp - 1;
        int csh[FPM];
#pragma unroll
        for (int i = 0; i < FPM; ++i) csh[i] = damp_shift(pri[i], cdmp);
        const int cslots = nblk * 16;
#pragma unroll 1
        for (int p = 0; p < 2; ++p) {
            uint32_t cacc[FPM];
#pragma unroll
            for (int i = 0; i < FPM; ++i) cacc[i] = 0;
            for (int q = threadIdx.x; q < cslots; q += blockDim.x) {
                const int k = q >> 4, b = blist[k];
                const int py = (b >> 3) * 4 + ((q >> 2) & 3), px = (b & 7) * 4 + (q & 3);
                const int pos = (py + 2) * CRC + px + 2;
                const int x = (int16_t)regc[p][pos], sv = srcc[p][py * SRCCP + px];
                int d[12], mx, mn;
                load_taps_at(edge_uv, regc[p], pos, boffc[b], x, d, mx, mn);
#pragma unroll
                for (int i = 0; i < FPM; ++i) {
                    if (i >= fp) continue;
                    // primary 0 and secondary 0: every tap term is 0, the pixel is kept
                    const int y = pri[i] ? cdef_round(x, prim_sum(d, pri[i], csh[i], cs), mn, mx) : x;
                    const int e = sv - y;
                    cacc[i] += (uint32_t)(e * e);
                }
            }
#pragma unroll
            for (int i = 0; i < FPM; ++i) {
                uint32_t v = cacc[i];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
                if (lane == 0) part[warp][NCM + p * FPM + i] = v;
            }
        }
    }
    __syncthreads();
    const int nw = (int)(blockDim.x >> 5);
    for (int c = threadIdx.x; c < NCM; c += blockDim.x) {
        const int i = c / NSM, j = c - i * NSM;
        if (i >= fp || j >= ns) continue;
        unsigned long long tot = 0;
        for (int w = 0; w < nw; ++w) tot += part[w][c];
        const int gi = j == 0 ? i : fp + i * (ns - 1) + (j - 1);
        row[gi] = (tot >> (2 * cs)) * (unsigned long long)sub;
    }
    for (int gi = threadIdx.x; gi < n_cand; gi += blockDim.x) {
        unsigned long long v = 0;
        if (f.chroma) {
            if (gi < fp) {
                unsigned long long tu = 0, tv = 0;
                for (int w = 0; w < nw; ++w) {
                    tu += part[w][NCM + gi];
                    tv += part[w][NCM + FPM + gi];
                }
                v = ((tu >> (2 * cs)) + (tv >> (2 * cs))) * (unsigned long long)cp.sub_uv;
            } else {
                v = 1040400ull * 64ull;
            }
        }
        row[n_cand + gi] = v;
    }
}

// Launch the search instantiation covering fp x ns (the largest over the
// batch's frames).
cudaError_t launch_cdef_search(int fp, int ns, int ctas, cudaStream_t st, const FrameDesc *frames,
                               const WorkItem *items, int nitems) {
    if (fp <= 2 && ns <= 2) k_cdef_search<2, 2><<<ctas, 256, 0, st>>>(frames, items, nitems);
    else if (fp <= 3 && ns <= 2) k_cdef_search<3, 2><<<ctas, 256, 0, st>>>(frames, items, nitems);
    else if (fp <= 5 && ns <= 4) k_cdef_search<5, 4><<<ctas, 256, 0, st>>>(frames, items, nitems);
    else if (fp <= 12 && ns <= 4) k_cdef_search<12, 4><<<ctas, 256, 0, st>>>(frames, items, nitems);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

// ---- finish: the joint strength search of one frame in one CTA ----------

// RDCOST (cdef.rs:814-816).
__device__ __forceinline__ unsigned long long rdc(unsigned long long lambda, unsigned long long rate,
                                                  unsigned long long dist) {
    return ((rate * lambda + 256) >> 9) + (dist << 7);
}

// finish_cdef_rd + the per-fb index (cdef.rs:897-944, :1326-1344).
//
// joint_strength_search_dual runs once per bit count i = 0..3 (nb = 1 << i
// strengths: nb greedy search_one_dual steps, then 4 nb refinement steps)
// and the four searches are independent, so each runs on its own cluster
// (16 CTAs where the device allows it, else 8; critical path: the 40 steps
// of i = 3). The filter blocks are split into one contiguous range per CTA;
// each CTA compacts
// the rows of its range (column-major u32: every per-filter-block mse is
// below 2^29 -- at most 4096 px x 1023^2 >> 4 per plane, times sub <= 4 --
// so the u32 copy is lossless and a luma + chroma row sum fits u32) into
// its shared memory.
//
// One step: warp w sums pairs w, w + 16, ... over the CTA's rows (lanes
// stride the rows, shuffle reduction), lane 0 writes the pair's partial to
// a double-buffered array, one cluster barrier, then every warp adds the
// cluster's partials over distributed shared memory and takes the argmin
// itself (strict <, lowest pair index on ties), keeping its own copy of the
// chosen strengths -- so a step has one barrier. The cluster that finishes
// last (a counter in the frame descriptor) picks the bit count with the
// lowest RD cost (strict <, in i order) and writes the per-fb indices.
constexpr int kFinCluster = 8;      // portable cluster size (the fallback)
constexpr int kFinClusterMax = 16;  // non-portable cluster size, where the device allows it
constexpr int kFinThreads = 512;
constexpr int kFinWarps = kFinThreads / 32;
constexpr int kFinRowsPerLane = 8;  // register-cached best for up to 256 rows per CTA
// Pair-per-thread steps: frames with at least kFinWideMinPairs strength
// pairs (20 or 48 candidates) and at most kFinBstMax rows per CTA.
constexpr int kFinWideMinPairs = 256;
constexpr int kFinBstMax = 512;

__global__ void __launch_bounds__(kFinThreads, 1)
    k_cdef_finish(FrameDesc *frames, const int *frame_ids, int smem_bytes) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    // dynamic: the double-buffered pair partials, then (when they fit) the
    // compacted rows and their filter-block ids
    extern __shared__ __align__(16) unsigned long long dyn64[];
    __shared__ uint8_t wlev[kFinWarps][2][16];
    __shared__ int scan[kFinThreads];
    __shared__ int local_sb, last_flag;
    const int rank = (int)cl.block_rank();
    const int CL = (int)cl.num_blocks();  // cluster size chosen at launch (8 or 16)
    const int cluster = blockIdx.x / CL;
    const int level = cluster % kFinLevels;
    FrameDesc &f = frames[frame_ids[cluster / kFinLevels]];
    CdefParams &cp = f.cdef;
    if (cp.mode != 1) return;  // uniform over the cluster
    const int nfb = f.nhfb * f.nvfb, n_cand = cp.ncand, n2 = 2 * n_cand, npairs = n_cand * n_cand;
    const int T = blockDim.x, t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int fb0 = (int)((int64_t)nfb * rank / CL), fb1 = (int)((int64_t)nfb * (rank + 1) / CL);
    // compaction of this range's filter blocks with rows, in fb order
    const int span = fb1 - fb0, chunk = (span + T - 1) / T;
    const int c0 = fb0 + min(span, t * chunk), c1 = fb0 + min(span, t * chunk + chunk);
    int cnt = 0;
    for (int fb = c0; fb < c1; ++fb) cnt += f.fb_row[fb];
    scan[t] = cnt;
    __syncthreads();
    for (int o = 1; o < T; o <<= 1) {
        const int v = t >= o ? scan[t - o] : 0;
        __syncthreads();
        scan[t] += v;
        __syncthreads();
    }
    const int sbr = scan[T - 1];
    // Pair partials, reduce-scatter: pair p is owned by rank p % CL; every
    // CTA stores its partial of p into the owner's inbox[buf][src rank][p /
    // CL] (one remote store per pair), the owners sum their pairs and take
    // the argmin over them, and the CL (best, pair) results are gathered
    // into every rank (one remote store per rank).
    const int owned = (npairs + CL - 1) / CL;
    const int pslots = CL * owned;
    unsigned long long *tot[2] = {dyn64, dyn64 + pslots};
    __shared__ unsigned long long g_bv[2][kFinClusterMax];
    __shared__ int g_bi[2][kFinClusterMax];
    uint32_t *dyn = reinterpret_cast<uint32_t *>(dyn64 + 2 * pslots);
    // rows in shared memory take an odd column stride where it fits (the
    // pair-per-thread step reads 20 or 48 columns at one row per lane: an
    // odd stride puts them in distinct banks); the global fallback keeps
    // the stride its slice was sized for
    const size_t pbytes = (size_t)2 * pslots * 8;
    const bool in_smem = pbytes + (size_t)sbr * (n2 + 1) * 4 <= (size_t)smem_bytes;
    const bool wide = npairs >= kFinWideMinPairs && sbr <= kFinBstMax;
    // the pair-per-thread step reads four rows of a column per 16-byte load:
    // columns 16-byte aligned at a stride of an odd multiple of 16 bytes, so
    // the eight loads of a quarter warp (eight columns) hit distinct banks;
    // the warp-per-pair step wants an odd word stride
    const int sbq = (sbr + 3) / 8 * 8 + 4, sbo = sbr | 1;
    auto fits = [&](int st) { return in_smem && pbytes + ((size_t)st * n2 + sbr) * 4 <= (size_t)smem_bytes; };
    const int sbp = wide && fits(sbq) ? sbq : !wide && fits(sbo) ? sbo : sbr;
    const bool quad = wide && sbp == sbq;
    uint32_t *R = in_smem ? dyn : f.cdef_rows32 + ((size_t)level * nfb + fb0) * n2;
    int *ids = in_smem ? reinterpret_cast<int *>(dyn + (size_t)sbp * n2) : f.cdef_ids + (size_t)level * nfb + fb0;
    {
        int pos = scan[t] - cnt;
        for (int fb = c0; fb < c1; ++fb)
            if (f.fb_row[fb]) ids[pos++] = fb;
    }
    if (t == 0) local_sb = sbr;
    cl.sync();
    int sb = 0;
    for (int r = 0; r < CL; ++r) sb += *cl.map_shared_rank(&local_sb, r);
    if (sb == 0) {  // every filter block all-skip: cdef.rs:282-288
        if (level == 0) {
            for (int fb = fb0 + t; fb < fb1; fb += T) f.fb_idx[fb] = 0;
            if (rank == 0 && t == 0) {
                cp.bits = 0;
                cp.y_str[0] = 0;
                cp.uv_str[0] = 0;
            }
        }
        cl.sync();
        return;
    }
    for (int q = t; q < sbr * n2; q += T) {
        const int k = q / sbr, s = q - k * sbr;  // column-major: R[k * sbp + s]
        R[k * sbp + s] = (uint32_t)f.mse[(int64_t)ids[s] * n2 + k];
    }
    if (lane < 16) {
        wlev[warp][0][lane] = 0;
        wlev[warp][1][lane] = 0;
    }
    __syncthreads();
    uint8_t *lev0 = wlev[warp][0], *lev1 = wlev[warp][1];

    int buf = 0;
    // One search_one_dual step (cdef.rs:824-862) over the whole frame for
    // strength slot nbs; returns the best total and records the pair.
    __shared__ __align__(16) uint32_t bsts[kFinBstMax];
    auto step = [&](int nbs) -> unsigned long long {
        if (wide) {
            // the best of the fixed strengths per row, then one pair per
            // thread over all of the CTA's rows: no cross-lane reduction
            for (int s = t; s < sbr; s += T) {
                uint32_t b = 0xffffffffu;  // +infinity for an empty strength set
                for (int gi = 0; gi < nbs; ++gi) {
                    const uint32_t c = R[lev0[gi] * sbp + s] + R[(n_cand + lev1[gi]) * sbp + s];
                    b = c < b ? c : b;
                }
                bsts[s] = b;
            }
            __syncthreads();
            for (int p = t; p < npairs; p += T) {
                const int j = p / n_cand, k = p - j * n_cand;
                const uint32_t *rj = R + (size_t)j * sbp, *rk = R + (size_t)(n_cand + k) * sbp;
                unsigned long long acc = 0;
                int s = 0;
                // four rows per u32 partial: each min is below 2^30
                if (quad)
                    for (; s + 4 <= sbr; s += 4) {
                        const uint4 a = *reinterpret_cast<const uint4 *>(rj + s);
                        const uint4 b = *reinterpret_cast<const uint4 *>(rk + s);
                        const uint4 c = *reinterpret_cast<const uint4 *>(bsts + s);
                        acc += min(a.x + b.x, c.x) + min(a.y + b.y, c.y) + min(a.z + b.z, c.z) + min(a.w + b.w, c.w);
                    }
                for (; s + 4 <= sbr; s += 4) {
                    uint32_t m = 0;
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const uint32_t c = rj[s + u] + rk[s + u], b = bsts[s + u];
                        m += c < b ? c : b;
                    }
                    acc += m;
                }
                for (; s < sbr; ++s) {
                    const uint32_t c = rj[s] + rk[s], b = bsts[s];
                    acc += c < b ? c : b;
                }
                *cl.map_shared_rank(tot[buf] + rank * owned + p / CL, p % CL) = acc;
            }
        }
        const bool cached = !wide && sbr <= 32 * kFinRowsPerLane;
        uint32_t bst[kFinRowsPerLane];
        if (cached) {
#pragma unroll
            for (int r = 0; r < kFinRowsPerLane; ++r) {
                const int s = lane + 32 * r;
                uint32_t b = 0xffffffffu;  // +infinity for an empty strength set
                if (s < sbr)
                    for (int gi = 0; gi < nbs; ++gi) {
                        const uint32_t c = R[lev0[gi] * sbp + s] + R[(n_cand + lev1[gi]) * sbp + s];
                        b = c < b ? c : b;
                    }
                bst[r] = b;
            }
        }
        for (int p = warp; p < npairs && !wide; p += kFinWarps) {
            const int j = p / n_cand, k = p - j * n_cand;
            const uint32_t *rj = R + (size_t)j * sbp, *rk = R + (size_t)(n_cand + k) * sbp;
            unsigned long long acc = 0;
            if (cached) {
#pragma unroll
                for (int r = 0; r < kFinRowsPerLane; ++r) {
                    const int s = lane + 32 * r;
                    if (s < sbr) {
                        const uint32_t c = rj[s] + rk[s];
                        acc += c < bst[r] ? c : bst[r];
                    }
                }
            } else {
                for (int s = lane; s < sbr; s += 32) {
                    uint32_t b = 0xffffffffu;
                    for (int gi = 0; gi < nbs; ++gi) {
                        const uint32_t c = R[lev0[gi] * sbp + s] + R[(n_cand + lev1[gi]) * sbp + s];
                        b = c < b ? c : b;
                    }
                    const uint32_t c = rj[s] + rk[s];
                    acc += c < b ? c : b;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (lane == 0) *cl.map_shared_rank(tot[buf] + rank * owned + p / CL, p % CL) = acc;
        }
        cl.sync();  // partials of this step delivered to their owners
        // warp 0: the argmin over this rank's pairs p = rank + CL k, then the
        // (best, pair) into every rank's gather slot
        if (warp == 0) {
            unsigned long long bv = ~0ull;
            int bi = 0x7fffffff;
            for (int k = lane; k < owned; k += 32) {
                const int p = rank + CL * k;
                if (p >= npairs) break;
                unsigned long long v = 0;
                for (int r = 0; r < CL; ++r) v += tot[buf][r * owned + k];
                if (v < bv) {  // p increases along a lane: strict < keeps the lowest
                    bv = v;
                    bi = p;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const unsigned long long ov = __shfl_xor_sync(0xffffffffu, bv, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ov < bv || (ov == bv && oi < bi)) {
                    bv = ov;
                    bi = oi;
                }
            }
            if (lane < CL) {
                *cl.map_shared_rank(&g_bv[buf][rank], lane) = bv;
                *cl.map_shared_rank(&g_bi[buf][rank], lane) = bi;
            }
        }
        cl.sync();  // every rank's best delivered everywhere
        unsigned long long bv = lane < CL ? g_bv[buf][lane] : ~0ull;
        int bi = lane < CL ? g_bi[buf][lane] : 0x7fffffff;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long ov = __shfl_xor_sync(0xffffffffu, bv, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov < bv || (ov == bv && oi < bi)) {
                bv = ov;
                bi = oi;
            }
        }
        if (bv >= (1ull << 63)) {  // best_tot starts at 1 << 63 with strict <
            bi = 0;
            bv = 1ull << 63;
        }
        if (lane == 0) {
            lev0[nbs] = (uint8_t)(bi / n_cand);
            lev1[nbs] = (uint8_t)(bi % n_cand);
        }
        __syncwarp();
        buf ^= 1;
        return bv;
    };

    const int nb = 1 << level;
    unsigned long long tt = 1ull << 63;
    for (int s = 0; s < nb; ++s) tt = step(s);
    for (int r = 0; r < 4 * nb; ++r) {
        if (lane == 0)
            for (int j = 0; j < nb - 1; ++j) {
                lev0[j] = lev0[j + 1];
                lev1[j] = lev1[j + 1];
            }
        __syncwarp();
        tt = step(nb - 1);
    }
    // publish this bit count's result; the last cluster of the frame decides
    if (rank == 0 && t == 0) {
        const unsigned long long total_bits = (unsigned long long)sb * level + nb * 12;
        f.fin_cost[level] = rdc(cp.lambda, total_bits << 9, tt * 16);
        for (int k = 0; k < 8; ++k) {
            f.fin_lev[level][k] = k < nb ? lev0[k] : 0;
            f.fin_lev[level][8 + k] = k < nb ? lev1[k] : 0;
        }
        __threadfence();
        last_flag = atomicAdd(&f.fin_done, 1) == kFinLevels - 1;
    }
    cl.sync();
    const bool last = *cl.map_shared_rank(&last_flag, 0) != 0;
    cl.sync();  // rank 0's shared memory must outlive every CTA's read of it
    if (!last) return;
    __threadfence();
    __shared__ int best_bits;
    __shared__ uint8_t blev[16];
    if (t == 0) {
        unsigned long long best_cost = 1ull << 63;
        int bb = 0;
        for (int i = 0; i < kFinLevels; ++i) {
            const unsigned long long c = __ldcg(&f.fin_cost[i]);
            if (c < best_cost) {
                best_cost = c;
                bb = i;
            }
        }
        best_bits = bb;
        for (int k = 0; k < 16; ++k) blev[k] = *(volatile uint8_t *)&f.fin_lev[bb][k];
    }
    __syncthreads();
    const int bnb = 1 << best_bits;
    for (int fb = fb0 + t; fb < fb1; fb += T) f.fb_idx[fb] = 0;
    __syncthreads();
    for (int s = t; s < sbr; s += T) {
        int best_gi = 0;
        unsigned long long bst = ~0ull;
        for (int gi = 0; gi < bnb; ++gi) {
            const unsigned long long c = (unsigned long long)R[blev[gi] * sbp + s] + R[(n_cand + blev[8 + gi]) * sbp + s];
            if (c < bst) {
                bst = c;
                best_gi = gi;
            }
        }
        f.fb_idx[ids[s]] = (uint8_t)best_gi;
    }
    if (rank == 0 && t == 0) {
        cp.bits = best_bits;
        for (int gi = 0; gi < 8; ++gi) {
            cp.y_str[gi] = gi < bnb ? (uint8_t)cp.fs[blev[gi]] : 0;
            cp.uv_str[gi] = gi < bnb ? (uint8_t)cp.fs[blev[8 + gi]] : 0;
        }
    }
}

// The same joint search with one 1024-thread CTA per (frame, bit count),
// for frames whose rows fit in one CTA's shared memory: no cluster
// barriers, rows padded to a multiple of 4 (zero rows add 0) and read as
// uint4. A step: the best of the fixed strengths per row into shared
// memory; then warps take (pair, row chunk) tasks -- four rows per lane per
// load, summed in u32 (each min < 2^30, four < 2^32) into a u64 -- and
// write per-task partials; warp 0 adds the chunks of each pair and takes the
// argmin (strict <, lowest pair index on ties). The last CTA of a frame
// picks the bit count as the cluster form does.
constexpr int kFin1Threads = 1024;
constexpr int kFin1Warps = kFin1Threads / 32;

__global__ void __launch_bounds__(kFin1Threads, 1) k_cdef_finish1(FrameDesc *frames, const int *frame_ids) {
    extern __shared__ __align__(16) unsigned char fin1_dyn[];
    __shared__ int scan[kFin1Threads];
    __shared__ uint8_t lev[2][16];
    __shared__ unsigned long long res_v;
    __shared__ int last_flag, best_bits;
    const int level = blockIdx.x % kFinLevels;
    FrameDesc &f = frames[frame_ids[blockIdx.x / kFinLevels]];
    CdefParams &cp = f.cdef;
    if (cp.mode != 1) return;
    const int nfb = f.nhfb * f.nvfb, n_cand = cp.ncand, n2 = 2 * n_cand, npairs = n_cand * n_cand;
    const int T = blockDim.x, t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int chunk = (nfb + T - 1) / T;
    const int c0 = min(nfb, t * chunk), c1 = min(nfb, t * chunk + chunk);
    int cnt = 0;
    for (int fb = c0; fb < c1; ++fb) cnt += f.fb_row[fb];
    scan[t] = cnt;
    __syncthreads();
    for (int o = 1; o < T; o <<= 1) {
        const int v = t >= o ? scan[t - o] : 0;
        __syncthreads();
        scan[t] += v;
        __syncthreads();
    }
    const int sb = scan[T - 1];
    if (sb == 0) {  // every filter block all-skip: cdef.rs:282-288
        if (level == 0) {
            for (int fb = t; fb < nfb; fb += T) f.fb_idx[fb] = 0;
            if (t == 0) {
                cp.bits = 0;
                cp.y_str[0] = 0;
                cp.uv_str[0] = 0;
            }
        }
        return;
    }
    const int nq = (sb + 3) >> 2, s4 = nq * 4;  // rows padded to a multiple of 4
    const int C = max(1, (4 * kFin1Warps + npairs - 1) / npairs);  // row chunks per pair
    const int ntasks = npairs * C;
    uint32_t *R = reinterpret_cast<uint32_t *>(fin1_dyn);  // R[k * s4 + s]
    uint32_t *best = R + (size_t)n2 * s4;
    unsigned long long *part = reinterpret_cast<unsigned long long *>(best + s4);
    int *ids = reinterpret_cast<int *>(part + ntasks);
    {
        int pos = scan[t] - cnt;
        for (int fb = c0; fb < c1; ++fb)
            if (f.fb_row[fb]) ids[pos++] = fb;
    }
    __syncthreads();
    for (int q = t; q < n2 * s4; q += T) {
        const int k = q / s4, s = q - k * s4;
        R[q] = s < sb ? (uint32_t)f.mse[(int64_t)ids[s] * n2 + k] : 0u;
    }
    if (t < 16) lev[0][t] = lev[1][t] = 0;
    __syncthreads();
    const uint4 *R4 = reinterpret_cast<const uint4 *>(R);
    uint4 *best4 = reinterpret_cast<uint4 *>(best);

    auto step = [&](int nbs) -> unsigned long long {
        for (int q = t; q < nq; q += T) {
            uint4 b = make_uint4(0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu);
            for (int gi = 0; gi < nbs; ++gi) {
                const uint4 a = R4[(size_t)lev[0][gi] * nq + q], c = R4[(size_t)(n_cand + lev[1][gi]) * nq + q];
                b.x = min(b.x, a.x + c.x);
                b.y = min(b.y, a.y + c.y);
                b.z = min(b.z, a.z + c.z);
                b.w = min(b.w, a.w + c.w);
            }
            best4[q] = b;
        }
        __syncthreads();
        for (int task = warp; task < ntasks; task += kFin1Warps) {
            const int p = task / C, c = task - p * C;
            const int j = p / n_cand, k = p - j * n_cand;
            const uint4 *rj = R4 + (size_t)j * nq, *rk = R4 + (size_t)(n_cand + k) * nq;
            const int q0 = (int)((int64_t)nq * c / C), q1 = (int)((int64_t)nq * (c + 1) / C);
            unsigned long long acc = 0;
            for (int q = q0 + lane; q < q1; q += 32) {
                const uint4 a = rj[q], b = rk[q], m = best4[q];
                acc += (unsigned long long)(min(a.x + b.x, m.x) + min(a.y + b.y, m.y) + min(a.z + b.z, m.z) +
                                            min(a.w + b.w, m.w));
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
            if (lane == 0) part[task] = acc;
        }
        __syncthreads();
        if (warp == 0) {
            unsigned long long bv = ~0ull;
            int bi = 0x7fffffff;
            for (int p = lane; p < npairs; p += 32) {
                unsigned long long v = 0;
                for (int c = 0; c < C; ++c) v += part[p * C + c];
                if (v < bv) {
                    bv = v;
                    bi = p;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const unsigned long long ov = __shfl_xor_sync(0xffffffffu, bv, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ov < bv || (ov == bv && oi < bi)) {
                    bv = ov;
                    bi = oi;
                }
            }
            if (bv >= (1ull << 63)) {  // best_tot starts at 1 << 63 with strict <
                bi = 0;
                bv = 1ull << 63;
            }
            if (lane == 0) {
                lev[0][nbs] = (uint8_t)(bi / n_cand);
                lev[1][nbs] = (uint8_t)(bi % n_cand);
                res_v = bv;
            }
        }
        __syncthreads();
        return res_v;
    };

    const int nb = 1 << level;
    unsigned long long tt = 1ull << 63;
    for (int s = 0; s < nb; ++s) tt = step(s);
    for (int r = 0; r < 4 * nb; ++r) {
        if (t == 0)
            for (int j = 0; j < nb - 1; ++j) {
                lev[0][j] = lev[0][j + 1];
                lev[1][j] = lev[1][j + 1];
            }
        __syncthreads();
        tt = step(nb - 1);
    }
    if (t == 0) {
        const unsigned long long total_bits = (unsigned long long)sb * level + nb * 12;
        f.fin_cost[level] = rdc(cp.lambda, total_bits << 9, tt * 16);
        for (int k = 0; k < 8; ++k) {
            f.fin_lev[level][k] = k < nb ? lev[0][k] : 0;
            f.fin_lev[level][8 + k] = k < nb ? lev[1][k] : 0;
        }
        __threadfence();
        last_flag = atomicAdd(&f.fin_done, 1) == kFinLevels - 1;
    }
    __syncthreads();
    if (!last_flag) return;
    __threadfence();
    if (t == 0) {
        unsigned long long best_cost = 1ull << 63;
        int bb = 0;
        for (int i = 0; i < kFinLevels; ++i) {
            const unsigned long long c = __ldcg(&f.fin_cost[i]);
            if (c < best_cost) {
                best_cost = c;
                bb = i;
            }
        }
        best_bits = bb;
        for (int k = 0; k < 16; ++k) lev[k >> 3][k & 7] = *(volatile uint8_t *)&f.fin_lev[bb][k];
    }
    __syncthreads();
    const int bnb = 1 << best_bits;
    for (int fb = t; fb < nfb; fb += T) f.fb_idx[fb] = 0;
    __syncthreads();
    for (int s = t; s < sb; s += T) {
        int best_gi = 0;
        unsigned long long bst = ~0ull;
        for (int gi = 0; gi < bnb; ++gi) {
            const unsigned long long c =
                (unsigned long long)R[(size_t)lev[0][gi] * s4 + s] + R[(size_t)(n_cand + lev[1][gi]) * s4 + s];
            if (c < bst) {
                bst = c;
                best_gi = gi;
            }
        }
        f.fb_idx[ids[s]] = (uint8_t)best_gi;
    }
    if (t == 0) {
        cp.bits = best_bits;
        for (int gi = 0; gi < 8; ++gi) {
            cp.y_str[gi] = gi < bnb ? (uint8_t)cp.fs[lev[0][gi]] : 0;
            cp.uv_str[gi] = gi < bnb ? (uint8_t)cp.fs[lev[1][gi]] : 0;
        }
    }
}

// ---- finish for the small candidate sets (4 or 6 candidates: presets 4-6)
//
// One kJointThreads-thread CTA per (frame, bit count), no cluster. Thread t
// owns the filter blocks t + r * kJointThreads (r < RPT) and their rows stay
// in shared memory at R[k][r * kJointThreads + t]; a block without a row (or
// past the frame) is a zero row, which adds 0 to every total, so rows need
// no compaction. The costs of the strengths in the current set are a shift
// register per owned row in registers: the best over the set (the reference's
// per-row `best`) costs a few register mins, not a pass over the set.
//
// Bounds: a row's luma entry is below 2^28 (<= 4096 px x 1023^2 >> 4, or x
// 255^2 at 8 bits, the subsampled sum times sub never exceeding the full
// block) and its joint chroma entry below 2^27, so a pair cost is below
// 3 * 2^27 and up to 5 rows per thread sum exactly in u32 -- two lanes of
// such sums still fit u32, the first reduce stage stays 32-bit.
//
// One step: per thread the NC^2 pair totals over its rows (min(l + c, best)
// by one add-min), a warp reduce-scatter that leaves each pair's warp sum in
// a lane, one partial per (warp, pair) in shared memory, a barrier, the sums
// and argmin in warp 0 (strict <, lowest pair index on ties), a barrier.
constexpr int kJointThreads = 512;
constexpr int kJointWarps = kJointThreads / 32;

// Warp reduce-scatter of N u32 values held by every lane (N = 4, 16 or 32;
// each value below 2^31): the sum over the warp of value i is written to
// out[i] by the lanes that end up holding it.
template <int N>
__device__ __forceinline__ void warp_scatter_sum(const uint32_t *v, int lane, unsigned long long *out) {
    static_assert(N == 4 || N == 16 || N == 32, "N");
    constexpr int H = N / 2;
    unsigned long long b[H];
    int idx = 0;
    {
        const bool up = (lane & 16) != 0;
#pragma unroll
        for (int i = 0; i < H; ++i) {
            const uint32_t s = up ? v[i] : v[i + H], k = up ? v[i + H] : v[i];
            b[i] = (unsigned long long)(k + __shfl_xor_sync(0xffffffffu, s, 16));
        }
        if (up) idx += H;
    }
#pragma unroll
    for (int st = 0; st < 4; ++st) {
        const int o = 8 >> st, n = H >> st;  // values held before this stage
        if (n > 1) {
            const int h = n >> 1;
            const bool up = (lane & o) != 0;
#pragma unroll
            for (int i = 0; i < h; ++i) {
                const unsigned long long s = up ? b[i] : b[i + h], k = up ? b[i + h] : b[i];
                b[i] = k + __shfl_xor_sync(0xffffffffu, s, o);
            }
            if (up) idx += h;
        } else {
            b[0] += __shfl_xor_sync(0xffffffffu, b[0], o);
        }
    }
    out[idx] = b[0];  // lanes holding the same index write the same sum
}

// joint_strength_search_dual (cdef.rs:866-885) for nb = NB strengths over
// the CTA's rows; returns the last step's total and leaves the strengths in
// lev[0][0..NB) (luma) and lev[1][0..NB) (chroma).
template <int NC, int RPT, int NB>
__device__ __forceinline__ unsigned long long joint_search(const uint32_t *R, unsigned long long *part,
                                                           uint8_t (*lev)[16], int *spick,
                                                           unsigned long long *sres) {
    constexpr int P = NC * NC, T = kJointThreads, S = T * RPT;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    uint32_t pc[RPT][NB];  // costs of the set's strengths, oldest first
    uint32_t bg[RPT];      // greedy phase: best over the strengths picked so far
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
        bg[r] = 0xffffffffu;
#pragma unroll
        for (int g = 0; g < NB; ++g) pc[r][g] = 0;
    }
    unsigned long long tt = 1ull << 63;
    for (int step = 0; step < 5 * NB; ++step) {
        const bool refine = step >= NB;
        uint32_t acc[P];
#pragma unroll
        for (int p = 0; p < P; ++p) acc[p] = 0;
#pragma unroll
        for (int r = 0; r < RPT; ++r) {
            // refinement: the set is the newest NB - 1 strengths (the
            // reference drops its oldest before the search)
            uint32_t bst = bg[r];
            if (refine) {
                bst = 0xffffffffu;
#pragma unroll
                for (int g = 1; g < NB; ++g) bst = min(bst, pc[r][g]);
            }
            uint32_t rl[NC], rc[NC];
#pragma unroll
            for (int k = 0; k < NC; ++k) {
                rl[k] = R[k * S + r * T + t];
                rc[k] = R[(NC + k) * S + r * T + t];
            }
#pragma unroll
            for (int j = 0; j < NC; ++j)
#pragma unroll
                for (int k = 0; k < NC; ++k) acc[j * NC + k] += __viaddmin_u32(rl[j], rc[k], bst);
        }
        if constexpr (P == 16) {
            warp_scatter_sum<16>(acc, lane, part + warp * P);
        } else {
            warp_scatter_sum<32>(acc, lane, part + warp * P);
            warp_scatter_sum<4>(acc + 32, lane, part + warp * P + 32);
        }
        __syncthreads();
        if (warp == 0) {
            unsigned long long bv = ~0ull;
            int bi = 0x7fffffff;
            for (int p = lane; p < P; p += 32) {
                unsigned long long v = 0;
#pragma unroll
                for (int w = 0; w < kJointWarps; ++w) v += part[w * P + p];
                if (v < bv) {  // p increases along a lane: strict < keeps the lowest
                    bv = v;
                    bi = p;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const unsigned long long ov = __shfl_xor_sync(0xffffffffu, bv, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ov < bv || (ov == bv && oi < bi)) {
                    bv = ov;
                    bi = oi;
                }
            }
            if (bv >= (1ull << 63)) {  // best_tot starts at 1 << 63 with strict <
                bi = 0;
                bv = 1ull << 63;
            }
            if (lane == 0) {
                *spick = bi;
                *sres = bv;
                const int slot = refine ? NB - 1 : step;
                if (refine)
                    for (int g = 0; g < NB - 1; ++g) {
                        lev[0][g] = lev[0][g + 1];
                        lev[1][g] = lev[1][g + 1];
                    }
                lev[0][slot] = (uint8_t)(bi / NC);
                lev[1][slot] = (uint8_t)(bi % NC);
            }
        }
        __syncthreads();
        const int bi = *spick, j = bi / NC, k = bi - j * NC;
        tt = *sres;
#pragma unroll
        for (int r = 0; r < RPT; ++r) {
            const uint32_t c = R[j * S + r * T + t] + R[(NC + k) * S + r * T + t];
            bg[r] = min(bg[r], c);
#pragma unroll
            for (int g = 0; g + 1 < NB; ++g) pc[r][g] = pc[r][g + 1];
            pc[r][NB - 1] = c;
        }
    }
    return tt;
}

template <int NC, int RPT>
__global__ void __launch_bounds__(kJointThreads, 1) k_cdef_joint(FrameDesc *frames, const int *frame_ids) {
    extern __shared__ __align__(16) unsigned char joint_dyn[];
    constexpr int T = kJointThreads, S = T * RPT, P = NC * NC;
    __shared__ unsigned long long part[kJointWarps * P];
    __shared__ uint8_t lev[2][16];
    __shared__ unsigned long long res_v;
    __shared__ int pick, last_flag, best_bits;
    const int level = blockIdx.x % kFinLevels;
    FrameDesc &f = frames[frame_ids[blockIdx.x / kFinLevels]];
    CdefParams &cp = f.cdef;
    if (cp.mode != 1) return;
    const int nfb = f.nhfb * f.nvfb, n2 = 2 * NC, t = threadIdx.x;
    uint32_t *R = reinterpret_cast<uint32_t *>(joint_dyn);  // R[k * S + slot]
    // rows of the owned blocks: every load issued before the stores, one
    // barrier for the row count
    __shared__ int s_rows;
    if (t == 0) s_rows = 0;
    int mine = 0;
    {
        bool row[RPT];
#pragma unroll
        for (int r = 0; r < RPT; ++r) {
            const int fb = r * T + t;
            row[r] = fb < nfb && f.fb_row[fb];
            mine += row[r];
        }
        uint32_t v[RPT][2 * NC];
#pragma unroll
        for (int r = 0; r < RPT; ++r) {
            const uint64_t *m = f.mse + (int64_t)(r * T + t) * n2;
#pragma unroll
            for (int k = 0; k < 2 * NC; ++k) v[r][k] = row[r] ? (uint32_t)m[k] : 0u;
        }
#pragma unroll
        for (int r = 0; r < RPT; ++r)
#pragma unroll
            for (int k = 0; k < 2 * NC; ++k) R[k * S + r * T + t] = v[r][k];
    }
    __syncthreads();
    if (mine) atomicAdd(&s_rows, mine);
    __syncthreads();
    const int sb = s_rows;
    if (sb == 0) {  // every filter block all-skip: cdef.rs:282-288
        if (level == 0) {
            for (int fb = t; fb < nfb; fb += T) f.fb_idx[fb] = 0;
            if (t == 0) {
                cp.bits = 0;
                cp.y_str[0] = 0;
                cp.uv_str[0] = 0;
            }
        }
        return;
    }
    if (t < 16) lev[0][t] = lev[1][t] = 0;
    __syncthreads();
    unsigned long long tt;
    switch (level) {
        case 0: tt = joint_search<NC, RPT, 1>(R, part, lev, &pick, &res_v); break;
        case 1: tt = joint_search<NC, RPT, 2>(R, part, lev, &pick, &res_v); break;
        case 2: tt = joint_search<NC, RPT, 4>(R, part, lev, &pick, &res_v); break;
        default: tt = joint_search<NC, RPT, 8>(R, part, lev, &pick, &res_v); break;
    }
    const int nb = 1 << level;
    if (t == 0) {
        const unsigned long long total_bits = (unsigned long long)sb * level + nb * 12;
        f.fin_cost[level] = rdc(cp.lambda, total_bits << 9, tt * 16);
        for (int k = 0; k < 8; ++k) {
            f.fin_lev[level][k] = k < nb ? lev[0][k] : 0;
            f.fin_lev[level][8 + k] = k < nb ? lev[1][k] : 0;
        }
        __threadfence();
        last_flag = atomicAdd(&f.fin_done, 1) == kFinLevels - 1;
    }
    __syncthreads();
    if (!last_flag) return;
    __threadfence();
    if (t == 0) {
        unsigned long long best_cost = 1ull << 63;
        int bb = 0;
        for (int i = 0; i < kFinLevels; ++i) {
            const unsigned long long c = __ldcg(&f.fin_cost[i]);
            if (c < best_cost) {
                best_cost = c;
                bb = i;
            }
        }
        best_bits = bb;
        for (int k = 0; k < 16; ++k) lev[k >> 3][k & 7] = *(volatile uint8_t *)&f.fin_lev[bb][k];
    }
    __syncthreads();
    const int bnb = 1 << best_bits;
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
        const int fb = r * T + t;
        if (fb >= nfb) continue;
        int best_gi = 0;
        if (f.fb_row[fb]) {
            unsigned long long bst = ~0ull;
            for (int gi = 0; gi < bnb; ++gi) {
                const unsigned long long c = (unsigned long long)R[lev[0][gi] * S + fb] + R[(NC + lev[1][gi]) * S + fb];
                if (c < bst) {
                    bst = c;
                    best_gi = gi;
                }
            }
        }
        f.fb_idx[fb] = (uint8_t)best_gi;
    }
    if (t == 0) {
        cp.bits = best_bits;
        for (int gi = 0; gi < 8; ++gi) {
            cp.y_str[gi] = gi < bnb ? (uint8_t)cp.fs[lev[0][gi]] : 0;
            cp.uv_str[gi] = gi < bnb ? (uint8_t)cp.fs[lev[1][gi]] : 0;
        }
    }
}

// Rows per thread k_cdef_joint needs for a frame: 1, 2 or 4; 0 when the
// frame is outside its range (other candidate counts, more filter blocks).
int joint_rows_per_thread(int nfb, int ncand) {
    if (ncand != 4 && ncand != 6) return 0;
    for (int rpt = 1; rpt <= 4; rpt *= 2)
        if (nfb <= rpt * kJointThreads) return rpt;
    return 0;
}

size_t joint_smem(int ncand, int rpt) { return (size_t)2 * ncand * kJointThreads * rpt * 4; }

cudaError_t launch_cdef_joint(int ncand, int rpt, int nframes, cudaStream_t st, FrameDesc *frames,
                              const int *frame_ids) {
    const size_t smem = joint_smem(ncand, rpt);
    const dim3 grid((unsigned)(nframes * kFinLevels));
#define ZF_JOINT(NC, RPT)                                                                              \
    if (ncand == NC && rpt == RPT) {                                                                   \
        k_cdef_joint<NC, RPT><<<grid, kJointThreads, smem, st>>>(frames, frame_ids);                   \
        return cudaGetLastError();                                                                     \
    }
    ZF_JOINT(4, 1) ZF_JOINT(4, 2) ZF_JOINT(4, 4) ZF_JOINT(6, 1) ZF_JOINT(6, 2) ZF_JOINT(6, 4)
#undef ZF_JOINT
    return cudaErrorInvalidValue;
}

// Opt k_cdef_joint's instantiations into their dynamic shared memory.
cudaError_t joint_set_attributes() {
    cudaError_t e = cudaSuccess;
#define ZF_JOINT_ATTR(NC, RPT)                                                                              \
    if (e == cudaSuccess)                                                                                   \
        e = cudaFuncSetAttribute(k_cdef_joint<NC, RPT>, cudaFuncAttributeMaxDynamicSharedMemorySize,        \
                                 (int)joint_smem(NC, RPT));
    ZF_JOINT_ATTR(4, 1) ZF_JOINT_ATTR(4, 2) ZF_JOINT_ATTR(4, 4) ZF_JOINT_ATTR(6, 1) ZF_JOINT_ATTR(6, 2)
    ZF_JOINT_ATTR(6, 4)
#undef ZF_JOINT_ATTR
    return e;
}

// Launch k_cdef_finish for `nclusters` (frame, bit count) clusters of `cl`
// CTAs (the cluster size is a launch attribute; 16 needs the non-portable
// attribute, set once per device by finish_cluster_size).
cudaError_t launch_cdef_finish(int nclusters, int cl, size_t smem, cudaStream_t st, FrameDesc *frames,
                               const int *frame_ids, int smem_bytes) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(nclusters * cl));
    cfg.blockDim = dim3(kFinThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)cl;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_cdef_finish, frames, frame_ids, smem_bytes);
}

// The cluster size for k_cdef_finish with `smem` dynamic bytes: 16 when the
// device can co-schedule a 16-CTA cluster of this kernel, else 8.
int finish_cluster_size(size_t smem) {
    static std::mutex mu;
    static int allowed = -1;                      // non-portable sizes opted in (per process)
    static size_t last_smem = 0;
    static int last_size = 0;
    std::lock_guard<std::mutex> lk(mu);
    if (last_size && last_smem == smem) return last_size;
    if (allowed < 0) {
        allowed = cudaFuncSetAttribute(k_cdef_finish, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
                          cudaSuccess
                      ? 1
                      : 0;
        cudaGetLastError();
    }
    last_smem = smem;
    last_size = kFinCluster;
    if (!allowed) return kFinCluster;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kFinClusterMax);
    cfg.blockDim = dim3(kFinThreads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kFinClusterMax;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, k_cdef_finish, &cfg) != cudaSuccess || n < 1) {
        cudaGetLastError();
        return kFinCluster;
    }
    last_size = kFinClusterMax;
    return kFinClusterMax;
}

// Shared memory k_cdef_finish1 needs for a frame (0 when it does not fit).
int finish1_smem(int nfb, int ncand, int cap) {
    const int64_t s4 = ((int64_t)nfb + 3) / 4 * 4, n2 = 2 * ncand, npairs = (int64_t)ncand * ncand;
    const int64_t C = std::max<int64_t>(1, (4 * kFin1Warps + npairs - 1) / npairs);
    const int64_t bytes = (n2 * s4 + s4) * 4 + npairs * C * 8 + (int64_t)nfb * 4;
    return bytes <= cap ? (int)bytes : 0;
}

// ---- apply: one CTA per filter block, B (post-deblock) -> A -----------

// Out-of-line copies of the direction search and the skip mask for the
// apply, where they run once per filter block beside the hot filter loop
// (inlined there they crowd it out of the instruction cache; the search
// keeps them inlined, which measured faster for it).
__device__ __noinline__ void find_dirs_ool(const uint16_t *reg, int rs, int cs, const int *blist, int nblk,
                                           int (*cost)[8], int *sdir, int *svar) {
    find_dirs(reg, rs, cs, blist, nblk, cost, sdir, svar);
}
__device__ __noinline__ uint64_t fb_dlist_ool(const FrameDesc &f, int fbr, int fbc, unsigned *part) {
    return fb_dlist(f, fbr, fbc, part);
}

// Copy the n x n block at (x0, y0) of a pw x ph plane (clipped to it) from
// src to dst: 4-byte words when both planes are word aligned (plane widths
// and block columns are multiples of 4 samples, so a word never straddles
// the plane's right edge), samples otherwise.
__device__ void copy_block(const uint8_t *src, uint8_t *dst, int pw, int ph, int x0, int y0, int n, int bd) {
    const int rows = min(n, ph - y0), cols = min(n, pw - x0);
    if (aligned4(src) && aligned4(dst)) {
        const int spw = word_samples(bd), wpr = cols / spw, bps = bd == 8 ? 1 : 2;
        for (int q = threadIdx.x; q < rows * wpr; q += blockDim.x) {
            const int ry = q / wpr, wx = q - ry * wpr;
            const int64_t o = ((int64_t)(y0 + ry) * pw + x0) * bps + wx * 4;
            *reinterpret_cast<uint32_t *>(dst + o) = *reinterpret_cast<const uint32_t *>(src + o);
        }
        return;
    }
    for (int q = threadIdx.x; q < rows * cols; q += blockDim.x) {
        const int ry = q / cols, cx = q - ry * cols;
        const int64_t o = (int64_t)(y0 + ry) * pw + x0 + cx;
        stpx(dst, o, bd, ldpx(src, o, bd));
    }
}

__global__ void __launch_bounds__(256) k_cdef_apply(FrameDesc *frames, const WorkItem *items, int nitems) {
    __shared__ uint16_t reg[CR * CRP];
    __shared__ uint16_t regc[2][CRC * CRC];
    __shared__ int sdir[64], svar[64];
    __shared__ int dcost[64][8];
    __shared__ int boff[64][6], boffc[64][6];
    __shared__ int bt[64];  // luma: adjusted primary strength | damping shift << 16
    __shared__ int blist[64];
    __shared__ int nblk;
    __shared__ uint32_t s_count;  // filtered | changed << 16 (8-bit counters)
    const int it = find_item(items, nitems, blockIdx.x);
    const WorkItem wi = items[it];
    const FrameDesc &f = frames[wi.frame];
    const CdefParams &cp = f.cdef;
    const int fb = blockIdx.x - wi.cta_begin;
    const int fbr = fb / f.nhfb, fbc = fb - fbr * f.nhfb;
    const int bd = f.bd, cs = bd - 8;
    const int x0 = fbc * 64, y0 = fbr * 64;
    const int vsize = min(64, f.h - y0), hsize = min(64, f.w - x0);
    // Decoder do_cdef gate (cdef.rs:84-88).
    const bool any = cp.bits != 0 || cp.y_str[0] != 0 || (f.chroma && cp.uv_str[0] != 0);
    __shared__ unsigned dl_part[2];
    if (threadIdx.x == 0) s_count = 0;  // ordered before its adds by the barriers below
    const uint64_t dl_all = fb_dlist_ool(f, fbr, fbc, dl_part);
    if (threadIdx.x == 0) f.fb_row[fb] = dl_all != 0;
    const uint64_t dl = any ? dl_all : 0;
    if (dl == 0) {  // copy-through
        copy_block(f.B[0], f.A[0], f.w, f.h, x0, y0, 64, bd);
        if (f.chroma)
            for (int p = 1; p <= 2; ++p) copy_block(f.B[p], f.A[p], f.w / 2, f.h / 2, x0 / 2, y0 / 2, 32, bd);
        return;
    }
    const int sidx = cp.bits == 0 ? 0 : f.fb_idx[fb];
    const int ys = cp.y_str[sidx], uvs = f.chroma ? cp.uv_str[sidx] : 0;
    const int lvl_y = (ys / 4) << cs, sec_y = ((ys % 4) + ((ys % 4) == 3)) << cs;
    const int lvl_uv = (uvs / 4) << cs, sec_uv = ((uvs % 4) + ((uvs % 4) == 3)) << cs;
    const int damping = cp.damping + cs;
    const int cw = f.w / 2, ch = f.h / 2, cx0 = x0 / 2, cy0 = y0 / 2;
    // every plane's window staged at once (luma, then U and V)
    load_region(f.B[0], bd, f.w, f.h, x0, y0, 64, reg, CRP);
    if (f.chroma)
#pragma unroll 1
        for (int p = 0; p < 2; ++p) load_region(f.B[p + 1], bd, cw, ch, cx0, cy0, 32, regc[p], CRC);
    if (threadIdx.x == 0) {
        int n = 0;
        for (int b = 0; b < 64; ++b)
            if ((dl >> b) & 1) blist[n++] = b;
        nblk = n;
    }
    __syncthreads();
    // directions: from this call's search of the same B when it ran (a
    // frame-uniform branch), else found here
    const bool have_dirs = f.cdir_ok != 0;
    if (!have_dirs) find_dirs_ool(reg, CRP, cs, blist, nblk, dcost, sdir, svar);
    for (int k = threadIdx.x; k < nblk; k += blockDim.x) {
        const int b = blist[k];
        int dir, t;
        if (have_dirs) {
            const int c = f.cdir[(int64_t)fb * 64 + b];
            dir = c & 7;
            t = adjust_strength_code(lvl_y, c >> 3);
        } else {
            dir = sdir[b];
            t = adjust_strength(lvl_y, svar[b]);
        }
        dir_offsets(lvl_y ? dir : 0, CRP, boff[b]);
        dir_offsets(lvl_uv ? dir : 0, CRC, boffc[b]);
        bt[b] = t | (damp_shift(t, damping) << 16);
    }
    __syncthreads();
    uint32_t filt = 0, changed = 0;
    const bool edge_y = !(x0 >= 2 && y0 >= 2 && x0 + 66 <= f.w && y0 + 66 <= f.h);
    const bool edge_uv = !(x0 >= 4 && y0 >= 4 && x0 / 2 + 34 <= f.w / 2 && y0 / 2 + 34 <= f.h / 2);
    const bool zero_y = lvl_y == 0 && sec_y == 0;
    const int ssh_y = damp_shift(sec_y, damping);
    // a warp takes half an 8x8 block (4 rows x 8 columns), so whether the
    // block is filtered is uniform over the warp
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int h = warp; h < 128; h += nwarps) {
        const int b = h >> 1;
        const int py = (b >> 3) * 8 + (h & 1) * 4 + (lane >> 3), px = (b & 7) * 8 + (lane & 7);
        if (py >= vsize || px >= hsize) continue;
        const int pos = (py + 2) * CRP + px + 2;
        const int x = (int16_t)reg[pos];
        int y = x;
        if (!zero_y && ((dl >> b) & 1)) {
            const int tp = bt[b], t = tp & 0xffff;
            if (!(t == 0 && sec_y == 0)) {  // cdef.rs:444-448
                int d[12], mx, mn;
                load_taps_at(edge_y, reg, pos, boff[b], x, d, mx, mn);
                // a zero strength constrains every tap to 0 (its taps still
                // bound the clamp); t is uniform over the warp, sec_y over the CTA
                int sum = 0;
                if (t) sum += prim_sum(d, t, tp >> 16, cs);
                if (sec_y) sum += sec_sum(d, sec_y, ssh_y);
                y = cdef_round(x, sum, mn, mx);
                filt += 1;
                changed += y != x;
            }
        }
        stpx(f.A[0], (int64_t)(y0 + py) * f.w + x0 + px, bd, y);
    }
    if (f.chroma) {
        const bool zero_uv = lvl_uv == 0 && sec_uv == 0;
        const int psh = damp_shift(lvl_uv, damping - 1), ssh = damp_shift(sec_uv, damping - 1);
#pragma unroll 1
        for (int p = 1; p <= 2; ++p) {
            const uint16_t *rc = regc[p - 1];
            // a warp takes two horizontally adjacent 4x4 blocks
            for (int bp = warp; bp < 32; bp += nwarps) {
                const int b = 2 * bp + (lane >> 4);
                const int py = (b >> 3) * 4 + ((lane >> 2) & 3), px = (b & 7) * 4 + (lane & 3);
                if (py >= vsize / 2 || px >= hsize / 2) continue;
                const int pos = (py + 2) * CRC + px + 2;
                const int x = (int16_t)rc[pos];
                int y = x;
                if (!zero_uv && ((dl >> b) & 1)) {
                    int d[12], mx, mn;
                    load_taps_at(edge_uv, rc, pos, boffc[b], x, d, mx, mn);
                    int sum = 0;
                    if (lvl_uv) sum += prim_sum(d, lvl_uv, psh, cs);
                    if (sec_uv) sum += sec_sum(d, sec_uv, ssh);
                    y = cdef_round(x, sum, mn, mx);
                    filt += 1;
                    changed += y != x;
                }
                stpx(f.A[p], (int64_t)(cy0 + py) * cw + cx0 + px, bd, y);
            }
        }
    }
    if (bd == 8 && f.cdef_stats) {
        // a thread filters at most 24 pixels, a CTA at most 6144: both
        // counts fit 16 bits of one word through the warp and CTA sums
        uint32_t v = (uint32_t)filt | ((uint32_t)changed << 16);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) atomicAdd(&s_count, v);
        __syncthreads();
        if (threadIdx.x == 0) {
            atomicAdd(&f.cdef_stats[0], (unsigned long long)(s_count & 0xffffu));
            atomicAdd(&f.cdef_stats[1], (unsigned long long)(s_count >> 16));
        }
    }
}

}  // namespace zf

// ===========================================================================
// Allocation-free CDEF strength search (zf_cdef_search_noalloc).
//
// Some callers cannot allocate device memory once they are running: an
// encoder loop that reserves every byte at start-up and must not touch the
// allocator per frame, code that runs while another component holds a
// stream capture open on a different stream (cudaMalloc is not allowed
// then), or a process on a GPU slice whose memory is already fully
// reserved. For them this entry point runs the same two kernels as
// zf_cdef_search, with all scratch in the file-scope array below instead of
// a context arena. The array is sizeof(NoAllocScratch), about 1.9 MiB
// (mse rows 640 KiB, compacted rows 1.25 MiB, ids 32 KiB), and every GPU
// that loads the library holds it until the process exits. Limits: at most
// kNoAllocMaxFb 64x64 filter blocks (a 3840x2160 frame has 2040) and at
// most kNoAllocMaxCand candidate strengths (presets 1..6; preset 0's 48
// candidates are rejected).
// ===========================================================================

#include <mutex>

#include "../../include/zf_filter.h"

namespace zf {
int describe_cdef_frame(const zf_frame *f, FrameDesc *d);  // zf_host.cu

constexpr int kNoAllocMaxFb = 2048;
constexpr int kNoAllocMaxCand = 20;

struct NoAllocScratch {
    FrameDesc desc;
    WorkItem item;
    int frame_id;
    int pad;
    uint64_t mse[kNoAllocMaxFb * 2 * kNoAllocMaxCand];
    uint32_t rows32[kFinLevels * kNoAllocMaxFb * 2 * kNoAllocMaxCand];
    int ids[kFinLevels * kNoAllocMaxFb];
    uint8_t fb_row[kNoAllocMaxFb];
    uint8_t fb_idx[kNoAllocMaxFb];
};

static_assert(sizeof(NoAllocScratch) < 2u * 1024 * 1024, "allocation-free scratch stays below 2 MiB");

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Device address of g_noalloc_scratch, looked up with cudaGetSymbolAddress
// on the first call made with a device current and again whenever that
// device's current context changed since (a cudaDeviceReset or any other
// teardown of the primary context reloads the module at a new address).
constexpr int kMaxDevices = 64;
struct NoAllocAddr {
    CUcontext ctx;
    NoAllocScratch *ptr;
};
static NoAllocAddr g_noalloc_addr[kMaxDevices];
static std::mutex g_noalloc_mu;

// cuCtxGetCurrent from the driver (the library links the runtime only).
static CUresult current_context(CUcontext *out) {
    using Fn = CUresult (*)(CUcontext *);
    static Fn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            p = nullptr;
        }
        return reinterpret_cast<Fn>(p);
    }();
    return fn ? fn(out) : CUDA_ERROR_NOT_FOUND;
}
}  // namespace zf

extern "C" int32_t zf_cdef_search_noalloc(void *stream, const zf_frame *f, zf_decisions *out) {
    using namespace zf;
    if (!f || !out) return ZF_ERR_ARG;
    if (!f->planes_on_device) return ZF_ERR_ARG;
    FrameDesc d;
    int e = describe_cdef_frame(f, &d);
    if (e != ZF_OK) return e;
    const int nfb = d.nhfb * d.nvfb;
    out->nhfb = d.nhfb;
    out->nvfb = d.nvfb;
    if (d.cdef.mode != 1) {  // qp closed form: no device work (cdef.rs:151)
        out->cdef_damping = (uint8_t)d.cdef.damping;
        out->cdef_bits = 0;
        std::memset(out->cdef_y, 0, 8);
        std::memset(out->cdef_uv, 0, 8);
        out->cdef_y[0] = d.cdef.y_str[0];
        out->cdef_uv[0] = d.cdef.uv_str[0];
        if (out->cdef_fb_idx) std::memset(out->cdef_fb_idx, 0, nfb);
        return ZF_OK;
    }
    if (nfb > kNoAllocMaxFb) return ZF_ERR_INVALID_DIMS;   // frame larger than the static scratch
    if (d.cdef.ncand > kNoAllocMaxCand) return ZF_ERR_UNSUPPORTED;  // preset 0
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return ZF_ERR_CUDA;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // The call synchronises its stream and copies from host stack memory, so
    // it cannot be recorded into a graph: refuse a stream that is capturing
    // (or the legacy stream while another stream captures in global mode).
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return ZF_ERR_UNSUPPORTED;
    }
    NoAllocScratch *sc;
    {
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        CUcontext cur = nullptr;
        if (current_context(&cur) != CUDA_SUCCESS) cur = nullptr;
        NoAllocAddr &a = g_noalloc_addr[dev];
        if (!a.ptr || !cur || a.ctx != cur) {
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
                cudaGetLastError();
                a.ptr = nullptr;
                return ZF_ERR_CUDA;
            }
            // the runtime may have created the primary context just now
            if (!cur && current_context(&cur) != CUDA_SUCCESS) cur = nullptr;
            a.ctx = cur;
            a.ptr = static_cast<NoAllocScratch *>(p);
        }
        sc = a.ptr;
    }
    for (int p = 0; p < 3; ++p) {
        const bool on = p == 0 || f->chroma_420;
        d.B[p] = on ? (uint8_t *)f->rec[p] : nullptr;
        d.S[p] = on ? (const uint8_t *)f->src[p] : nullptr;
    }
    d.mi = f->mi;
    d.mse = sc->mse;
    d.fb_row = sc->fb_row;
    d.fb_idx = sc->fb_idx;
    d.cdef_ids = sc->ids;
    d.cdef_rows32 = sc->rows32;
    d.cdef_stats = nullptr;
    WorkItem item;
    item.frame = 0;
    item.plane = 0;
    item.a = item.b = 0;
    item.cta_begin = 0;
    item.ctas = nfb;
    const int frame_id = 0;
    // Every field the kernels read is rewritten here; the kernels write every
    // mse row, fb_row and fb_idx entry they later read, so nothing left from
    // a previous call is consumed.
    if (cudaMemcpyAsync(&sc->desc, &d, sizeof(d), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(&sc->item, &item, sizeof(item), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(&sc->frame_id, &frame_id, sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess)
        return ZF_ERR_CUDA;
    if (launch_cdef_search(d.cdef.first_pass_num, d.cdef.ncand / d.cdef.first_pass_num, nfb, st, &sc->desc,
                           &sc->item, 1) != cudaSuccess)
        return ZF_ERR_CUDA;
    // pair partials (an inbox per rank) + compacted rows (a padded column
    // stride) and ids: at most 51 + 44 KiB for ncand <= 20 and nfb <= 2048
    const int np = d.cdef.ncand * d.cdef.ncand;
    const int CL = kFinCluster;
    const int rows = (nfb + CL - 1) / CL;
    const int per_cta = (int)fin_pair_bytes(np, CL) + (rows + 12) * 2 * d.cdef.ncand * 4 + rows * 4;
    // raise the kernel's dynamic shared memory opt-in when this launch needs
    // more, never lower it: the attribute is per function and device, and a
    // context set it to its own cap at creation
    if (per_cta > 48 * 1024) {
        cudaFuncAttributes fa;
        if (cudaFuncGetAttributes(&fa, k_cdef_finish) != cudaSuccess) return ZF_ERR_CUDA;
        if (per_cta > fa.maxDynamicSharedSizeBytes &&
            cudaFuncSetAttribute(k_cdef_finish, cudaFuncAttributeMaxDynamicSharedMemorySize, per_cta) != cudaSuccess)
            return ZF_ERR_CUDA;
    }
    if (launch_cdef_finish(kFinLevels, CL, per_cta, st, &sc->desc, &sc->frame_id, per_cta) != cudaSuccess)
        return ZF_ERR_CUDA;
    if (cudaGetLastError() != cudaSuccess) return ZF_ERR_CUDA;
    FrameDesc back;
    if (cudaMemcpyAsync(&back, &sc->desc, sizeof(back), cudaMemcpyDeviceToHost, st) != cudaSuccess) return ZF_ERR_CUDA;
    if (out->cdef_fb_idx &&
        cudaMemcpyAsync(out->cdef_fb_idx, sc->fb_idx, nfb, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return ZF_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return ZF_ERR_CUDA;
    out->cdef_damping = (uint8_t)back.cdef.damping;
    out->cdef_bits = (uint8_t)back.cdef.bits;
    std::memcpy(out->cdef_y, back.cdef.y_str, 8);
    std::memcpy(out->cdef_uv, back.cdef.uv_str, 8);
    if (out->cdef_fb_idx && back.cdef.bits == 0) std::memset(out->cdef_fb_idx, 0, nfb);
    return ZF_OK;
}
