// zf_deblock.cu -- AV1 deblocking filter on the GPU.
//
// Semantics follow the reference's decoder-exact frame pass
// (svtav1-encoder/src/deblock.rs:811-1006): every vertical edge of a plane
// is filtered, then every horizontal edge, with the edge set, filter length
// and thresholds of lpf_params (deblock.rs:698-796) and the lpf kernels of
// svtav1-dsp/src/loop_filter.rs:67-412 / hbd.rs:1066-1440.
//
// GPU formulation. Within one pass the edge windows never overlap (the
// filter length is capped by the transform widths on both sides), so all
// edges of a pass are independent. A CTA owns a 64x64 output tile; it loads
// the tile plus a 12-pixel halo into shared memory, filters every vertical
// edge that can touch the tile's columns over all halo rows, synchronises,
// filters every horizontal edge that can touch the tile's rows, and writes
// (apply) or scores (level search) the tile. The halo covers the farthest
// reach of the 14-tap filter (an edge 5 px outside modifies the tile and
// reads 7 px further), so each tile is exact in isolation and the plane is
// read once and written once.
//
// An edge position (x, y) on the 4x4 grid filters exactly when the
// sequential walk of filter_plane would visit it and lpf_params returns a
// length: the walk visits the transform origins, which for a tiling of
// transforms aligned to their own size are the positions with
// coord % tx_dim == 0 (the host packer rejects any other tiling).
#include "zf_dev.cuh"

namespace zf {

constexpr int DB_T = 64;             // output tile edge
constexpr int DB_H = 12;             // halo
constexpr int DB_R = DB_T + 2 * DB_H;  // region edge (88)
// Region row pitch in 2-byte samples: 45 words. In the vertical-edge pass a
// warp filters 8 edges (2 words apart) x 4 lines of each; their 32 words
// cannot all fall in distinct banks, and 45 words per row keep it at 2-way
// (the region's own 44 words: up to 3-way). Rows stay 4-byte aligned.
constexpr int DB_P = DB_R + 2;
constexpr int DB_BANDS = DB_R / 4;   // 22 four-row bands in the region
constexpr int DB_EDGES = 19;         // edges at tile origin -4 .. +68

struct Thr {
    int mblim, lim, hev;
};

// lf_thresholds (svtav1-dsp/src/loop_filter.rs:50-65).
__device__ __forceinline__ Thr lf_thresholds(int level, int sharp) {
    int bil = level >> ((sharp > 0) + (sharp > 4));
    if (sharp > 0 && bil > 9 - sharp) bil = 9 - sharp;
    if (bil < 1) bil = 1;
    Thr t;
    t.mblim = 2 * (level + 2) + bil;
    t.lim = bil;
    t.hev = level >> 4;
    return t;
}

__device__ __forceinline__ int clamp_sc(int t, int bd) {
    int lo = -(128 << (bd - 8)), hi = (128 << (bd - 8)) - 1;
    return t < lo ? lo : (t > hi ? hi : t);
}

// highbd_filter4 (hbd.rs:1211-1232); at bd 8 it is the 8-bit filter4
// (loop_filter.rs:181-203) with the sign flip written as a bias.
__device__ __forceinline__ void filter4(int mask, int hev, int *w, int bd) {
    int bias = 0x80 << (bd - 8);
    int ps1 = w[0] - bias, ps0 = w[1] - bias, qs0 = w[2] - bias, qs1 = w[3] - bias;
    int filter = clamp_sc(ps1 - qs1, bd) & hev;
    filter = clamp_sc(filter + 3 * (qs0 - ps0), bd) & mask;
    int f1 = clamp_sc(filter + 4, bd) >> 3;
    int f2 = clamp_sc(filter + 3, bd) >> 3;
    w[2] = clamp_sc(qs0 - f1, bd) + bias;
    w[1] = clamp_sc(ps0 + f2, bd) + bias;
    int outer = ((f1 + 1) >> 1) & ~hev;
    w[3] = clamp_sc(qs1 - outer, bd) + bias;
    w[0] = clamp_sc(ps1 + outer, bd) + bias;
}

// One line of one edge. `p` points at q0 in shared memory, `st` is the tap
// step (1 for vertical edges, the row pitch for horizontal edges). The
// filter mask is computed from the inner taps first: a line whose mask fails
// is left as it is (every branch of the reference then writes back the
// values it read), so it loads nothing more and stores nothing; otherwise
// only the samples a branch changes are stored.
__device__ __forceinline__ void filter_line(uint16_t *p, int st, int len, Thr t, int bd) {
    const int sh = bd - 8;
    const int lim = t.lim << sh, blim = t.mblim << sh, thr = t.hev << sh, one = 1 << sh;
    auto ad = [](int a, int b) { return a > b ? a - b : b - a; };
    auto at = [&](int k) -> int { return p[k * st]; };        // k: offset from q0
    auto put = [&](int k, int v) { p[k * st] = (uint16_t)v; };
    if (len == 4) {
        int w[4] = {at(-2), at(-1), at(0), at(1)};
        const int p1 = w[0], p0 = w[1], q0 = w[2], q1 = w[3];
        const bool m = ad(p1, p0) <= lim && ad(q1, q0) <= lim && ad(p0, q0) * 2 + ad(p1, q1) / 2 <= blim;
        if (!m) return;
        const int hev = (ad(p1, p0) > thr || ad(q1, q0) > thr) ? -1 : 0;
        filter4(-1, hev, w, bd);
#pragma unroll
        for (int k = 0; k < 4; ++k) put(k - 2, w[k]);
    } else if (len == 6) {
        int w[6] = {at(-3), at(-2), at(-1), at(0), at(1), at(2)};
        const int p2 = w[0], p1 = w[1], p0 = w[2], q0 = w[3], q1 = w[4], q2 = w[5];
        const bool m = ad(p2, p1) <= lim && ad(p1, p0) <= lim && ad(q1, q0) <= lim && ad(q2, q1) <= lim &&
                       ad(p0, q0) * 2 + ad(p1, q1) / 2 <= blim;
        if (!m) return;
        const bool flat = ad(p1, p0) <= one && ad(q1, q0) <= one && ad(p2, p0) <= one && ad(q2, q0) <= one;
        if (flat) {
            w[1] = (p2 * 3 + p1 * 2 + p0 * 2 + q0 + 4) >> 3;
            w[2] = (p2 + p1 * 2 + p0 * 2 + q0 * 2 + q1 + 4) >> 3;
            w[3] = (p1 + p0 * 2 + q0 * 2 + q1 * 2 + q2 + 4) >> 3;
            w[4] = (p0 + q0 * 2 + q1 * 2 + q2 * 3 + 4) >> 3;
        } else {
            const int hev = (ad(p1, p0) > thr || ad(q1, q0) > thr) ? -1 : 0;
            filter4(-1, hev, w + 1, bd);
        }
#pragma unroll
        for (int k = 1; k < 5; ++k) put(k - 3, w[k]);
    } else {
        // the [p3..q3] window first; the outer taps of the 14-tap filter
        // only when the line is flat
        int v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = at(k - 4);
        const int p3 = v[0], p2 = v[1], p1 = v[2], p0 = v[3], q0 = v[4], q1 = v[5], q2 = v[6], q3 = v[7];
        const bool m = ad(p3, p2) <= lim && ad(p2, p1) <= lim && ad(p1, p0) <= lim && ad(q1, q0) <= lim &&
                       ad(q2, q1) <= lim && ad(q3, q2) <= lim && ad(p0, q0) * 2 + ad(p1, q1) / 2 <= blim;
        if (!m) return;
        const bool flat = ad(p1, p0) <= one && ad(q1, q0) <= one && ad(p2, p0) <= one && ad(q2, q0) <= one &&
                          ad(p3, p0) <= one && ad(q3, q0) <= one;
        if (len == 14 && flat) {
            const int p6 = at(-7), p5 = at(-6), p4 = at(-5), q4 = at(4), q5 = at(5), q6 = at(6);
            const bool flat2 = ad(p5, p0) <= one && ad(q5, q0) <= one && ad(p4, p0) <= one && ad(q4, q0) <= one &&
                               ad(p6, p0) <= one && ad(q6, q0) <= one;
            if (flat2) {
                put(-6, (p6 * 7 + p5 * 2 + p4 * 2 + p3 + p2 + p1 + p0 + q0 + 8) >> 4);
                put(-5, (p6 * 5 + p5 * 2 + p4 * 2 + p3 * 2 + p2 + p1 + p0 + q0 + q1 + 8) >> 4);
                put(-4, (p6 * 4 + p5 + p4 * 2 + p3 * 2 + p2 * 2 + p1 + p0 + q0 + q1 + q2 + 8) >> 4);
                put(-3, (p6 * 3 + p5 + p4 + p3 * 2 + p2 * 2 + p1 * 2 + p0 + q0 + q1 + q2 + q3 + 8) >> 4);
                put(-2, (p6 * 2 + p5 + p4 + p3 + p2 * 2 + p1 * 2 + p0 * 2 + q0 + q1 + q2 + q3 + q4 + 8) >> 4);
                put(-1, (p6 + p5 + p4 + p3 + p2 + p1 * 2 + p0 * 2 + q0 * 2 + q1 + q2 + q3 + q4 + q5 + 8) >> 4);
                put(0, (p5 + p4 + p3 + p2 + p1 + p0 * 2 + q0 * 2 + q1 * 2 + q2 + q3 + q4 + q5 + q6 + 8) >> 4);
                put(1, (p4 + p3 + p2 + p1 + p0 + q0 * 2 + q1 * 2 + q2 * 2 + q3 + q4 + q5 + q6 * 2 + 8) >> 4);
                put(2, (p3 + p2 + p1 + p0 + q0 + q1 * 2 + q2 * 2 + q3 * 2 + q4 + q5 + q6 * 3 + 8) >> 4);
                put(3, (p2 + p1 + p0 + q0 + q1 + q2 * 2 + q3 * 2 + q4 * 2 + q5 + q6 * 4 + 8) >> 4);
                put(4, (p1 + p0 + q0 + q1 + q2 + q3 * 2 + q4 * 2 + q5 * 2 + q6 * 5 + 8) >> 4);
                put(5, (p0 + q0 + q1 + q2 + q3 + q4 * 2 + q5 * 2 + q6 * 7 + 8) >> 4);
                return;
            }
        }
        if (flat) {
            put(-3, (p3 + p3 + p3 + 2 * p2 + p1 + p0 + q0 + 4) >> 3);
            put(-2, (p3 + p3 + p2 + 2 * p1 + p0 + q0 + q1 + 4) >> 3);
            put(-1, (p3 + p2 + p1 + 2 * p0 + q0 + q1 + q2 + 4) >> 3);
            put(0, (p2 + p1 + p0 + 2 * q0 + q1 + q2 + q3 + 4) >> 3);
            put(1, (p1 + p0 + q0 + 2 * q1 + q2 + q3 + q3 + 4) >> 3);
            put(2, (p0 + q0 + q1 + 2 * q2 + q3 + q3 + q3 + 4) >> 3);
        } else {
            const int hev = (ad(p1, p0) > thr || ad(q1, q0) > thr) ? -1 : 0;
            filter4(-1, hev, v + 2, bd);
#pragma unroll
            for (int k = 2; k < 6; ++k) put(k - 4, v[k]);
        }
    }
}

// Transform dims of a packed mi for a plane: luma TX grid, or the chroma TX
// max(b/2, 4) of the covering block (deblock.rs:728-743).
__device__ __forceinline__ void tx_dims(uint32_t r, int plane, int *tw, int *th) {
    if (plane == 0) {
        *tw = mi_tw(r);
        *th = mi_th(r);
    } else {
        *tw = max(mi_bw(r) >> 1, 4);
        *th = max(mi_bh(r) >> 1, 4);
    }
}

// Filter length for the edge at plane position (x, y) (both multiples of 4),
// 0 when nothing is filtered (lpf_params, deblock.rs:698-796).
__device__ int edge_len(const FrameDesc &f, bool vert, int x, int y, int plane, int level) {
    const int ss = plane ? 1 : 0;
    if (level == 0) return 0;
    if (x >= (f.tw >> ss) || y >= (f.th >> ss)) return 0;
    const int mr = ss | ((y << ss) >> 2), mc = ss | ((x << ss) >> 2);
    if (mr >= f.mi_rows || mc >= f.mi_cols) return 0;
    const uint32_t cur = f.mi[(int64_t)mr * f.mi_cols + mc];
    int tw, th;
    tx_dims(cur, plane, &tw, &th);
    const int ts = vert ? tw : th;
    const int coord = vert ? x : y;
    if ((coord & (ts - 1)) != 0 || coord == 0) return 0;
    const int pr = vert ? mr : mr - (1 << ss), pc = vert ? mc - (1 << ss) : mc;
    const uint32_t prv = f.mi[(int64_t)pr * f.mi_cols + pc];
    int ptw, pth;
    tx_dims(prv, plane, &ptw, &pth);
    const int pv = vert ? ptw : pth;
    // pu_edge: different covering blocks <=> different aligned block origins.
    const int cbw = mi_bw(cur) >> 2, cbh = mi_bh(cur) >> 2, pbw = mi_bw(prv) >> 2, pbh = mi_bh(prv) >> 2;
    const bool pu_edge = (mr & ~(cbh - 1)) != (pr & ~(pbh - 1)) || (mc & ~(cbw - 1)) != (pc & ~(pbw - 1));
    if (!mi_skip_inter(prv) || !mi_skip_inter(cur) || pu_edge) {
        const int md = min(ts, pv);
        return md == 4 ? 4 : (plane ? 6 : (md == 8 ? 8 : 14));
    }
    return 0;
}

struct DbTile {
    const FrameDesc *f;
    int plane, pw, ph, x0, y0;
};

// Word-wide plane access. Plane rows start 4-byte aligned when the plane
// base is (a row is a multiple of 4 bytes: luma width % 8 == 0, chroma
// width % 4 == 0), tile columns start at multiples of 4 samples and plane
// widths are multiples of 4, so a 4-byte word (4 u8 or 2 u16 samples) is
// either wholly inside the plane or wholly outside.
__device__ __forceinline__ bool word_ok(const void *p) { return ((uintptr_t)p & 3) == 0; }

// Samples of a word as packed u16 pairs (lo, hi): 4 samples at 8 bits, 2 at 10.
__device__ __forceinline__ void unpack_word(uint32_t v, int bd, uint16_t *o) {
    if (bd == 8) {
        *reinterpret_cast<uint32_t *>(o) = (v & 0xffu) | ((v & 0xff00u) << 8);
        *reinterpret_cast<uint32_t *>(o + 2) = ((v >> 16) & 0xffu) | ((v >> 8) & 0xff0000u);
    } else {
        *reinterpret_cast<uint32_t *>(o) = v;
    }
}
__device__ __forceinline__ uint32_t pack_word(const uint16_t *o, int bd) {
    if (bd == 8) {
        const uint32_t a = *reinterpret_cast<const uint32_t *>(o), b = *reinterpret_cast<const uint32_t *>(o + 2);
        return (a & 0xffu) | ((a >> 8) & 0xff00u) | ((b & 0xffu) << 16) | ((b & 0xff0000u) << 8);
    }
    return *reinterpret_cast<const uint32_t *>(o);
}
__device__ __forceinline__ const uint32_t *word_at(const uint8_t *plane, int64_t sample, int bd) {
    return reinterpret_cast<const uint32_t *>(plane + sample * (bd == 8 ? 1 : 2));
}

// Load the region of a tile into shared memory as u16.
__device__ __forceinline__ void db_load_bd(const DbTile &t, const uint8_t *plane, uint16_t *reg, const int bd) {
    if (word_ok(plane)) {
        const int spw = bd == 8 ? 4 : 2, wpr = DB_R / spw;
        // flat over (row, word), four words per thread at a time: their
        // loads are issued before any is unpacked, so the latencies overlap
        const int total = DB_R * wpr;
        for (int i0 = threadIdx.x; i0 < total; i0 += 4 * blockDim.x) {
            uint32_t v[4];
            int off[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int i = i0 + j * blockDim.x;
                const int ry = i / wpr, wx = i - ry * wpr;
                const int y = t.y0 - DB_H + ry, x = t.x0 - DB_H + wx * spw;
                off[j] = i < total ? ry * DB_P + wx * spw : -1;
                v[j] = 0;
                if (i < total && x >= 0 && x < t.pw && y >= 0 && y < t.ph) v[j] = *word_at(plane, (int64_t)y * t.pw + x, bd);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (off[j] >= 0) unpack_word(v[j], bd, reg + off[j]);
        }
        return;
    }
    for (int i = threadIdx.x; i < DB_R * DB_R; i += blockDim.x) {
        int ry = i / DB_R, rx = i - ry * DB_R;
        int y = t.y0 - DB_H + ry, x = t.x0 - DB_H + rx;
        int v = 0;
        if (x >= 0 && x < t.pw && y >= 0 && y < t.ph) v = ldpx(plane, (int64_t)y * t.pw + x, bd);
        reg[ry * DB_P + rx] = (uint16_t)v;
    }
}

// The loader compiled once with the bit depth a constant for 8-bit planes
// (samples per word and their unpacking resolved at compile time), once for
// other depths.
__device__ void db_load(const DbTile &t, const uint8_t *plane, uint16_t *reg) {
    if (t.f->bd == 8) db_load_bd(t, plane, reg, 8);
    else db_load_bd(t, plane, reg, t.f->bd);
}

// The filtering edges of a tile, bucketed by filter length (4, 6, 8, 14):
// v[bucket][k] = band * DB_EDGES + edge for vertical edges over the region
// rows, h[bucket][k] = column band * DB_EDGES + edge for horizontal edges
// over the tile columns. Edges within a pass are independent, so each
// bucket runs with every thread on one compile-time filter length.
// Buckets 0 and 1 share one array (bucket 0 from the front, bucket 1 from
// the back), buckets 2 and 3 another: a pass has at most one entry per
// edge, so each pair fits. Horizontal entries are edge * 16 + column band:
// listed band-minor, the 8 segments of a warp are 8 adjacent column bands
// of one edge row (16 consecutive words: no bank conflict); listed
// edge-minor they were rows 4 apart, 0 or 16 banks apart (4-way).
constexpr int DB_NV = DB_BANDS * DB_EDGES, DB_NH = (DB_T / 4) * DB_EDGES;
struct DbEdges {
    uint16_t v[2][DB_NV];
    uint16_t h[2][DB_NH];
    int nv[4], nh[4];
};
__device__ __forceinline__ uint16_t &edge_slot(uint16_t (*lists)[DB_NV], int bk, int k) {
    return lists[bk >> 1][(bk & 1) ? DB_NV - 1 - k : k];
}
__device__ __forceinline__ uint16_t &edge_slot(uint16_t (*lists)[DB_NH], int bk, int k) {
    return lists[bk >> 1][(bk & 1) ? DB_NH - 1 - k : k];
}
__device__ __forceinline__ int len_bucket(int len) { return len == 4 ? 0 : len == 6 ? 1 : len == 8 ? 2 : 3; }

// Every thread of the CTA calls this; the lists are complete after the
// caller's next barrier.
__device__ void db_params(const DbTile &t, int lvl_v, int lvl_h, DbEdges &E) {
    const FrameDesc &f = *t.f;
    if (threadIdx.x < 4) E.nv[threadIdx.x] = E.nh[threadIdx.x] = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < DB_BANDS * DB_EDGES; i += blockDim.x) {
        int band = i / DB_EDGES, e = i - band * DB_EDGES;
        int y = t.y0 - DB_H + band * 4, x = t.x0 - 4 + e * 4;
        int len = 0;
        if (y >= 0 && y < t.ph && x >= 0 && x < t.pw) len = edge_len(f, true, x, y, t.plane, lvl_v);
        if (len) {
            const int bk = len_bucket(len);
            edge_slot(E.v, bk, atomicAdd(&E.nv[bk], 1)) = (uint16_t)i;
        }
    }
    for (int i = threadIdx.x; i < DB_NH; i += blockDim.x) {
        int e = i >> 4, cb = i & 15;
        int x = t.x0 + cb * 4, y = t.y0 - 4 + e * 4;
        int len = 0;
        if (y >= 0 && y < t.ph && x >= 0 && x < t.pw) len = edge_len(f, false, x, y, t.plane, lvl_h);
        if (len) {
            const int bk = len_bucket(len);
            edge_slot(E.h, bk, atomicAdd(&E.nh[bk], 1)) = (uint16_t)i;
        }
    }
}

__device__ __forceinline__ void filter_bucket(int bk, uint16_t *p, int st, Thr t, int bd) {
    switch (bk) {  // a constant length per call site after inlining
        case 0: filter_line(p, st, 4, t, bd); break;
        case 1: filter_line(p, st, 6, t, bd); break;
        case 2: filter_line(p, st, 8, t, bd); break;
        default: filter_line(p, st, 14, t, bd); break;
    }
}

// Both passes on the region in shared memory.
__device__ void db_filter(const DbTile &t, uint16_t *reg, const DbEdges &E, int lvl_v, int lvl_h) {
    const int bd = t.f->bd, sharp = t.f->sharpness;
    const Thr tv = lf_thresholds(lvl_v, sharp), th = lf_thresholds(lvl_h, sharp);
    for (int bk = 0; bk < 4; ++bk)
        for (int i = threadIdx.x; i < E.nv[bk] * 4; i += blockDim.x) {
            const int be = edge_slot(const_cast<uint16_t (*)[DB_NV]>(E.v), bk, i >> 2), line = i & 3;
            const int band = be / DB_EDGES, e = be - band * DB_EDGES;
            const int ry = band * 4 + line, rx = DB_H - 4 + e * 4;
            filter_bucket(bk, reg + ry * DB_P + rx, 1, tv, bd);
        }
    __syncthreads();
    for (int bk = 0; bk < 4; ++bk)
        for (int i = threadIdx.x; i < E.nh[bk] * 4; i += blockDim.x) {
            const int be = edge_slot(const_cast<uint16_t (*)[DB_NH]>(E.h), bk, i >> 2), line = i & 3;
            const int e = be >> 4, cb = be & 15;
            const int rx = DB_H + cb * 4 + line, ry = DB_H - 4 + e * 4;
            filter_bucket(bk, reg + ry * DB_P + rx, DB_P, th, bd);
        }
    __syncthreads();
}

__device__ __forceinline__ void plane_geom(const FrameDesc &f, int plane, int *pw, int *ph) {
    *pw = plane ? f.w / 2 : f.w;
    *ph = plane ? f.h / 2 : f.h;
}

// Apply: IN -> B for one 64x64 tile. Plane gating of apply_deblock_frame
// (deblock.rs:951-967): both luma levels zero disables every plane; a chroma
// plane needs its own level.
__global__ void __launch_bounds__(256, 5) k_deblock_apply(const FrameDesc *frames, const WorkItem *items, int nitems) {
    __shared__ __align__(16) uint16_t reg[DB_R * DB_P];
    __shared__ DbEdges edges;
    const int it = find_item(items, nitems, blockIdx.x);
    const WorkItem wi = items[it];
    const FrameDesc &f = frames[wi.frame];
    const int plane = wi.plane;
    int pw, ph;
    plane_geom(f, plane, &pw, &ph);
    const int tiles_x = (pw + DB_T - 1) / DB_T;
    const int tix = blockIdx.x - wi.cta_begin;
    DbTile t{&f, plane, pw, ph, (tix % tiles_x) * DB_T, (tix / tiles_x) * DB_T};
    int lv, lh;
    if (f.lf[0] == 0 && f.lf[1] == 0) {
        lv = lh = 0;
    } else if (plane == 0) {
        lv = f.lf[0];
        lh = f.lf[1];
    } else {
        lv = lh = f.lf[1 + plane];
    }
    const int bd = f.bd;
    const int spw = bd == 8 ? 4 : 2, wpr = DB_T / spw, lgw = bd == 8 ? 4 : 5;  // wpr = 1 << lgw
    const bool words = word_ok(f.IN[plane]) && word_ok(f.B[plane]);
    if (lv == 0 && lh == 0 && words) {  // copy-through, word-wide
        for (int i = threadIdx.x; i < DB_T * wpr; i += blockDim.x) {
            const int ty = i >> lgw, wx = i & (wpr - 1);
            const int y = t.y0 + ty, x = t.x0 + wx * spw;
            if (x < pw && y < ph) {
                const int64_t o = (int64_t)y * pw + x;
                *const_cast<uint32_t *>(word_at(f.B[plane], o, bd)) = *word_at(f.IN[plane], o, bd);
            }
        }
        return;
    }
    if (lv == 0 && lh == 0) {  // copy-through
        for (int i = threadIdx.x; i < DB_T * DB_T; i += blockDim.x) {
            int y = t.y0 + i / DB_T, x = t.x0 + (i % DB_T);
            if (x < pw && y < ph) {
                int64_t o = (int64_t)y * pw + x;
                stpx(f.B[plane], o, bd, ldpx(f.IN[plane], o, bd));
            }
        }
        return;
    }
    db_load(t, f.IN[plane], reg);
    db_params(t, lv, lh, edges);
    __syncthreads();
    db_filter(t, reg, edges, lv, lh);
    if (word_ok(f.B[plane])) {
        for (int i = threadIdx.x; i < DB_T * wpr; i += blockDim.x) {
            const int ty = i >> lgw, wx = i & (wpr - 1);
            const int y = t.y0 + ty, x = t.x0 + wx * spw;
            if (x < pw && y < ph)
                *const_cast<uint32_t *>(word_at(f.B[plane], (int64_t)y * pw + x, bd)) =
                    pack_word(reg + (ty + DB_H) * DB_P + DB_H + wx * spw, bd);
        }
        return;
    }
    for (int i = threadIdx.x; i < DB_T * DB_T; i += blockDim.x) {
        int ty = i / DB_T, tx = i % DB_T;
        int y = t.y0 + ty, x = t.x0 + tx;
        if (x < pw && y < ph) stpx(f.B[plane], (int64_t)y * pw + x, bd, reg[(ty + DB_H) * DB_P + tx + DB_H]);
    }
}

// Level search: SSE(source, plane filtered at level L in both directions)
// over the full aligned plane (try_filter_plane, deblock.rs:228-293), for
// up to kDbLevels candidate levels per (frame, plane) slot and launch: the
// tile and its halo are staged once and filtered at every level of the
// slot. items[].a = slot index; levels[slot * nl + k] (< 0: unused) and
// sse[slot * nl + k] the SSE accumulated for it.
__global__ void __launch_bounds__(256, 5) k_deblock_sse(const FrameDesc *frames, const WorkItem *items, int nitems,
                                                     const int *levels, int nl, unsigned long long *sse) {
    __shared__ __align__(16) uint16_t reg[DB_R * DB_P];
    __shared__ __align__(16) uint16_t pristine[DB_R * DB_P];
    __shared__ __align__(16) uint16_t srct[DB_T * DB_T];  // the source tile, staged once for every level
    __shared__ DbEdges edges;
    __shared__ unsigned long long part[8];
    const int it = find_item(items, nitems, blockIdx.x);
    const WorkItem wi = items[it];
    const FrameDesc &f = frames[wi.frame];
    const int plane = wi.plane, slot = wi.a;
    int pw, ph;
    plane_geom(f, plane, &pw, &ph);
    const int tiles_x = (pw + DB_T - 1) / DB_T;
    const int tix = blockIdx.x - wi.cta_begin;
    DbTile t{&f, plane, pw, ph, (tix % tiles_x) * DB_T, (tix / tiles_x) * DB_T};
    const int bd = f.bd;
    // the region and the tile's source samples (0 outside the plane: such
    // positions are skipped by the sum below), word-wide where the planes
    // allow
    const int spw = bd == 8 ? 4 : 2, wpr = DB_T / spw, lgw = bd == 8 ? 4 : 5;  // wpr = 1 << lgw
    if (bd != 8 && word_ok(f.IN[plane]) && word_ok(f.S[plane])) {
        // 16-bit samples land in shared memory as they are: every word of
        // the region and the source tile as a 4-byte asynchronous copy, all
        // in flight at once (zeros outside the plane), one wait
        const int rpr = DB_R / 2, tot_r = DB_R * rpr, tot = tot_r + DB_T * wpr;
        for (int i = threadIdx.x; i < tot; i += blockDim.x) {
            if (i < tot_r) {
                const int ry = i / rpr, wx = i - ry * rpr;
                const int y = t.y0 - DB_H + ry, x = t.x0 - DB_H + wx * 2;
                const bool in = x >= 0 && x < t.pw && y >= 0 && y < t.ph;
                cp_async4(pristine + ry * DB_P + wx * 2, in ? (const void *)word_at(f.IN[plane], (int64_t)y * t.pw + x, bd)
                                                           : (const void *)f.IN[plane],
                          in ? 4u : 0u);
            } else {
                const int k = i - tot_r, ty = k >> lgw, wx = k & (wpr - 1);
                const int y = t.y0 + ty, x = t.x0 + wx * 2;
                const bool in = x < pw && y < ph;
                cp_async4(srct + ty * DB_T + wx * 2, in ? (const void *)word_at(f.S[plane], (int64_t)y * pw + x, bd)
                                                       : (const void *)f.S[plane],
                          in ? 4u : 0u);
            }
        }
        cp_async_wait_all();
    } else if (word_ok(f.S[plane])) {
        db_load(t, f.IN[plane], pristine);
        for (int i = threadIdx.x; i < DB_T * wpr; i += blockDim.x) {
            const int ty = i >> lgw, wx = i & (wpr - 1);
            const int y = t.y0 + ty, x = t.x0 + wx * spw;
            const uint32_t v = (x < pw && y < ph) ? *word_at(f.S[plane], (int64_t)y * pw + x, bd) : 0u;
            unpack_word(v, bd, srct + ty * DB_T + wx * spw);
        }
    } else {
        db_load(t, f.IN[plane], pristine);
        for (int i = threadIdx.x; i < DB_T * DB_T; i += blockDim.x) {
            const int ty = i / DB_T, tx = i % DB_T, y = t.y0 + ty, x = t.x0 + tx;
            srct[i] = (uint16_t)((x < pw && y < ph) ? ldpx(f.S[plane], (int64_t)y * pw + x, bd) : 0);
        }
    }
    // edge lengths do not depend on a nonzero level: computed once
    bool any = false;
    for (int k = 0; k < nl; ++k) any = any || levels[slot * nl + k] > 0;
    if (any) db_params(t, 1, 1, edges);
    __syncthreads();
    // rows and columns of the tile inside the plane (pw, ph are multiples of
    // 4; two samples per word of the u16 rows)
    const int rows = min(DB_T, ph - t.y0), pairs = min(DB_T, pw - t.x0) >> 1;
    for (int k = 0; k < nl; ++k) {
        const int lvl = levels[slot * nl + k];
        if (lvl < 0) continue;
        for (int i = threadIdx.x; i < DB_R * DB_P / 2; i += blockDim.x)
            reinterpret_cast<uint32_t *>(reg)[i] = reinterpret_cast<const uint32_t *>(pristine)[i];
        __syncthreads();
        if (lvl != 0) db_filter(t, reg, edges, lvl, lvl);
        unsigned long long acc = 0;
        for (int i = threadIdx.x; i < DB_T * (DB_T / 2); i += blockDim.x) {
            const int ty = i >> 5, px = i & 31;
            if (ty < rows && px < pairs) {
                const uint32_t sv = reinterpret_cast<const uint32_t *>(srct + ty * DB_T)[px];
                const uint32_t rv = reinterpret_cast<const uint32_t *>(reg + (ty + DB_H) * DB_P + DB_H)[px];
                const int d0 = (int)(sv & 0xffffu) - (int)(rv & 0xffffu), d1 = (int)(sv >> 16) - (int)(rv >> 16);
                acc += (unsigned long long)(uint32_t)(d0 * d0 + d1 * d1);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long s = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += part[w];
            atomicAdd(&sse[slot * nl + k], s);
        }
        __syncthreads();
    }
}

}  // namespace zf
