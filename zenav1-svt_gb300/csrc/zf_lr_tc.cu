// zf_lr_tc.cu -- Wiener statistics of 8-bit planes (5-tap window) on the
// tensor cores: tcgen05.mma kind::f16 with fp32 accumulators in tensor
// memory, exact integer results.
//
// Reference: compute_stats (svtav1-dsp/src/restoration.rs:567-632) with
// find_average (:198) and sse_region (:1666) folded in, as the CUDA-core
// kernel k_lr_stats (zf_lr.cu) computes them: the raw-sample sums
//   Hr[a][b] = sum d_a d_b (b >= a),  Mr[a] = sum d_a s,  S[a] = sum d_a,
// sum s and the three sse_region parts over a restoration unit, where d_a is
// the post-CDEF sample at window offset a = (ca, ra) of an output pixel
// (index ca * 5 + ra) and s the source sample; k_lr_solve applies the
// average correction. This kernel produces the same integers.
//
// The Gram as one MMA. A CTA owns a band of TR output rows of a unit and
// walks it in tiles of TW columns. K runs over the tile's output pixels
// (row-major, K = rows * TW). With e = d - 128 (exact in fp16), the
// operand row (r, c) at K position (y, x) must hold e at window offset
// (ca = c, ra = r): e[y + r - 2][x + c - 2]. In the canonical no-swizzle
// K-major layout a core matrix is 8 rows x 8 fp16 of K, core matrices are
// LBO bytes apart along K and SBO bytes apart along M. The tile's "stream"
// stores, for every window row y' (tile rows plus 4) and 8-pixel chunk of
// columns, one core matrix whose row c (0..4) is e[y' - 2][x + c - 2] for
// the chunk's 8 pixels x. With SBO = one window row of chunks, M group r
// of an operand descriptor at K position (y, x) lands on window row y + r:
// every window offset (r, c) of the output pixel, with no copy per r. A and
// B are the same descriptor (M = 64: groups r = 0..7, of which 0..4 are
// window rows; N = 40: groups r' = 0..4), so D[(r, c)][(r', c')] =
// sum e_a e_b over the tile. Core-matrix rows 5 and 6 carry s - 128 and 1
// at the output pixel (window row y' - 2 == y): the columns (2, 5) and
// (2, 6) of D are then sum e_a (s - 128) and sum e_a. LBO is 144 bytes, not
// 128, so that the 16-byte stores of eight consecutive threads hit eight
// different bank groups.
//
// Exactness: |e|, |s - 128| <= 128, so every product is <= 2^14 and a
// chain of at most 1024 K elements stays below 2^24, where fp32 holds every
// integer: each chain starts a fresh accumulator (set 0 or 1 of the CTA's
// 128 tensor-memory columns), and after the tile's MMAs complete the
// folding warps convert each needed accumulator to int32 and add it up
// (a band of 32 x 384 pixels sums to < 2^28). The int32 sums become the raw
// int64 sums by Hr = Hc + 128 (E_a + E_b) + 128^2 n, Mr = Mc + 128 E_a +
// 128 S' + 128^2 n, S = E + 128 n (n pixels, S' = sum (s - 128)).
#include <cuda_fp16.h>

#include "zf_dev.cuh"

namespace zf {
namespace lrtc {

constexpr int TR = 32;                   // output rows per band (CTA)
constexpr int TW = 64;                   // output columns per tile
constexpr int NCH = TW / 8;              // 8-pixel K chunks per window row
constexpr int CMB = 144;                 // bytes between K-adjacent core matrices (LBO)
constexpr int SBO = NCH * CMB;           // bytes between window rows (M/N groups)
constexpr int SROWS = TR + 8;            // window rows TR + 4, plus M groups r = 5..7 of the last rows
constexpr int STREAM = SROWS * SBO;      // 46080 bytes
constexpr int EROWS = TR + 4;            // staged e rows: window rows of the band
constexpr int EP = 144;                  // bytes per staged e row (72 fp16: TW + 4 used, 8 read past)
constexpr int SP = TW * 2;               // bytes per staged s - 128 row
constexpr int CHAIN = 1024;              // K elements per accumulation chain
constexpr int THREADS = 128;
constexpr uint32_t TMEM_COLS = 128;      // sets 0 and 1 at columns 0 and 64, N = 40 each
// instruction descriptor: D f32, A and B f16, both K-major, N = 40, M = 64
constexpr uint32_t IDESC = (1u << 4) | ((40u >> 3) << 17) | ((64u >> 4) << 24);

struct Smem {
    uint8_t stream[STREAM];
    uint8_t erow[EROWS * EP];
    uint8_t srow[TR * SP];
    int hacc[25 * 25];
    int macc[25], eacc[25];
    unsigned long long red[4];           // sum s, sse blocks, right strip, bottom strip
    uint64_t mbar;
    uint32_t tmem;
};
static_assert(STREAM % 16 == 0 && (EROWS * EP) % 16 == 0 && (TR * SP) % 16 == 0, "16-byte aligned parts");

// Shared-memory matrix descriptor (tcgen05): start address, leading (K)
// and stride (M/N) byte offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ void mma_f16(uint32_t dtmem, uint64_t desc, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %3, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %1, %2, p;\n}\n" ::"r"(dtmem),
        "l"(desc), "r"(IDESC), "r"(accumulate)
        : "memory");
}

// 16 (8) accumulator columns from column `taddr` of this warp's 32 lanes
// (lane i <-> accumulator row 16 w + i for i < 16 under M = 64).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&v)[16]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ int f2i(uint32_t v) { return __float2int_rz(__uint_as_float(v)); }

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// fp16 halves k..k+1 of the 12-half string w[0..5] (k = 0..10).
__device__ __forceinline__ uint32_t halves_at(const uint32_t (&w)[6], int k) {
    return (k & 1) ? __byte_perm(w[k >> 1], w[(k >> 1) + 1], 0x5432) : w[k >> 1];
}

}  // namespace lrtc

using namespace lrtc;

// Items: a = unit of plane `plane` of `frame`, CTA offset = band of TR rows.
__global__ void __launch_bounds__(lrtc::THREADS, 3) k_lr_stats_tc(FrameDesc *frames, const WorkItem *items, int nitems) {
    extern __shared__ __align__(128) uint8_t lrtc_dyn[];
    Smem &S = *reinterpret_cast<Smem *>(lrtc_dyn);
    const int it = find_item(items, nitems, blockIdx.x);
    const WorkItem wi = items[it];
    FrameDesc &f = frames[wi.frame];
    const LrPlane &pl = f.lr[wi.plane];
    const UnitRect ur = pl.rects[wi.a];
    LrUnit &u = pl.units[wi.a];
    const int stride = wi.plane ? f.w / 2 : f.w;
    const int uw = ur.h_end - ur.h_start, uh = ur.v_end - ur.v_start;
    const int y0 = ((int)blockIdx.x - wi.cta_begin) * TR;  // first output row of the band (unit rows)
    const int rows = min(TR, uh - y0);
    const uint8_t *dg = f.A[wi.plane], *sr = f.S[wi.plane];
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;

    // the stream starts zeroed: its rows past the band's window rows are read
    // only into accumulator rows that are never used, and must hold finite values
    for (int i = t; i < STREAM / 16; i += THREADS) reinterpret_cast<uint4 *>(S.stream)[i] = make_uint4(0, 0, 0, 0);
    if (t < 4) S.red[t] = 0;
    if (t == 0) mbar_init(&S.mbar, 1);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem;

    // folding lanes: accumulator row m = 16 warp + lane (warps 0..2, lanes
    // 0..15) = window offset (r = m >> 3, c = m & 7); rows with r, c <= 4
    // are the Gram's rows
    const int m = 16 * warp + lane;
    const bool fold_lane = warp < 3 && lane < 16;
    int acc[27];  // [r' * 5 + c'] = sum e_a e_(r', c'); [25] = sum e_a (s - 128); [26] = sum e_a
#pragma unroll
    for (int j = 0; j < 27; ++j) acc[j] = 0;
    unsigned s_sum = 0, e_blk = 0, e_rgt = 0, e_bot = 0;
    const int jr = uw - uw % 16, ib_ = uh - uh % 16;  // sse_region's right and bottom strips
    uint32_t phase = 0;
    bool failed = false;

    const int ntiles = (uw + TW - 1) / TW;
    for (int tile = 0; tile < ntiles; ++tile) {
        const int x0 = tile * TW, wv = min(TW, uw - x0);
        // 1. e = d - 128 over the band's window rows and the tile's columns
        //    (-2 .. TW + 2), coordinates clamped to the plane
        const int er = rows + 4;
#pragma unroll 4
        for (int i = t; i < er * (TW + 4); i += THREADS) {
            const int yy = i / (TW + 4), xx = i - yy * (TW + 4);
            const int gy = clampi(ur.v_start + y0 - 2 + yy, 0, pl.ph - 1);
            const int gx = clampi(ur.h_start + x0 - 2 + xx, 0, pl.pw - 1);
            reinterpret_cast<__half *>(S.erow + yy * EP)[xx] = __int2half_rn((int)dg[(int64_t)gy * stride + gx] - 128);
        }
        __syncthreads();
        // 2. s - 128 at the output pixels (0 past the tile's valid columns),
        //    sum s and the sse_region parts
#pragma unroll 4
        for (int i = t; i < rows * TW; i += THREADS) {
            const int yy = i / TW, xx = i - yy * TW;
            int sv = 0;
            if (xx < wv) {
                const int s = sr[(int64_t)(ur.v_start + y0 + yy) * stride + ur.h_start + x0 + xx];
                const int d = __half2int_rn(reinterpret_cast<const __half *>(S.erow + (yy + 2) * EP)[xx + 2]) + 128;
                const unsigned e2 = (unsigned)((s - d) * (s - d));
                s_sum += (unsigned)s;
                if (x0 + xx >= jr) e_rgt += e2;
                else if (y0 + yy >= ib_) e_bot += e2;
                else e_blk += e2;
                sv = s - 128;
            }
            reinterpret_cast<__half *>(S.srow + yy * SP)[xx] = __int2half_rn(sv);
        }
        __syncthreads();
        // 3. the stream: one core matrix per (window row, 8-pixel chunk)
#pragma unroll 1
        for (int q = t; q < er * NCH; q += THREADS) {
            const int yy = q / NCH, j = q - yy * NCH;
            uint8_t *cm = S.stream + (size_t)(yy * NCH + j) * CMB;
            const uint4 a = *reinterpret_cast<const uint4 *>(S.erow + yy * EP + j * 16);
            const uint2 b = *reinterpret_cast<const uint2 *>(S.erow + yy * EP + j * 16 + 16);
            const uint32_t w[6] = {a.x, a.y, a.z, a.w, b.x, b.y};
            const int nval = wv - 8 * j;  // valid pixels of the chunk
            // half-pair masks of the chunk's valid pixels
            uint32_t mk[4];
#pragma unroll
            for (int k = 0; k < 4; ++k)
                mk[k] = (2 * k + 1 < nval ? 0xFFFF0000u : 0u) | (2 * k < nval ? 0x0000FFFFu : 0u);
#pragma unroll
            for (int c = 0; c < 5; ++c) {
                uint4 v;
                v.x = halves_at(w, c) & mk[0];
                v.y = halves_at(w, c + 2) & mk[1];
                v.z = halves_at(w, c + 4) & mk[2];
                v.w = halves_at(w, c + 6) & mk[3];
                *reinterpret_cast<uint4 *>(cm + c * 16) = v;
            }
            const bool out_row = yy >= 2 && yy < rows + 2;
            const uint4 s5 = out_row ? *reinterpret_cast<const uint4 *>(S.srow + (yy - 2) * SP + j * 16)
                                     : make_uint4(0, 0, 0, 0);
            const uint32_t one2 = 0x3C003C00u;  // fp16 1.0 in both halves
            const uint4 s6 = out_row ? make_uint4(one2 & mk[0], one2 & mk[1], one2 & mk[2], one2 & mk[3])
                                     : make_uint4(0, 0, 0, 0);
            *reinterpret_cast<uint4 *>(cm + 5 * 16) = s5;
            *reinterpret_cast<uint4 *>(cm + 6 * 16) = s6;
            *reinterpret_cast<uint4 *>(cm + 7 * 16) = make_uint4(0, 0, 0, 0);
        }
        // 4. the generic-proxy stores become visible to the MMA, then one
        //    thread issues the tile's chains (1024 K elements each)
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        const int K = rows * TW, nch = (K + CHAIN - 1) / CHAIN;
        if (t == 0) {
            const uint32_t base = smem_u32(S.stream);
            for (int ch = 0; ch < nch; ++ch) {
                const int k1 = min(K, (ch + 1) * CHAIN);
                for (int k = ch * CHAIN; k < k1; k += 16)
                    mma_f16(tmem + (uint32_t)(ch * 64), smem_desc(base + (uint32_t)(k / 8) * CMB, CMB, SBO),
                            k > ch * CHAIN ? 1u : 0u);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&S.mbar))
                         : "memory");
        }
        // 5. bounded wait for the MMAs (the stream and the accumulators are
        //    reused after it; the context's wait limit, in ~100 ns steps); on
        //    a timeout the frame's error word is set and the MMAs are waited
        //    for once more before the CTA frees its tensor-memory columns
        const uint32_t lim = f.wait_limit == 0xFFFFFFFFu ? 0u : f.wait_limit;  // ZF_WAIT_GIVE_UP: a test
        const bool late = !mbar_wait_timed(&S.mbar, phase, lim, kWaitStepNs);
        if (__syncthreads_or(late)) {
            if (t == 0) atomicOr(&f.cdef_stats[3], 2ull);
            mbar_wait_bounded(&S.mbar, phase, kDrainWaitLimit);
            failed = true;
            break;
        }
        phase ^= 1u;
        tc_fence_after();
        // 6. fold the tile's chains into int32
        if (warp < 3) {
            for (int ch = 0; ch < nch; ++ch) {
                // columns n = r' * 8 + c': 0..15 hold r' = 0, 1; 16..31 hold
                // r' = 2 (with (2, 5) at 21 and (2, 6) at 22) and 3; 32..39 r' = 4
                const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(ch * 64);
                uint32_t v[16];
                tmem_ld16(ta, v);
#pragma unroll
                for (int k = 0; k < 5; ++k) {
                    acc[k] += f2i(v[k]);
                    acc[5 + k] += f2i(v[8 + k]);
                }
                tmem_ld16(ta + 16, v);
#pragma unroll
                for (int k = 0; k < 5; ++k) {
                    acc[10 + k] += f2i(v[k]);
                    acc[15 + k] += f2i(v[8 + k]);
                }
                acc[25] += f2i(v[5]);
                acc[26] += f2i(v[6]);
                tmem_ld8(ta + 32, v);
#pragma unroll
                for (int k = 0; k < 5; ++k) acc[20 + k] += f2i(v[k]);
            }
        }
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
    }

    if (!failed) {
        // 7. the band's sums: Gram rows by their lanes, then the raw sums
        //    into the unit with one atomic per entry
        const int r = m >> 3, c = m & 7;
        if (fold_lane && r < 5 && c < 5) {
            const int ia = c * 5 + r;
#pragma unroll
            for (int j = 0; j < 25; ++j) S.hacc[ia * 25 + (j % 5) * 5 + j / 5] = acc[j];
            S.macc[ia] = acc[25];
            S.eacc[ia] = acc[26];
        }
        unsigned v4[4] = {s_sum, e_blk, e_rgt, e_bot};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            unsigned x = v4[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if (lane == 0) atomicAdd(&S.red[k], (unsigned long long)x);
        }
        __syncthreads();
        const long long n = (long long)rows * uw, sp = (long long)S.red[0] - 128 * n, k2 = 16384 * n;
        for (int q = t; q < 625; q += THREADS) {
            const int ia = q / 25, ib = q - ia * 25;
            if (ib < ia) continue;
            const long long h = (long long)S.hacc[q] + 128 * ((long long)S.eacc[ia] + S.eacc[ib]) + k2;
            if (h) atomicAdd((unsigned long long *)&u.h[q], (unsigned long long)h);
        }
        if (t < 25) {
            const long long e = S.eacc[t];
            atomicAdd((unsigned long long *)&u.m[t], (unsigned long long)((long long)S.macc[t] + 128 * e + 128 * sp + k2));
            atomicAdd((unsigned long long *)&u.s[t], (unsigned long long)(e + 128 * n));
        } else if (t == 32) {
            atomicAdd((unsigned long long *)&u.sum_src, S.red[0]);
            atomicAdd(&u.sse_blk, S.red[1]);
            atomicAdd(&u.sse_rgt, S.red[2]);
            atomicAdd(&u.sse_bot, S.red[3]);
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

size_t lr_stats_tc_smem() { return sizeof(Smem); }
int lr_stats_tc_rows() { return TR; }

}  // namespace zf
