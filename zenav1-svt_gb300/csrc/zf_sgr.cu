// zf_sgr.cu -- self-guided restoration (RESTORE_SGRPROJ) on the GPU.
//
// The reference encoder never searches or signals SGRPROJ
// (svtav1-dsp/src/restoration.rs:1280, svtav1-encoder/src/restoration.rs:8);
// its project documents the filter (specs/08-loop-filters.md:371-421). The
// arithmetic here is the AV1 specification's box filter process and
// self-guided filter process (section 7.17.3) with the decoder's
// stripe-aware sample fetch for the apply; the per-unit search (every set
// of a mask, least-squares projection weights solved exactly in 128-bit
// integers, SSE of the filtered unit) is this library's own.
//
// Work is tiled 64 columns x 32 rows. A CTA stages its tile with a 3-sample
// halo, forms the box sums of radius 1 and 2 once (they do not depend on
// the parameter set), then per set the A/B images of the two passes over
// the tile extended by one sample, then the filter outputs of its pixels.
//   k_sgr_search (phase 0): per (unit, set) the projection sums
//       H00 = sum f0^2, H01 = sum f0 f1, H11 = sum f1^2, C0 = sum f0 s,
//       C1 = sum f1 s (f = flt - u, s = (src << 4) - u, u = dgd << 4) and
//       the unit's unfiltered SSE;
//   k_sgr_solve: the weights of every (unit, set);
//   k_sgr_search (phase 1): the SSE of the unit filtered with them;
//   k_sgr_pick: the set of the smallest SSE per unit (lowest set on ties);
//   k_sgr_apply: decoder-exact apply per (stripe, tile).
#include "zf_kernels.cuh"

namespace zf {

namespace {

constexpr int kTW = kSgrTileWHost, kTH = kSgrTileHHost;  // tile
constexpr int kXW = kTW + 6, kXH = kTH + 6;               // staged samples (halo 3)
constexpr int kPW = kTW + 2, kPH = kTH + 2;               // A/B positions (halo 1)
constexpr int kNP = kPW * kPH;
constexpr int kThreads = 256;

// Sgr_Params of the AV1 specification: (r0, eps0, r1, eps1).
__constant__ int c_sgr_params[16][4] = {{2, 12, 1, 4},  {2, 15, 1, 6},  {2, 18, 1, 8},  {2, 21, 1, 9},
                                        {2, 24, 1, 10}, {2, 29, 1, 11}, {2, 36, 1, 12}, {2, 45, 1, 13},
                                        {2, 56, 1, 14}, {2, 68, 1, 15}, {0, 0, 1, 5},   {0, 0, 1, 8},
                                        {0, 0, 1, 11},  {0, 0, 1, 14},  {2, 30, 0, 0},  {2, 75, 0, 0}};

struct SgrSmem {
    int16_t X[kXH * kXW];   // staged samples
    int16_t S2[kNP], S1[kNP];  // box sums of radius 2 and 1 (<= 25 * 1023)
    int32_t Q2[kNP], Q1[kNP];  // box sums of squares
    int16_t A0[kNP], A1[kNP];  // a2 of pass 0 / 1 (<= 256)
    int32_t B0[kNP], B1[kNP];
    int16_t xbx[256];          // ((z << 8) + z / 2) / (z + 1), z < 255
    long long red[kThreads / 32][6];
};

__device__ __forceinline__ int ldpx_s(const uint8_t *p, int64_t idx, int bd) {
    return bd == 8 ? (int)p[idx] : (int)reinterpret_cast<const uint16_t *>(p)[idx];
}

// Stage rows [y0 - 3, y0 + h + 3) x cols [x0 - 3, x0 + w + 3). Search
// (stripe_start > stripe_end): samples clamped to the plane. Apply: the
// decoder's get_source_sample for the stripe [stripe_start, stripe_end].
__device__ void sgr_stage(SgrSmem &sm, const SgrPlaneDesc &P, int x0, int y0, int w, int h, int stripe_start,
                          int stripe_end) {
    const bool apply = stripe_start <= stripe_end;
    const int rows = h + 6, cols = w + 6;
    for (int q = threadIdx.x; q < rows * cols; q += blockDim.x) {
        const int r = q / cols, c = q - r * cols;
        const int x = min(max(x0 - 3 + c, 0), P.pw - 1);
        int y = min(max(y0 - 3 + r, 0), P.ph - 1);
        const uint8_t *pl = P.dgd;
        if (apply) {
            if (y < stripe_start) {
                y = max(stripe_start - 2, y);
                pl = P.pre;
            } else if (y > stripe_end) {
                y = min(stripe_end + 2, y);
                pl = P.pre;
            }
        }
        sm.X[r * kXW + c] = (int16_t)ldpx_s(pl, (int64_t)y * P.pw + x, P.bd);
    }
}

// Box sums of radius 1 and 2 at the positions [-1, h + 1) x [-1, w + 1).
__device__ void sgr_box_sums(SgrSmem &sm, int w, int h) {
    const int pw = w + 2, np = pw * (h + 2);
    for (int q = threadIdx.x; q < np; q += blockDim.x) {
        const int i = q / pw, j = q - i * pw;  // position (i - 1, j - 1); staged centre (i + 2, j + 2)
        int s2 = 0, q2 = 0, s1 = 0, q1 = 0;
#pragma unroll
        for (int dy = 0; dy < 5; ++dy)
#pragma unroll
            for (int dx = 0; dx < 5; ++dx) {
                const int c = sm.X[(i + dy) * kXW + j + dx];
                s2 += c;
                q2 += c * c;
                if (dy >= 1 && dy <= 3 && dx >= 1 && dx <= 3) {
                    s1 += c;
                    q1 += c * c;
                }
            }
        sm.S2[i * kPW + j] = (int16_t)s2;
        sm.Q2[i * kPW + j] = q2;
        sm.S1[i * kPW + j] = (int16_t)s1;
        sm.Q1[i * kPW + j] = q1;
    }
}

__device__ __forceinline__ int round2i(int x, int n) { return n ? (x + (1 << (n - 1))) >> n : x; }

// A/B of one pass (radius r, scale s) from the box sums.
__device__ __forceinline__ void sgr_ab(const SgrSmem &sm, int r, int s, int bd, int sum, int sq, int16_t &A,
                                       int32_t &B) {
    const int n = (2 * r + 1) * (2 * r + 1);
    const int one_over_n = r == 1 ? 455 : 164;  // ((1 << 12) + n / 2) / n
    const int a = round2i(sq, 2 * (bd - 8)), d = round2i(sum, bd - 8);
    const int p = max(0, a * n - d * d);
    const unsigned long long ps = (unsigned long long)p * (unsigned)s;
    const unsigned z = (unsigned)((ps + (1ull << 19)) >> 20);
    const int a2 = z >= 255 ? 256 : (z == 0 ? 1 : sm.xbx[z]);
    const unsigned b2 = (unsigned)(256 - a2) * (unsigned)sum * (unsigned)one_over_n;
    A = (int16_t)a2;
    B = (int32_t)((b2 + (1u << 11)) >> 12);
}

__device__ __forceinline__ int sgr_scale(int r, int eps) {
    const int n = (2 * r + 1) * (2 * r + 1), n2e = n * n * eps;
    return ((1 << 20) + n2e / 2) / n2e;
}

// A/B images of both passes of a set over the positions.
__device__ void sgr_set_ab(SgrSmem &sm, int set, int bd, int w, int h) {
    const int r0 = c_sgr_params[set][0], r1 = c_sgr_params[set][2];
    const int s0 = r0 ? sgr_scale(r0, c_sgr_params[set][1]) : 0;
    const int s1 = r1 ? sgr_scale(r1, c_sgr_params[set][3]) : 0;
    const int pw = w + 2, np = pw * (h + 2);
    for (int q = threadIdx.x; q < np; q += blockDim.x) {
        const int i = q / pw, j = q - i * pw, k = i * kPW + j;
        if (r0) sgr_ab(sm, 2, s0, bd, sm.S2[k], sm.Q2[k], sm.A0[k], sm.B0[k]);
        if (r1) sgr_ab(sm, 1, s1, bd, sm.S1[k], sm.Q1[k], sm.A1[k], sm.B1[k]);
    }
}

// Filter outputs of the two passes at tile pixel (i, j) (absolute row y).
__device__ __forceinline__ void sgr_flt(const SgrSmem &sm, int set, int i, int j, int y, int px, int &f0,
                                        int &f1) {
    const int r0 = c_sgr_params[set][0], r1 = c_sgr_params[set][2];
    const int k = (i + 1) * kPW + (j + 1);
    f0 = f1 = 0;
    if (r0) {
        int a, b, shift;
        if (y & 1) {  // odd row: its own A/B row, weights 6 / 5
            a = 6 * sm.A0[k] + 5 * (sm.A0[k - 1] + sm.A0[k + 1]);
            b = 6 * sm.B0[k] + 5 * (sm.B0[k - 1] + sm.B0[k + 1]);
            shift = 4;
        } else {  // even row: the rows above and below
            const int u = k - kPW, d = k + kPW;
            a = 6 * (sm.A0[u] + sm.A0[d]) + 5 * (sm.A0[u - 1] + sm.A0[u + 1] + sm.A0[d - 1] + sm.A0[d + 1]);
            b = 6 * (sm.B0[u] + sm.B0[d]) + 5 * (sm.B0[u - 1] + sm.B0[u + 1] + sm.B0[d - 1] + sm.B0[d + 1]);
            shift = 5;
        }
        f0 = round2i(a * px + b, 8 + shift - 4);
    }
    if (r1) {
        const int u = k - kPW, d = k + kPW;
        const int a = 4 * (sm.A1[k] + sm.A1[k - 1] + sm.A1[k + 1] + sm.A1[u] + sm.A1[d]) +
                      3 * (sm.A1[u - 1] + sm.A1[u + 1] + sm.A1[d - 1] + sm.A1[d + 1]);
        const int b = 4 * (sm.B1[k] + sm.B1[k - 1] + sm.B1[k + 1] + sm.B1[u] + sm.B1[d]) +
                      3 * (sm.B1[u - 1] + sm.B1[u + 1] + sm.B1[d - 1] + sm.B1[d + 1]);
        f1 = round2i(a * px + b, 8 + 5 - 4);
    }
}

// The self-guided projection: restored sample from the centre sample, the
// pass outputs and the weights (w2 = 128 - w0 - w1).
__device__ __forceinline__ int sgr_project(int set, int bd, int px, int f0, int f1, int w0, int w1) {
    const int w2 = 128 - w0 - w1, u = px << 4;
    int v = w1 * u;
    v += c_sgr_params[set][0] ? w0 * f0 : w0 * u;
    v += c_sgr_params[set][2] ? w2 * f1 : w2 * u;
    const int o = (v + (1 << 10)) >> 11;
    return min(max(o, 0), (1 << bd) - 1);
}

__device__ void sgr_fill_xbx(SgrSmem &sm) {
    for (int z = threadIdx.x; z < 256; z += blockDim.x) sm.xbx[z] = (int16_t)(z ? ((z << 8) + z / 2) / (z + 1) : 1);
}

// Block sum of up to 6 int64 values; thread 0 holds the result.
__device__ void block_sum6(SgrSmem &sm, long long (&v)[6], int nv) {
    for (int k = 0; k < nv; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
        for (int k = 0; k < nv; ++k) sm.red[warp][k] = v[k];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < nv; ++k) {
            long long t = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sm.red[w][k];
            v[k] = t;
        }
    __syncthreads();
}

}  // namespace

__global__ void __launch_bounds__(kThreads) k_sgr_search(SgrPlaneDesc P, const SgrTile *tiles, const int *sets,
                                                         int nsets, SgrAcc *acc, long long *sse_none, int phase) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    SgrSmem &sm = *reinterpret_cast<SgrSmem *>(smem_raw);
    const SgrTile t = tiles[blockIdx.x];
    sgr_fill_xbx(sm);
    sgr_stage(sm, P, t.x0, t.y0, t.w, t.h, 1, 0);
    __syncthreads();
    sgr_box_sums(sm, t.w, t.h);
    const int npx = t.w * t.h;
    if (phase == 0) {
        long long v[6] = {0, 0, 0, 0, 0, 0};
        for (int q = threadIdx.x; q < npx; q += blockDim.x) {
            const int i = q / t.w, j = q - i * t.w;
            const int64_t idx = (int64_t)(t.y0 + i) * P.pw + t.x0 + j;
            const int e = ldpx_s(P.src, idx, P.bd) - sm.X[(i + 3) * kXW + j + 3];
            v[0] += e * e;
        }
        block_sum6(sm, v, 1);
        if (threadIdx.x == 0) atomicAdd((unsigned long long *)&sse_none[t.unit], (unsigned long long)v[0]);
    }
    for (int si = 0; si < nsets; ++si) {
        const int set = sets[si];
        __syncthreads();  // box sums ready / the previous set's outputs read
        sgr_set_ab(sm, set, P.bd, t.w, t.h);
        __syncthreads();
        SgrAcc &a = acc[(size_t)t.unit * nsets + si];
        const int w0 = phase ? a.w[0] : 0, w1 = phase ? a.w[1] : 0;
        const bool r0 = c_sgr_params[set][0] != 0, r1 = c_sgr_params[set][2] != 0;
        long long v[6] = {0, 0, 0, 0, 0, 0};
        for (int q = threadIdx.x; q < npx; q += blockDim.x) {
            const int i = q / t.w, j = q - i * t.w;
            const int px = sm.X[(i + 3) * kXW + j + 3];
            const int sv = ldpx_s(P.src, (int64_t)(t.y0 + i) * P.pw + t.x0 + j, P.bd);
            int f0, f1;
            sgr_flt(sm, set, i, j, t.y0 + i, px, f0, f1);
            if (phase == 0) {
                const int u = px << 4, s = (sv << 4) - u;
                const long long g0 = r0 ? f0 - u : 0, g1 = r1 ? f1 - u : 0;
                v[0] += g0 * g0;
                v[1] += g0 * g1;
                v[2] += g1 * g1;
                v[3] += g0 * s;
                v[4] += g1 * s;
            } else {
                const int e = sv - sgr_project(set, P.bd, px, f0, f1, w0, w1);
                v[5] += (long long)e * e;
            }
        }
        block_sum6(sm, v, 6);
        if (threadIdx.x == 0) {
            if (phase == 0)
                for (int k = 0; k < 5; ++k) atomicAdd((unsigned long long *)&a.sums[k], (unsigned long long)v[k]);
            else
                atomicAdd((unsigned long long *)&a.sse, (unsigned long long)v[5]);
        }
    }
}

namespace {
// n * 128 / d rounded half away from zero (d > 0).
__device__ long long div_round128(__int128 n, __int128 d) {
    const __int128 q = n * 128;
    return (long long)(q >= 0 ? (2 * q + d) / (2 * d) : -((-2 * q + d) / (2 * d)));
}
}  // namespace

__global__ void k_sgr_solve(const int *sets, int nsets, SgrAcc *acc, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    SgrAcc &a = acc[k];
    const int set = sets[k % nsets];
    const long long H00 = a.sums[0], H01 = a.sums[1], H11 = a.sums[2], C0 = a.sums[3], C1 = a.sums[4];
    const int r0 = c_sgr_params[set][0], r1 = c_sgr_params[set][2];
    long long xq0 = 0, xq1 = 0;
    if (r0 && r1) {
        const __int128 det = (__int128)H00 * H11 - (__int128)H01 * H01;
        if (det > 0) {
            xq0 = div_round128((__int128)H11 * C0 - (__int128)H01 * C1, det);
            xq1 = div_round128((__int128)H00 * C1 - (__int128)H01 * C0, det);
        }
    } else if (r0) {
        if (H00 > 0) xq0 = div_round128(C0, H00);
    } else if (H11 > 0) {
        xq1 = div_round128(C1, H11);
    }
    auto clampw = [](long long v, int lo, int hi) { return (int)min(max(v, (long long)lo), (long long)hi); };
    int w0, w1;
    if (r0 && r1) {
        w0 = clampw(xq0, -96, 31);
        w1 = clampw(128 - w0 - xq1, -32, 95);
    } else if (r0) {
        w0 = clampw(xq0, -96, 31);
        w1 = clampw(128 - w0, -32, 95);
    } else {
        w0 = 0;
        w1 = clampw(128 - xq1, -32, 95);
    }
    a.w[0] = w0;
    a.w[1] = w1;
}

__global__ void k_sgr_pick(const int *sets, int nsets, const SgrAcc *acc, const long long *sse_none,
                           zf_sgr_unit *out, int nunits) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nunits) return;
    int best = -1;
    long long bsse = 0;
    for (int k = 0; k < nsets; ++k) {  // sets ascend: strict < keeps the lowest on ties
        const SgrAcc &a = acc[(size_t)u * nsets + k];
        if (best < 0 || a.sse < bsse) {
            best = k;
            bsse = a.sse;
        }
    }
    zf_sgr_unit o;
    o.set = sets[best];
    o.xqd[0] = acc[(size_t)u * nsets + best].w[0];
    o.xqd[1] = acc[(size_t)u * nsets + best].w[1];
    o.pad = 0;
    o.sse = bsse;
    o.sse_none = sse_none[u];
    out[u] = o;
}

__global__ void __launch_bounds__(kThreads) k_sgr_apply(SgrPlaneDesc P, const SgrTile *tiles, const zf_sgr_unit *units) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    SgrSmem &sm = *reinterpret_cast<SgrSmem *>(smem_raw);
    const SgrTile t = tiles[blockIdx.x];
    const zf_sgr_unit u = units[t.unit];
    const int npx = t.w * t.h;
    if (u.set < 0) {
        for (int q = threadIdx.x; q < npx; q += blockDim.x) {
            const int i = q / t.w, j = q - i * t.w;
            const int64_t idx = (int64_t)(t.y0 + i) * P.pw + t.x0 + j;
            if (P.bd == 8) P.dst[idx] = P.dgd[idx];
            else reinterpret_cast<uint16_t *>(P.dst)[idx] = reinterpret_cast<const uint16_t *>(P.dgd)[idx];
        }
        return;
    }
    sgr_fill_xbx(sm);
    sgr_stage(sm, P, t.x0, t.y0, t.w, t.h, t.stripe_start, t.stripe_end);
    __syncthreads();
    sgr_box_sums(sm, t.w, t.h);
    __syncthreads();
    sgr_set_ab(sm, u.set, P.bd, t.w, t.h);
    __syncthreads();
    for (int q = threadIdx.x; q < npx; q += blockDim.x) {
        const int i = q / t.w, j = q - i * t.w;
        const int64_t idx = (int64_t)(t.y0 + i) * P.pw + t.x0 + j;
        const int px = ldpx_s(P.dgd, idx, P.bd);  // the centre sample is the post-CDEF plane's
        int f0, f1;
        sgr_flt(sm, u.set, i, j, t.y0 + i, px, f0, f1);
        const int o = sgr_project(u.set, P.bd, px, f0, f1, u.xqd[0], u.xqd[1]);
        if (P.bd == 8) P.dst[idx] = (uint8_t)o;
        else reinterpret_cast<uint16_t *>(P.dst)[idx] = (uint16_t)o;
    }
}

size_t sgr_smem_bytes() { return sizeof(SgrSmem); }

cudaError_t sgr_set_attributes() {
    cudaError_t e = cudaFuncSetAttribute(k_sgr_search, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(SgrSmem));
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_sgr_apply, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SgrSmem));
}

}  // namespace zf
