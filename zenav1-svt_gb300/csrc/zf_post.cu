// zf_post.cu -- the steps on either side of loop restoration: the normative
// superres upscale (after CDEF, before restoration when superres is on) and
// the film-grain estimate that follows the filter stage, plus the grain
// synthesis that pairs with it.
//
// Reference: svtav1-dsp/src/superres.rs (upscale_convolve_step :117,
// upscale_convolve_x0 :128, scaled_size :140, upscale_normative_row :208,
// upscale_normative_plane :252) and svtav1-encoder/src/film_grain.rs
// (estimate_film_grain :74, synthesize_grain :127; called after the
// restoration apply at pipeline.rs:3484-3485, its result unused).
#include "../../include/zf_av1_tables.h"
#include "zf_kernels.cuh"

namespace zf {

__device__ int16_t g_superres_filter[64][8] = ZF_SUPERRES_FILTER_INIT;

// A CTA per row: the filter table and the source row staged in shared
// memory (coalesced), then one output sample per thread step: x_qn = x0 +
// x * step (the reference's running x_qn += x_step_qn, exact for rows up to
// 16384 samples), taps at (x_qn >> 14) - 4 + k replicated at both edges (one
// tile column), rounded by 7 bits and clipped.
__global__ void __launch_bounds__(256) k_superres_upscale(const uint8_t *src, int src_w, int src_stride,
                                                          uint8_t *dst, int dst_w, int dst_stride, int bd,
                                                          int x_step, int x0) {
    __shared__ int16_t filt[64 * 8];
    extern __shared__ __align__(16) uint8_t srow_raw[];  // src_w samples of this row
    const int r = blockIdx.x;
    for (int q = threadIdx.x; q < 64 * 8; q += blockDim.x) filt[q] = (&g_superres_filter[0][0])[q];
    if (bd == 8) {
        const uint8_t *row = src + (int64_t)r * src_stride;
        for (int x = threadIdx.x; x < src_w; x += blockDim.x) srow_raw[x] = row[x];
    } else {
        const uint16_t *row = reinterpret_cast<const uint16_t *>(src) + (int64_t)r * src_stride;
        uint16_t *sr = reinterpret_cast<uint16_t *>(srow_raw);
        for (int x = threadIdx.x; x < src_w; x += blockDim.x) sr[x] = row[x];
    }
    __syncthreads();
    const int top = (1 << bd) - 1;
    for (int x = threadIdx.x; x < dst_w; x += blockDim.x) {
        const int x_qn = x0 + x * x_step;
        const int base = (x_qn >> 14) - 4;
        const int16_t *f = filt + ((x_qn & 16383) >> 8) * 8;
        int sum = 0;
        if (bd == 8) {
#pragma unroll
            for (int k = 0; k < 8; ++k) sum += (int)srow_raw[min(max(base + k, 0), src_w - 1)] * f[k];
        } else {
            const uint16_t *sr = reinterpret_cast<const uint16_t *>(srow_raw);
#pragma unroll
            for (int k = 0; k < 8; ++k) sum += (int)sr[min(max(base + k, 0), src_w - 1)] * f[k];
        }
        const int v = min(max((sum + 64) >> 7, 0), top);
        if (bd == 8) dst[(int64_t)r * dst_stride + x] = (uint8_t)v;
        else reinterpret_cast<uint16_t *>(dst)[(int64_t)r * dst_stride + x] = (uint16_t)v;
    }
}

// Sums of (source - recon) and its square over a u8 plane, four-byte dot
// products, one 64-bit atomic pair per CTA. Contiguous 16-byte-aligned
// planes (stride == width) are one flat run of 16-byte chunks, four loads
// in flight per thread; other layouts walk rows (16-byte chunks where the
// rows allow, otherwise bytes), rows_per_cta rows per CTA.
__device__ __forceinline__ void grain_chunk(const uint4 &va, const uint4 &vb, long long &s, unsigned long long &q) {
    const uint32_t xa[4] = {va.x, va.y, va.z, va.w}, xb[4] = {vb.x, vb.y, vb.z, vb.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        s += (long long)__dp4a(xa[i], 0x01010101u, 0u) - (long long)__dp4a(xb[i], 0x01010101u, 0u);
        const uint32_t e = __vabsdiffu4(xa[i], xb[i]);
        q += __dp4a(e, e, 0u);
    }
}

__global__ void __launch_bounds__(256) k_grain_sums(const uint8_t *src, const uint8_t *rec, int w, int h,
                                                    int stride, int rows_per_cta, unsigned long long *out) {
    long long s = 0;
    unsigned long long q = 0;
    const bool aligned = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(rec)) & 15) == 0;
    if (rows_per_cta == 0) {  // flat: stride == w, aligned
        const long long total = (long long)w * h, nchunk = total >> 4;
        const uint4 *a = reinterpret_cast<const uint4 *>(src), *b = reinterpret_cast<const uint4 *>(rec);
        const long long step = (long long)gridDim.x * blockDim.x;
        long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
        for (; k + 3 * step < nchunk; k += 4 * step) {
            uint4 va[4], vb[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                va[u] = a[k + u * step];
                vb[u] = b[k + u * step];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) grain_chunk(va[u], vb[u], s, q);
        }
        for (; k < nchunk; k += step) grain_chunk(a[k], b[k], s, q);
        if (blockIdx.x == 0)
            for (long long c = (nchunk << 4) + threadIdx.x; c < total; c += blockDim.x) {
                const int e = (int)src[c] - (int)rec[c];
                s += e;
                q += (unsigned long long)(e * e);
            }
    } else {
        const int r0 = blockIdx.x * rows_per_cta, r1 = min(h, r0 + rows_per_cta);
        const bool vec = (stride & 15) == 0 && aligned;
        for (int r = r0; r < r1; ++r) {
            const uint8_t *a = src + (int64_t)r * stride, *b = rec + (int64_t)r * stride;
            int c0 = 0;
            if (vec) {
                const int nchunk = w >> 4;
                for (int k = threadIdx.x; k < nchunk; k += blockDim.x)
                    grain_chunk(reinterpret_cast<const uint4 *>(a)[k], reinterpret_cast<const uint4 *>(b)[k], s, q);
                c0 = nchunk << 4;
            }
            for (int c = c0 + threadIdx.x; c < w; c += blockDim.x) {
                const int e = (int)a[c] - (int)b[c];
                s += e;
                q += (unsigned long long)(e * e);
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, o);
        q += __shfl_down_sync(0xffffffffu, q, o);
    }
    __shared__ long long ss[8];
    __shared__ unsigned long long sq[8];
    if ((threadIdx.x & 31) == 0) {
        ss[threadIdx.x >> 5] = s;
        sq[threadIdx.x >> 5] = q;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long ts = 0;
        unsigned long long tq = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
            ts += ss[k];
            tq += sq[k];
        }
        atomicAdd(&out[0], (unsigned long long)ts);
        atomicAdd(&out[1], tq);
    }
}

// synthesize_grain's linear congruential sequence, one update per pixel in
// raster order (index r * w + c). A thread takes kGrainRun consecutive
// pixels and starts from the state after `start` updates: the affine map
// s -> a s + c raised to that power by squaring (mod 2^32).
constexpr int kGrainRun = 32;
__global__ void __launch_bounds__(256) k_grain_synth(uint8_t *frame, int w, int h, int stride, uint32_t seed,
                                                     int scaling) {
    const long long total = (long long)w * h;
    const long long start = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * kGrainRun;
    if (start >= total) return;
    uint32_t A = 1, C = 0;  // f^start
    uint32_t pa = 1103515245u, pc = 12345u;  // f^(2^i)
    for (unsigned long long n = (unsigned long long)start; n; n >>= 1) {
        if (n & 1) {  // f^(2^i) after the accumulated map
            C = pa * C + pc;
            A = pa * A;
        }
        pc = pa * pc + pc;
        pa = pa * pa;
    }
    uint32_t st = A * seed + C;
    const int m = 2 * scaling + 1;
    const long long end = min(total, start + kGrainRun);
    int r = (int)(start / w), c = (int)(start - (long long)r * w);
    for (long long k = start; k < end; ++k) {
        st = st * 1103515245u + 12345u;
        const int noise = (int)(st >> 16) % m - scaling;
        uint8_t &p = frame[(int64_t)r * stride + c];
        p = (uint8_t)min(max((int)p + noise, 0), 255);
        if (++c == w) {
            c = 0;
            ++r;
        }
    }
}

}  // namespace zf
