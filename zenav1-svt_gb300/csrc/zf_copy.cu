// zf_copy.cu -- many plane copies in one launch, between the context's arena
// and caller host memory that the device addresses directly (page-locked
// memory mapped into the device address space: cudaPointerGetAttributes
// reports a device pointer for it).
//
// A batch of small images through host buffers is otherwise hundreds of
// cudaMemcpyAsync calls, each with its own fixed cost; here the copies are
// split into 64 KiB chunks and the CTAs of one launch take the chunks, with
// 16-byte accesses where both ends are 16-byte aligned, so the device reads
// (and writes) the host memory over the chip-to-chip link at streaming rate.
#include <algorithm>

#include "zf_kernels.cuh"

namespace zf {

__global__ void __launch_bounds__(256) k_copy_list(const CopyJob *jobs, int njobs, uint64_t nchunks) {
    for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        // the job whose chunk range holds c: the last with first_chunk <= c
        int lo = 0, hi = njobs - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (jobs[mid].first_chunk <= c) lo = mid;
            else hi = mid - 1;
        }
        const CopyJob j = jobs[lo];
        const uint64_t off = (c - j.first_chunk) * (uint64_t)kCopyChunk;
        if (off >= j.bytes) continue;
        const uint64_t n = min((uint64_t)kCopyChunk, j.bytes - off);
        const uint8_t *s = j.src + off;
        uint8_t *d = j.dst + off;
        const uintptr_t align = (uintptr_t)s | (uintptr_t)d;
        uint64_t done = 0;
        if ((align & 15) == 0) {
            const uint64_t n16 = n >> 4;
            const uint4 *s16 = reinterpret_cast<const uint4 *>(s);
            uint4 *d16 = reinterpret_cast<uint4 *>(d);
            for (uint64_t i = threadIdx.x; i < n16; i += blockDim.x) d16[i] = s16[i];
            done = n16 << 4;
        } else if ((align & 3) == 0) {
            const uint64_t n4 = n >> 2;
            const uint32_t *s4 = reinterpret_cast<const uint32_t *>(s);
            uint32_t *d4 = reinterpret_cast<uint32_t *>(d);
            for (uint64_t i = threadIdx.x; i < n4; i += blockDim.x) d4[i] = s4[i];
            done = n4 << 2;
        }
        for (uint64_t i = done + threadIdx.x; i < n; i += blockDim.x) d[i] = s[i];
    }
}

cudaError_t launch_copy_list(const CopyJob *jobs, int njobs, uint64_t nchunks, cudaStream_t st) {
    if (njobs <= 0 || nchunks == 0) return cudaSuccess;
    const int ctas = (int)std::min<uint64_t>(nchunks, 152ull * 8);
    k_copy_list<<<ctas, 256, 0, st>>>(jobs, njobs, nchunks);
    return cudaGetLastError();
}

}  // namespace zf
