// zf_kernels.cuh -- kernel entry points of the filter stage (defined in
// zf_deblock.cu, zf_cdef.cu, zf_lr.cu; launched from zf_host.cu).
#pragma once

#include "../../include/zf_filter.h"
#include "zf_dev.cuh"

namespace zf {

__global__ void k_deblock_apply(const FrameDesc *frames, const WorkItem *items, int nitems);
// Wiener statistics of 8-bit 5-tap planes on the tensor cores
// (zf_lr_tc.cu): 128 threads, lr_stats_tc_smem() dynamic shared memory,
// one CTA per band of lr_stats_tc_rows() output rows of a unit.
__global__ void k_lr_stats_tc(FrameDesc *frames, const WorkItem *items, int nitems);
size_t lr_stats_tc_smem();
int lr_stats_tc_rows();
// levels per (frame, plane) slot in one k_deblock_sse launch (at most)
constexpr int kDbLevels = 8;
__global__ void k_deblock_sse(const FrameDesc *frames, const WorkItem *items, int nitems, const int *levels, int nl,
                              unsigned long long *sse);

// CDEF search over a batch whose candidate grids are at most fp x ns.
cudaError_t launch_cdef_search(int fp, int ns, int ctas, cudaStream_t st, const FrameDesc *frames,
                               const WorkItem *items, int nitems);
__global__ void k_cdef_finish(FrameDesc *frames, const int *frame_ids, int smem_bytes);
__global__ void k_cdef_finish1(FrameDesc *frames, const int *frame_ids);
// Dynamic shared memory of k_cdef_finish1 for a frame; 0 when over `cap`.
int finish1_smem(int nfb, int ncand, int cap);
constexpr int kFin1ThreadsHost = 1024;
constexpr int kFinClusterMaxHost = 16;  // k_cdef_finish: non-portable cluster size when allowed
// k_cdef_finish over `nclusters` clusters of `cl` CTAs (cluster size set at launch).
cudaError_t launch_cdef_finish(int nclusters, int cl, size_t smem, cudaStream_t st, FrameDesc *frames,
                               const int *frame_ids, int smem_bytes);
// 16 when a 16-CTA cluster of k_cdef_finish with `smem` dynamic bytes fits the device, else 8.
int finish_cluster_size(size_t smem);
// k_cdef_joint (one CTA per (frame, bit count), rows in registers' reach):
// rows per thread for a frame (1, 2 or 4; 0 when the frame is outside its
// range), the launch over `nframes` frames of one (ncand, rpt) group, and
// the dynamic shared memory opt-in (once per device).
int joint_rows_per_thread(int nfb, int ncand);
cudaError_t launch_cdef_joint(int ncand, int rpt, int nframes, cudaStream_t st, FrameDesc *frames,
                              const int *frame_ids);
cudaError_t joint_set_attributes();
__global__ void k_cdef_apply(FrameDesc *frames, const WorkItem *items, int nitems);

cudaError_t launch_lr_stats(int win, int bd, int ctas, cudaStream_t st, FrameDesc *frames, const WorkItem *items,
                            int nitems);
__global__ void k_lr_solve(FrameDesc *frames, const WorkItem *items, int nitems);
// max_tiles: tiles per CTA its dynamic shared memory (lr_trial_smem) holds.
__global__ void k_lr_trial(FrameDesc *frames, const WorkItem *items, int nitems, int max_tiles);
size_t lr_trial_smem(int max_tiles);
__host__ __device__ int lr_trial_tiles_per_cta(int uw, int uh);
constexpr int kTrialMaxTilesHost = 9;  // a unit of at most 383 x 383: 6 x 12 tiles of 64 x 32 over 8 CTAs
// k_lr_trial_tiles<tl> (tile edge 32 or 64) over `ctas` tiles.
cudaError_t launch_lr_trial_tiles(int tl, int ctas, cudaStream_t st, FrameDesc *frames, const WorkItem *items,
                                  int nitems);
constexpr int kTrialClusterHost = 8;  // k_lr_trial: CTAs per unit (cluster size)
constexpr int kLrFinThreadsHost = 1024;  // k_lr_finish CTA size
constexpr int kLrPairMaxHost = 20100;   // k_lr_finish pair-table entries (units <= 200)
__global__ void k_lr_finish(FrameDesc *frames, int nframes);
__global__ void k_lr_apply(FrameDesc *frames, const WorkItem *items, int nitems, int group);

// One plane copy of a gathered copy launch (zf_copy.cu): bytes from src to
// dst (device addresses; host memory through its mapped address), taking
// chunks [first_chunk, first_chunk + ceil(bytes / kCopyChunk)) of the launch.
struct CopyJob {
    const uint8_t *src;
    uint8_t *dst;
    uint64_t bytes;
    uint64_t first_chunk;
};
constexpr int kCopyChunk = 64 * 1024;
cudaError_t launch_copy_list(const CopyJob *jobs, int njobs, uint64_t nchunks, cudaStream_t st);

// Fills dims and the CDEF policy of *d from a frame (host; zf_host.cu).
int describe_cdef_frame(const zf_frame *f, FrameDesc *d);

constexpr int kFinClusterHost = 8;  // k_cdef_finish: CTAs per cluster
constexpr int kFinThreadsHost = 512;
// k_lr_stats<win>: rows per CTA over the unit's rows extended by win/2 on
// both sides (one thread per (row, row offset), one per (row, window row)
// and one per row)
constexpr int stat_rows_host(int win) { return 256 / (3 * win); }

// ---- self-guided restoration (zf_sgr.cu) ----------------------------------
constexpr int kSgrTileWHost = 64, kSgrTileHHost = 32;  // tile (columns x rows)
struct SgrPlaneDesc {
    int bd, pw, ph, ss;      // tight planes: rows are pw samples apart
    const uint8_t *dgd;      // post-CDEF plane
    const uint8_t *src;      // source (search)
    const uint8_t *pre;      // post-deblock plane (apply: stripe-boundary rows)
    uint8_t *dst;            // apply output
};
struct SgrTile {
    int unit, x0, y0, w, h;
    int stripe_start, stripe_end;  // apply: the tile's stripe rows
    int pad;
};
struct SgrAcc {                // one (unit, set) of the search
    long long sums[5];         // H00, H01, H11, C0, C1
    long long sse;
    int w[2];
};
__global__ void k_sgr_search(SgrPlaneDesc P, const SgrTile *tiles, const int *sets, int nsets, SgrAcc *acc,
                             long long *sse_none, int phase);
__global__ void k_sgr_solve(const int *sets, int nsets, SgrAcc *acc, int n);
__global__ void k_sgr_pick(const int *sets, int nsets, const SgrAcc *acc, const long long *sse_none,
                           zf_sgr_unit *out, int nunits);
__global__ void k_sgr_apply(SgrPlaneDesc P, const SgrTile *tiles, const zf_sgr_unit *units);
size_t sgr_smem_bytes();
cudaError_t sgr_set_attributes();

// ---- superres upscale, film grain (zf_post.cu) ------------------------------
__global__ void k_superres_upscale(const uint8_t *src, int src_w, int src_stride, uint8_t *dst, int dst_w,
                                   int dst_stride, int bd, int x_step, int x0);
__global__ void k_grain_sums(const uint8_t *src, const uint8_t *rec, int w, int h, int stride, int rows_per_cta,
                             unsigned long long *out);
__global__ void k_grain_synth(uint8_t *frame, int w, int h, int stride, uint32_t seed, int scaling);
constexpr int kGrainRunHost = 32;  // k_grain_synth: pixels per thread

}  // namespace zf
