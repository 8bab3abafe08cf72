"""Filter-stage throughput on GB300 (one JSON line on stdout).

Workload (N=1): the plain per-image 4K configuration -- four 3840x2160
8-bit 4:2:0 stills, presets {4, 6} x qp {24, 40}, seeded synthetic content
and stage inputs (zenav1-svt_gb300/synth.py). One step = the four frames,
each through zf_filter_stage (deblock pick + apply, CDEF search + apply,
Wiener search + apply), on four contexts (four streams) driven by four host
threads, one frame each.

  value  MPix/s with inputs resident in HBM (device pointers), timed by CUDA
         events that bracket every stream, L2 flushed between steps.
  e2e    the same through the C ABI with pinned HOST buffers (H2D of source,
         recon and geometry, D2H of the filtered recon and decisions inside
         the timed region).
  single_context  both, on one context, frame after frame.
  contexts  the device step on 1, 2 and 3 contexts (frames round-robin).

More keys on the same line (N=1 only):
  highres_10bit  one 4096x3072 10-bit preset-2 frame per step (u16 planes,
           20 CDEF candidates, deblock level search, Wiener refinement).
  batched  the 256-image mixed batch (sizes 64..2048, 8/10-bit) as one
           zf_submit_batch per step vs one zf_filter_stage per image on the
           same images (MPix/s each, their ratio, outputs identical),
           plus the batch through host buffers.
  sgr      self-guided restoration on one 3840x2160 8-bit frame's three
           planes: the per-unit search over all 16 parameter sets and the
           decoder-exact apply (the reference encoder has no SGRPROJ).
  post     the steps on either side of restoration on one 3840x2160 frame:
           the film-grain estimate (an HBM-streaming reduction; achieved
           GB/s against the measured copy peak) and the normative superres
           upscale of the luma plane from the denominator-16 width.
  served   Poisson arrivals at 50/200/800 req/s (sizes 128^2..6000x4000)
           through the continuous-batching loop (serve.py): p50/p99 latency
           and served MPix/s per rate.

--impl reference times the reference algorithm on the host cores: the
Rust reference cannot be built here, so this is the C++ oracle port on the
same four frames, as many copies of each at once as fill the host's cores,
one thread per copy.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

import __graft_entry__ as ge  # noqa: E402

METRIC = "byte-exact filter-stage MPix/s on 1 GB300, batched vs plain; p50/p99 latency"
DATA = ("synthetic (seeded 1/f^2 fields + shapes + noise; synthetic MD geometry; quantised-transform "
        "recon stand-in)")
WORKLOAD = [(4, 24), (4, 40), (6, 24), (6, 40)]  # (preset, qp)
W4K, H4K = 3840, 2160


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def make_workload(w=W4K, h=H4K, idx=0):
    """The four frames of the plain per-image workload (synth.workload_4k:
    the frames the full-size parity tests pin against the oracle); other
    sizes for profiling runs use the same seeds."""
    ge._pkg()
    from zenav1_svt_gb300 import synth
    if (w, h) == (W4K, H4K):
        return [synth.workload_4k(preset, qp, idx) for preset, qp in WORKLOAD]
    return [synth.make_frame(synth.frame_seed(2, idx * 16 + preset * 2 + (qp > 30)), w, h, 8, qp, preset, "power")
            for preset, qp in WORKLOAD]


def _gen_frame(job):
    """One synthetic frame (runs in a spawned worker process)."""
    ge._pkg()
    from zenav1_svt_gb300 import synth
    seed, w, h, bd, qp, preset, content = job
    return synth.make_frame(seed, w, h, bd, qp, preset, content)


def gen_frames(jobs):
    """Frames for (seed, w, h, bd, qp, preset, content) jobs on all host cores."""
    import multiprocessing as mp
    procs = max(1, min(len(jobs), (os.cpu_count() or 2) - 1))
    with mp.get_context("spawn").Pool(procs) as pool:
        return pool.map(_gen_frame, jobs, chunksize=1)


def batch_jobs(n):
    ge._pkg()
    from zenav1_svt_gb300 import synth
    return [(synth.frame_seed(4, i), w, h, bd, qp, 6, "cosine")
            for i, (w, h, bd, qp) in enumerate(synth.batch_specs(n))]


def served_jobs(n):
    ge._pkg()
    from zenav1_svt_gb300 import synth
    return [(synth.frame_seed(5, i), w, h, bd, qp, 6, "cosine")
            for i, (w, h, bd, qp) in enumerate(synth.served_specs(n))]


def stage_bytes(f):
    """Mandatory bytes of one frame: recon in, source in, recon out (1.5
    planes each at 1 or 2 bytes per sample) plus 4 bytes per 4x4 mi."""
    b = 1 if f.bd == 8 else 2
    return 3 * b * 1.5 * f.w * f.h + 4 * (f.w // 4) * (f.h // 4)


# --------------------------------------------------------------------------
# clocks
# --------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.tmp = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.tmp, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.tmp.flush()
        self.tmp.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.tmp.read().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.tmp.name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------------------
# reference arm: the oracle port on host cores
# --------------------------------------------------------------------------
def ours_config(nframes, world=1):
    """The `config` of the plain workload, shared by both arms' lines."""
    return {"workload": "plain per-image 3840x2160 8-bit 4:2:0, presets {4,6} x qp {24,40}",
            "frames_per_step": nframes,
            "l2": "GPU arm: flushed between steps (256 MB write); CPU arm: not applicable",
            "concurrency": "GPU arm: one context (one stream) per frame, one host thread each; "
                           "CPU arm: one host thread per frame copy",
            "parallelism": "replicas" if world > 1 else "single"}


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.lib()
    # the same four 3840x2160 frames as the GPU arm's step; the reference
    # stage is single-threaded per frame, so a step runs `reps` copies of
    # each frame at once, one host thread per copy, to keep every core busy
    frames = make_workload()
    cores = os.cpu_count() or 1
    reps = max(1, cores // len(frames))
    px = sum(f.luma_px for f in frames) * reps

    def step():
        jobs = [(f, f.copy_rec()) for f in frames for _ in range(reps)]
        ths = [threading.Thread(target=oracle.filter_stage, args=job) for job in jobs]
        t0 = time.perf_counter()
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        return time.perf_counter() - t0

    for _ in range(args.warmup):
        step()
    times = [step() for _ in range(args.steps)]
    tot = sum(times)
    value = px * len(times) / tot / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "MPix/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(tot / len(times) * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": DATA, "config": ours_config(len(frames), world),
            "cpu_baseline": {"value": round(value, 3), "unit": "MPix/s", "cores": min(cores, len(frames) * reps),
                             "kind": "port",
                             "sample": "the GPU arm's four 3840x2160 frames, %d copies of each per step, one host "
                                       "thread per copy (C++ oracle port; %d host cores)" % (reps, cores)},
            "e2e": {"value": round(value, 3), "unit": "MPix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def cpu_baseline_sample():
    """The oracle on one 3840x544 strip per (preset, qp), single thread."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.lib()
    frames = make_workload(W4K, 544, idx=1)
    t0 = time.perf_counter()
    for f in frames:
        oracle.filter_stage(f)
    dt = time.perf_counter() - t0
    px = sum(f.luma_px for f in frames)
    return {"value": round(px / dt / 1e6, 3), "unit": "MPix/s", "cores": 1, "kind": "port",
            "sample": "4 frames 3840x544 (presets {4,6} x qp {24,40}), one core, %.1f s" % dt}


# --------------------------------------------------------------------------
# our arm
# --------------------------------------------------------------------------
# Algorithmic bytes per launch for each kernel over one frame of W x H at
# `px` bytes per pixel (planes: luma + two quarter-size chroma = 1.5 W H).
def kernel_bytes(name, w, h, px):
    plane = 1.5 * w * h * px
    return {
        "k_deblock_apply": 2 * plane,      # read recon, write deblocked
        "k_deblock_sse": 2 * plane,        # read recon + source
        "k_cdef_search": 2 * plane,        # read deblocked + source
        "k_cdef_apply": 2 * plane,         # read deblocked, write CDEF output
        "k_lr_stats5": 2 * plane,          # read post-CDEF + source
        "k_lr_stats7": 2 * plane,
        "k_lr_trial": 2 * plane,
        "k_lr_trial_tiles": 3 * plane,     # read post-CDEF + source, write the restored plane
        "k_lr_apply": 2 * plane,           # at most: read post-CDEF, write restored (units without Wiener)
    }.get(name, 0.0)


# DRAM bytes (read + write) per luma pixel of one launch, from one ncu
# capture of each kernel's first launch in the bench's profile run (the
# 3840x2160 8-bit preset-4 qp-24 frame; the committed summary of the top
# kernels' captures); the roofline's `traffic` scales them to the launch's
# frame. The level trials' launches cover one plane kind each, so theirs is
# DRAM bytes per algorithmic byte of the captured launch (luma slot, four
# levels), scaled by the library's byte count of the average launch.
KERNEL_DRAM_BYTES_PER_PX = {
    "k_cdef_apply": 14.181376e6 / (3840 * 2160),
    "k_cdef_search": 26.4896e6 / (3840 * 2160),
    "k_lr_stats5": 25.799424e6 / (3840 * 2160),
    "k_cdef_finish": 0.19712e6 / (3840 * 2160),
    "k_deblock_apply": 14.568448e6 / (3840 * 2160),
    "k_lr_trial_tiles": (26.008064e6 + 2560.0) / (3840 * 2160),
    "k_lr_apply": 0.049664e6 / (3840 * 2160),
}
KERNEL_DRAM_PER_ALGO_BYTE = {
    "k_deblock_sse": 18.717952e6 / (2 * 3840 * 2160),
}


# Warp instructions executed per luma pixel of the plain 4K step, per
# kernel (ncu smsp__inst_executed.sum summed over the kernel's launches in
# one pass of the bench's four frames, divided by their luma pixels; the
# committed summary of the instruction-mix capture gives the command). The
# issue roofline of these integer-instruction-bound kernels: achieved warp
# instructions per second (these counts over the bench's own CUDA-event
# times of the same step) against the issue peak, four warp instructions
# per clock per SM at the SM clock sampled during the timed region.
KERNEL_WARP_INST_PER_PX = {
    "k_deblock_sse": 17.7277,
    "k_deblock_apply": 4.9196,
    "k_cdef_search": 11.2519,
    "k_cdef_apply": 5.2361,
    "k_lr_stats5": 5.3851,
    "k_lr_trial_tiles": 7.2574,
}


def issue_roofline(prof, frames, sm_count, sm_mhz):
    """int_frac of the three kernels with the largest device time in one step."""
    if not KERNEL_WARP_INST_PER_PX or not sm_mhz:
        return None
    peak = 4.0 * sm_count * sm_mhz * 1e6  # warp instructions per second
    px_step = float(sum(f.luma_px for f in frames))
    out = []
    for name, (nl, ms) in sorted(prof.items(), key=lambda kv: -kv[1][1]):
        ipp = KERNEL_WARP_INST_PER_PX.get(name)
        if ipp is None or ms <= 0:
            continue
        achieved = ipp * px_step / (ms / 1e3)
        out.append({"kernel": name, "warp_inst_per_px": round(ipp, 4), "achieved_winst_per_s": round(achieved, 1),
                    "peak_winst_per_s": round(peak, 1), "int_frac": round(achieved / peak, 4)})
        if len(out) == 3:
            break
    return {"unit": "warp instructions/s", "peak": "4 warp instructions/clock/SM x %d SMs x %.0f MHz (sampled)"
            % (sm_count, sm_mhz), "kernels": out}


def run_concurrent(ctxs, streams, work):
    """One step of the plain path on several contexts at once: host thread k
    runs work[k] (a list of (zf_frame, Decisions, ZfStats)) through
    zf_filter_stage on ctxs[k]. Device time from an event on streams[0]
    before any launch (the other streams wait on it) to an event on
    streams[0] after every stream's last launch (it waits on theirs), in
    ms."""
    import threading
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(streams[0])
    for st in streams[1:]:
        st.wait_event(e0)

    def worker(k):
        for s, d, stt in work[k]:
            ctxs[k].filter_stage_raw(s, d, stt)

    ths = [threading.Thread(target=worker, args=(k,)) for k in range(len(ctxs))]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    for st in streams[1:]:
        ev = torch.cuda.Event()
        ev.record(st)
        streams[0].wait_event(ev)
    e1.record(streams[0])
    e1.synchronize()
    return e0.elapsed_time(e1)


def run_ours(args):
    import torch
    rank, world, local = env_rank()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    ge.build()
    pkg = ge._pkg()
    from zenav1_svt_gb300 import abi, replicas

    frames = make_workload()
    mis = [pkg.pack_geom(f.geom) for f in frames]
    ctx = pkg.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    # the step runs on one context (one stream) per frame, one host thread
    # each, so one frame's copies, host round trips and few-CTA passes
    # overlap the others' streaming kernels (the four 4K frames: 2.44 ms a
    # step against 2.62 ms on two contexts, 3.31 ms on one)
    ctxs, streams = [ctx], [stream]
    for _ in range(1, len(frames)):
        c = pkg.Context(local)
        ctxs.append(c)
        streams.append(torch.cuda.ExternalStream(c.stream_handle(), device=dev))

    # device-resident inputs + a pristine copy of each recon
    d_src, d_rec, d_rec0, d_mi, structs, decs, stats = [], [], [], [], [], [], []
    for f, mi in zip(frames, mis):
        s = [torch.from_numpy(p.copy()).to(dev) for p in f.src]
        r0 = [torch.from_numpy(p.copy()).to(dev) for p in f.rec]
        r = [x.clone() for x in r0]
        m = torch.from_numpy(mi.view(np.int32).copy()).to(dev)
        d_src.append(s)
        d_rec0.append(r0)
        d_rec.append(r)
        d_mi.append(m)
        structs.append(abi.make_frame_struct(f, [x.data_ptr() for x in s], [x.data_ptr() for x in r], m.data_ptr(),
                                             on_device=True))
        decs.append(abi.Decisions(f.w, f.h, f.true_w, f.true_h))
        stats.append(abi.ZfStats())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # > 129 MB L2
    torch.cuda.synchronize()

    def restore():
        for r, r0 in zip(d_rec, d_rec0):
            for a, b in zip(r, r0):
                a.copy_(b)
        flush.fill_(1)
        torch.cuda.synchronize()

    def step_device():
        for s, d, st in zip(structs, decs, stats):
            ctx.filter_stage_raw(s, d, st)

    def split(items, nc=len(ctxs)):  # frames round-robin over nc contexts
        return [items[k::nc] for k in range(nc)]

    dev_work = split(list(zip(structs, decs, stats)))

    # correctness of the timed configuration: device run == oracle on frame 0
    # is covered by the -m gpu tests; here only the determinism across steps.
    for _ in range(args.warmup):
        restore()
        run_concurrent(ctxs, streams, dev_work)
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = sum(c.launch_count() for c in ctxs)
    times = []
    torch.cuda.synchronize()
    for _ in range(args.steps):
        restore()
        times.append(run_concurrent(ctxs, streams, dev_work))
    torch.cuda.synchronize()
    launches = sum(c.launch_count() for c in ctxs) - launches0
    clk = clocks.stop()
    px_step = sum(f.luma_px for f in frames)
    ms = float(np.mean(times))
    t_max = replicas.max_over_ranks(ms, device=dev)  # replicas: the slowest rank's time
    # the same step on one context, frame after frame
    single = []
    for k in range(args.warmup + args.steps):
        restore()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step_device()
        e1.record(stream)
        e1.synchronize()
        if k >= args.warmup:
            single.append(e0.elapsed_time(e1))
    single_ms = float(np.mean(single))
    # the same step on fewer contexts (frames round-robin, one host thread each)
    by_contexts = {}
    for nc in range(1, len(ctxs)):
        work = split(list(zip(structs, decs, stats)), nc)
        t_nc = []
        for k in range(args.warmup + args.steps):
            restore()
            ms_nc = run_concurrent(ctxs[:nc], streams[:nc], work)
            if k >= args.warmup:
                t_nc.append(ms_nc)
        by_contexts[str(nc)] = {"ms_per_step": round(float(np.mean(t_nc)), 3),
                                "value": round(px_step / (float(np.mean(t_nc)) / 1e3) / 1e6, 3)}

    # the same step with each call's launches run as a CUDA graph (not the
    # headline: a comparison of the two launch modes)
    g_times = []
    ctx.use_graphs(True)
    for k in range(args.warmup + args.steps):
        restore()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step_device()
        e1.record(stream)
        e1.synchronize()
        if k >= args.warmup:
            g_times.append(e0.elapsed_time(e1))
    g_stats = ctx.graph_stats()
    ctx.use_graphs(False)
    graphs = {"ms_per_step": round(float(np.mean(g_times)), 3), "direct_ms_per_step": round(single_ms, 3),
              "graph_launches": int(g_stats[0]), "updates": int(g_stats[1]), "instantiations": int(g_stats[2])}
    value = replicas.job_rate(px_step, world, t_max / 1e3) / 1e6

    # e2e: pinned host buffers through the C ABI
    h_src = [[torch.from_numpy(p.copy()).pin_memory() for p in f.src] for f in frames]
    h_rec0 = [[torch.from_numpy(p.copy()) for p in f.rec] for f in frames]
    h_rec = [[x.clone().pin_memory() for x in r] for r in h_rec0]
    h_mi = [torch.from_numpy(mi.view(np.int32).copy()).pin_memory() for mi in mis]
    e_structs = []
    for f, s, r, m in zip(frames, h_src, h_rec, h_mi):
        st = abi.ZfFrame()
        st.bit_depth, st.width, st.height = f.bd, f.w, f.h
        st.true_width, st.true_height, st.chroma_420 = f.true_w, f.true_h, 1
        st.preset, st.qindex, st.sharpness, st.sc_class5 = f.preset, f.qindex, 0, 0
        st.enable_restoration, st.planes_on_device = 1, 0
        for p in range(3):
            st.src[p] = s[p].data_ptr()
            st.rec[p] = r[p].data_ptr()
        st.mi = m.data_ptr()
        e_structs.append(st)
    h2d = sum(x.numel() * x.element_size() for r in h_rec for x in r) * 2 + sum(m.numel() * 4 for m in h_mi)
    d2h = sum(x.numel() * x.element_size() for r in h_rec for x in r)

    def restore_host():
        for r, r0 in zip(h_rec, h_rec0):
            for a, b in zip(r, r0):
                a.copy_(b)
        flush.fill_(1)
        torch.cuda.synchronize()

    host_work = split(list(zip(e_structs, decs, stats)))
    for _ in range(args.warmup):
        restore_host()
        run_concurrent(ctxs, streams, host_work)
    e_times = []
    for _ in range(args.steps):
        restore_host()
        e_times.append(run_concurrent(ctxs, streams, host_work))
    e_ms = replicas.max_over_ranks(float(np.mean(e_times)), device=dev)
    e2e = replicas.job_rate(px_step, world, e_ms / 1e3) / 1e6
    # one context, frame after frame
    e_single = []
    for k in range(args.warmup + args.steps):
        restore_host()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for s, d, st in zip(e_structs, decs, stats):
            ctx.filter_stage_raw(s, d, st)
        e1.record(stream)
        e1.synchronize()
        if k >= args.warmup:
            e_single.append(e0.elapsed_time(e1))
    e_single_ms = float(np.mean(e_single))

    # per-kernel device times (separate profiled pass, CUDA events per launch)
    restore()
    ctx.profile(True)
    ctx.profile_reset()
    step_device()
    ctx.sync()
    prof_b = ctx.profile_read_bytes()
    prof = {k: v[:2] for k, v in prof_b.items()}
    ctx.profile(False)
    # the dominant kernel among those that stream planes (the joint strength
    # search reads only the mse rows and is latency bound: it is listed in
    # `kernels` with the rest)
    streaming = {k: v for k, v in prof.items() if kernel_bytes(k, 64, 64, 1) > 0}
    top = max(streaming.items(), key=lambda kv: kv[1][1]) if streaming else ("none", (1, 0.0))
    name, (nl, tot_ms) = top
    per_launch_ms = tot_ms / max(nl, 1)
    # the library's own count where it records one (the level trials: each
    # launch reads the slots' planes and source planes once), else the
    # kernel's whole-frame formula
    lib_bytes = prof_b.get(name, (0, 0.0, 0))[2]
    bytes_per_launch = (lib_bytes / max(nl, 1) if lib_bytes
                        else np.mean([kernel_bytes(name, f.w, f.h, 1) for f in frames]))
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = bytes_per_launch / (per_launch_ms / 1e3) / 1e9 if per_launch_ms > 0 else 0.0
    bpp = KERNEL_DRAM_BYTES_PER_PX.get(name)
    if name in KERNEL_DRAM_PER_ALGO_BYTE:
        traffic = int(KERNEL_DRAM_PER_ALGO_BYTE[name] * bytes_per_launch)
        traffic_source = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of one luma trial launch of a "
                          "3840x2160 frame, per algorithmic byte, times the average launch's algorithmic bytes")
    else:
        traffic = int(bpp * np.mean([f.luma_px for f in frames])) if bpp else None
        traffic_source = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of one 4K launch, scaled by luma "
                          "pixels") if traffic else None
    roofline = {"bound": "hbm", "kernel": name, "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 5), "traffic": traffic,
                "algorithmic_bytes": int(bytes_per_launch),
                "traffic_source": traffic_source,
                "peak_source": "of measured" if "hbm_gbs" in peaks else "of fallback",
                "stage_bytes_per_px": 4.75,
                "stage_frac": round((4.75 * px_step / (ms / 1e3) / 1e9) / peak, 5)}
    kernels = {k: {"launches": v[0], "ms": round(v[1], 4)} for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])}

    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 3), "unit": "MPix/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t_max, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
                "data": DATA, "config": ours_config(len(frames), world),
                "e2e": {"value": round(e2e, 3), "unit": "MPix/s", "h2d_bytes_per_step": int(h2d),
                        "d2h_bytes_per_step": int(d2h), "ms_per_step": round(e_ms, 3)},
                "gpu_launches": int(launches),
                "single_context": {"ms_per_step": round(single_ms, 3),
                                   "value": round(px_step / (single_ms / 1e3) / 1e6, 3),
                                   "e2e_ms_per_step": round(e_single_ms, 3),
                                   "e2e_value": round(px_step / (e_single_ms / 1e3) / 1e6, 3)},
                "contexts": by_contexts,
                "roofline": roofline, "kernels": kernels, "clocks": clk, "graphs": graphs}
        sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
        ir = issue_roofline(prof, frames, sm_count, clk.get("sm_mhz"))
        if ir:
            line["roofline"]["int"] = ir
            line["roofline"]["int_frac"] = {k["kernel"]: k["int_frac"] for k in ir["kernels"]}
        if not args.no_cpu:
            line["cpu_baseline"] = cpu_baseline_sample()
        if world == 1:
            restore()  # the tuner copies the pre-deblock recon it is given
            line["autotune_4k"] = run_autotune_4k(ctx, frames, structs)
            line["plain_512"] = run_plain512(args, ctx, stream, dev)
            line["highres_10bit"] = run_highres10(args, ctx, stream, dev)
            line["sgr"] = run_sgr(args, ctx, stream, dev, frames[0])
            line["post"] = run_post(args, ctx, stream, dev, frames[0])
        if world == 1 and not args.no_batched:
            line["batched"] = run_batched(args, ctx, stream, dev, gen_frames(batch_jobs(args.batch_n)))
            print("batched:", json.dumps(line["batched"]), file=sys.stderr)
        if world == 1 and not args.no_served:
            line["served"] = run_served(args, local, gen_frames(served_jobs(32)))
        print(json.dumps(line))
    for c in ctxs:
        c.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_autotune_4k(ctx, frames, structs):
    """The autotuner on each 4K frame of the plain workload alone
    (zf_filter_stage per setting, the frame's recon restored before every
    call): the setting it keeps against the default, per frame."""
    pkg = ge._pkg()
    from zenav1_svt_gb300 import abi
    default = (0, 1, 8, 0, 64, 8)
    keys = ("graphs", "stats_tma", "apply_group", "stats_tc", "trial_tile", "db_levels")
    out = []
    for f, s in zip(frames, structs):
        one = (abi.ZfFrame * 1)()
        one[0] = s
        best, cands = ctx.autotune_raw(one, 1, reps=3)
        dflt = [c for c in cands if tuple(c[k] for k in keys) == default]
        out.append({"frame": "preset %d qp %d" % (f.preset, {96: 24, 160: 40}.get(f.qindex, f.qindex)),
                    "best": {k: best[k] for k in keys}, "best_ms": best["ms"],
                    "default_ms": dflt[0]["ms"] if dflt else None, "settings_timed": len(cands)})
        ctx.set_tune(*default)
    return out


def run_plain512(args, ctx, stream, dev):
    """The plain drop-in configuration: one 512x512 8-bit still, preset 6,
    qp 32 (closed-form deblock levels, 4 CDEF candidates), one
    zf_filter_stage per step: device-resident (L2 flushed between steps) and
    from pinned host buffers (copies inside the timed call), with the
    oracle's single-core time on the same frame beside it."""
    import torch
    pkg = ge._pkg()
    from zenav1_svt_gb300 import abi, synth
    f = synth.workload_plain_512()
    mi = pkg.pack_geom(f.geom)
    src = [torch.from_numpy(p).to(dev) for p in f.src]
    rec0 = [torch.from_numpy(p).to(dev) for p in f.rec]
    rec = [x.clone() for x in rec0]
    m = torch.from_numpy(mi.view(np.int32)).to(dev)
    s = abi.make_frame_struct(f, [x.data_ptr() for x in src], [x.data_ptr() for x in rec], m.data_ptr(),
                              on_device=True)
    h_src = [torch.from_numpy(p.copy()).pin_memory() for p in f.src]
    h_rec = [torch.from_numpy(p.copy()).pin_memory() for p in f.rec]
    h_mi = torch.from_numpy(mi.view(np.int32).copy()).pin_memory()
    hs = abi.make_frame_struct(f, [x.numpy() for x in h_src], [x.numpy() for x in h_rec], h_mi.numpy())
    d = abi.Decisions(f.w, f.h, f.true_w, f.true_h)
    st = abi.ZfStats()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def timed(struct, restore):
        out = []
        for k in range(args.warmup + max(args.steps, 10)):
            restore()
            flush.fill_(1)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.filter_stage_raw(struct, d, st)
            e1.record(stream)
            e1.synchronize()
            if k >= args.warmup:
                out.append(e0.elapsed_time(e1))
        return float(np.mean(out)), float(np.percentile(out, 99))

    def restore_dev():
        for a, b in zip(rec, rec0):
            a.copy_(b)

    def restore_host():
        for a, b in zip(h_rec, f.rec):
            a.numpy()[...] = b

    ms, p99 = timed(s, restore_dev)
    e_ms, e_p99 = timed(hs, restore_host)
    out = {"workload": "512x512 8-bit 4:2:0, preset 6, qp 32 (one frame per step)",
           "mpix_per_s": round(f.luma_px / (ms / 1e3) / 1e6, 3), "ms": round(ms, 4), "p99_ms": round(p99, 4),
           "e2e_mpix_per_s": round(f.luma_px / (e_ms / 1e3) / 1e6, 3), "e2e_ms": round(e_ms, 4),
           "e2e_p99_ms": round(e_p99, 4), "lf": d.as_dict()["lf"], "cdef_bits": d.as_dict()["cdef_bits"]}
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        t0 = time.perf_counter()
        for _ in range(5):
            oracle.filter_stage(f)
        cpu_ms = (time.perf_counter() - t0) / 5 * 1e3
        out["cpu_oracle_ms"] = round(cpu_ms, 3)
        out["cpu_oracle_mpix_per_s"] = round(f.luma_px / (cpu_ms / 1e3) / 1e6, 3)
    return out


def run_highres10(args, ctx, stream, dev):
    """The 10-bit high-resolution configuration: one 4096x3072 10-bit frame
    (u16 planes), preset 2 (20 CDEF candidates, deblock level search,
    Wiener refinement), qp 28; device-resident, one zf_filter_stage per
    step, L2 flushed between steps."""
    import torch
    pkg = ge._pkg()
    from zenav1_svt_gb300 import abi, synth
    f = synth.workload_10bit_4096()
    src = [torch.from_numpy(p).to(dev) for p in f.src]
    rec0 = [torch.from_numpy(p).to(dev) for p in f.rec]
    rec = [x.clone() for x in rec0]
    m = torch.from_numpy(pkg.pack_geom(f.geom).view(np.int32)).to(dev)
    s = abi.make_frame_struct(f, [x.data_ptr() for x in src], [x.data_ptr() for x in rec], m.data_ptr(),
                              on_device=True)
    d = abi.Decisions(f.w, f.h, f.true_w, f.true_h)
    st = abi.ZfStats()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    times = []
    for k in range(args.warmup + args.steps):
        for a, b in zip(rec, rec0):
            a.copy_(b)
        flush.fill_(1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.filter_stage_raw(s, d, st)
        e1.record(stream)
        e1.synchronize()
        if k >= args.warmup:
            times.append(e0.elapsed_time(e1))
    ms = float(np.mean(times))
    for a, b in zip(rec, rec0):
        a.copy_(b)
    torch.cuda.synchronize()
    ctx.profile(True)
    ctx.profile_reset()
    ctx.filter_stage_raw(s, d, st)
    ctx.sync()
    kern = {k: round(v[1], 4) for k, v in sorted(ctx.profile_read().items(), key=lambda kv: -kv[1][1])}
    ctx.profile(False)
    return {"workload": "4096x3072 10-bit 4:2:0 (u16), preset 2, qp 28, device-resident",
            "mpix_per_s": round(f.luma_px / (ms / 1e3) / 1e6, 3), "ms": round(ms, 3),
            "lf": d.as_dict()["lf"], "cdef_bits": d.as_dict()["cdef_bits"], "kernel_ms": kern}


def run_sgr(args, ctx, stream, dev, f):
    """Self-guided restoration of one 4K frame (Y, U, V): zf_sgr_search over
    all 16 sets, then zf_sgr_apply with the picked units; device-resident
    planes (the frame's recon stands in for the post-CDEF plane and for the
    post-deblock stripe lines), CUDA-event timed, L2 flushed per step."""
    import torch
    dsrc = [torch.from_numpy(p.astype(np.int16) if p.dtype == np.uint16 else p).to(dev) for p in f.src]
    ddgd = [torch.from_numpy(p.astype(np.int16) if p.dtype == np.uint16 else p).to(dev) for p in f.rec]
    dout = [torch.empty_like(x) for x in ddgd]
    bd = 8 if f.src[0].dtype == np.uint8 else 10
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def step():
        for pl in range(3):
            u = ctx.sgr_search(bd, ddgd[pl], dsrc[pl], ss_y=1 if pl else 0, on_device=True)
            ctx.sgr_apply(bd, ddgd[pl], ddgd[pl], u, ss_y=1 if pl else 0, dst=dout[pl], on_device=True)
        return u

    times = []
    for k in range(args.warmup + args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        e1.synchronize()
        if k >= args.warmup:
            times.append(e0.elapsed_time(e1))
    ms = float(np.mean(times))
    ctx.profile(True)
    ctx.profile_reset()
    step()
    ctx.sync()
    kern = {k: round(v[1], 4) for k, v in sorted(ctx.profile_read().items(), key=lambda kv: -kv[1][1])}
    ctx.profile(False)
    return {"workload": "3840x2160 8-bit 4:2:0 (Y, U, V), SGRPROJ search over 16 sets + apply, device-resident",
            "mpix_per_s": round(f.luma_px / (ms / 1e3) / 1e6, 3), "ms": round(ms, 3), "kernel_ms": kern}


def run_post(args, ctx, stream, dev, f):
    """Film-grain estimate (source vs recon, luma) and superres upscale
    (denominator 16: 1920 -> 3840 columns, 2160 rows) on device planes,
    CUDA-event timed per call, L2 flushed before each; the estimate's
    algorithmic bytes are the two luma planes it reads."""
    import torch
    import ctypes as C
    pkg = ge._pkg()
    from zenav1_svt_gb300 import abi
    L = pkg.lib()
    h, w = f.src[0].shape
    src = torch.from_numpy(f.src[0]).to(dev)
    rec = torch.from_numpy(f.rec[0]).to(dev)
    coded = L.zf_superres_scaled_size(w, 16)
    small = torch.from_numpy(np.ascontiguousarray(f.rec[0][:, :coded])).to(dev)
    up = torch.empty((h, w), dtype=torch.uint8, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    p = abi.ZfFilmGrain()

    def timed(fn):
        out = []
        for k in range(args.warmup + args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            ctx.profile(True)
            ctx.profile_reset()
            fn()
            ctx.sync()
            prof = ctx.profile_read()
            ctx.profile(False)
            if k >= args.warmup:
                out.append(sum(v[1] for v in prof.values()))
        return float(np.mean(out))

    ms_est = timed(lambda: ctx._check(L.zf_film_grain_estimate(ctx.h, src.data_ptr(), rec.data_ptr(), w, h, w, 1,
                                                                C.byref(p))))
    ms_up = timed(lambda: ctx._check(L.zf_superres_upscale(ctx.h, small.data_ptr(), coded, coded, up.data_ptr(), w,
                                                            w, h, 8, 1)))
    peak = _peaks().get("hbm_gbs")
    gbs = 2 * w * h / (ms_est / 1e3) / 1e9
    return {"workload": "3840x2160 8-bit luma: film-grain estimate; superres upscale %d -> %d columns" % (coded, w),
            "film_grain_ms": round(ms_est, 4), "film_grain_gbs": round(gbs, 1),
            "film_grain_frac_of_hbm": round(gbs / peak, 4) if peak else None,
            "film_grain_noise_var": round(p.noise_var, 4), "apply_grain": bool(p.apply_grain),
            "superres_ms": round(ms_up, 4),
            "superres_gbs": round((coded + w) * h / (ms_up / 1e3) / 1e9, 1)}


def run_batched(args, ctx, stream, dev, frames):
    """The 256-image mixed batch (W, H ~ U[64, 2048], ~20 % odd, 70 % 8-bit,
    qp ~ U[20, 50], preset 6): one zf_submit_batch call per step, against the
    plain path (one zf_filter_stage call per image) on the same images.
    Both device-resident; the batch also through host buffers (e2e)."""
    import torch
    pkg = ge._pkg()
    from zenav1_svt_gb300 import abi
    n = len(frames)
    mis = [pkg.pack_geom(f.geom) for f in frames]
    d_src = [[torch.from_numpy(p).to(dev) for p in f.src] for f in frames]
    d_rec0 = [[torch.from_numpy(p).to(dev) for p in f.rec] for f in frames]
    d_rec = [[x.clone() for x in r] for r in d_rec0]
    d_mi = [torch.from_numpy(m.view(np.int32)).to(dev) for m in mis]
    arr = (abi.ZfFrame * n)()
    darr = (abi.ZfDecisions * n)()
    st = (abi.ZfStats * n)()
    decs = [abi.Decisions(f.w, f.h, f.true_w, f.true_h) for f in frames]
    plain_decs = [abi.Decisions(f.w, f.h, f.true_w, f.true_h) for f in frames]
    singles = []
    for i, f in enumerate(frames):
        arr[i] = abi.make_frame_struct(f, [x.data_ptr() for x in d_src[i]], [x.data_ptr() for x in d_rec[i]],
                                       d_mi[i].data_ptr(), on_device=True)
        darr[i] = decs[i].c
        singles.append(abi.make_frame_struct(f, [x.data_ptr() for x in d_src[i]],
                                             [x.data_ptr() for x in d_rec[i]], d_mi[i].data_ptr(),
                                             on_device=True))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    px = sum(f.luma_px for f in frames)
    mand = sum(stage_bytes(f) for f in frames)

    def restore():
        for r, r0 in zip(d_rec, d_rec0):
            for a, b in zip(r, r0):
                a.copy_(b)
        flush.fill_(1)
        torch.cuda.synchronize()

    def timed(fn, steps):
        out = []
        for _ in range(steps):
            restore()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            out.append(e0.elapsed_time(e1))
        return float(np.mean(out))

    def batch():
        ctx.submit_batch_raw(arr, n, darr, st)

    one = abi.ZfStats()

    def plain():
        for s, d in zip(singles, plain_decs):
            ctx.filter_stage_raw(s, d, one)

    for _ in range(2):
        restore()
        batch()
    l0 = ctx.launch_count()
    b_ms = timed(batch, args.steps)
    b_launches = (ctx.launch_count() - l0) // max(args.steps, 1)
    out_batch = [[x.clone() for x in r] for r in d_rec]
    for i in range(n):
        decs[i].c = darr[i]
    dec_batch = [d.as_dict() for d in decs]
    # per-kernel device time of one batch (CUDA events per launch)
    restore()
    ctx.profile(True)
    ctx.profile_reset()
    batch()
    ctx.sync()
    b_kernels = {k: round(v[1], 4) for k, v in sorted(ctx.profile_read().items(), key=lambda kv: -kv[1][1])}
    ctx.profile(False)
    restore()
    plain()
    p_ms = timed(plain, max(2, args.steps // 2))
    # both forms again with every call's launches run as a CUDA graph
    ctx.use_graphs(True)
    restore()
    plain()
    pg_ms = timed(plain, max(2, args.steps // 2))
    restore()
    batch()
    bg_ms = timed(batch, args.steps)
    ctx.use_graphs(False)
    same = all(torch.equal(a, b) for ra, rb in zip(out_batch, d_rec) for a, b in zip(ra, rb))
    for a, d in zip(dec_batch, plain_decs):
        b = d.as_dict()
        same = same and a["lf"] == b["lf"] and a["cdef_y"] == b["cdef_y"] and a["cdef_uv"] == b["cdef_uv"] \
            and a["cdef_bits"] == b["cdef_bits"] and bool((a["cdef_fb_idx"] == b["cdef_fb_idx"]).all()) \
            and a["lr"] == b["lr"]

    # the same batch as two halves (images alternating) on two contexts at
    # once, one zf_submit_batch each from two host threads
    import threading
    ctx2 = pkg.Context(dev.index or 0)
    stream2 = torch.cuda.ExternalStream(ctx2.stream_handle(), device=dev)
    halves = [list(range(0, n, 2)), list(range(1, n, 2))]
    decs2 = [abi.Decisions(f.w, f.h, f.true_w, f.true_h) for f in frames]
    parts = []
    for hv in halves:
        ha = (abi.ZfFrame * len(hv))()
        hd = (abi.ZfDecisions * len(hv))()
        for k, i in enumerate(hv):
            ha[k] = arr[i]
            hd[k] = decs2[i].c
        parts.append((ha, len(hv), hd, (abi.ZfStats * len(hv))()))  # submit_batch_raw's arguments

    def batch2():
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        stream2.wait_event(e0)
        ths = [threading.Thread(target=c.submit_batch_raw, args=part) for c, part in zip((ctx, ctx2), parts)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        ev = torch.cuda.Event()
        ev.record(stream2)
        stream.wait_event(ev)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    for _ in range(2):
        restore()
        batch2()
    b2 = []
    for _ in range(args.steps):
        restore()
        b2.append(batch2())
    b2_ms = float(np.mean(b2))
    for hv, (ha, hn, hd, hs) in zip(halves, parts):
        for k, i in enumerate(hv):
            decs2[i].c = hd[k]
    same2 = all(torch.equal(a, b) for ra, rb in zip(out_batch, d_rec) for a, b in zip(ra, rb))
    for a, d in zip(dec_batch, decs2):
        b = d.as_dict()
        same2 = same2 and a["lf"] == b["lf"] and a["cdef_y"] == b["cdef_y"] and a["cdef_bits"] == b["cdef_bits"] \
            and bool((a["cdef_fb_idx"] == b["cdef_fb_idx"]).all()) and a["lr"] == b["lr"]
    ctx2.close()
    del out_batch

    # e2e: the batch from pinned host buffers (H2D and D2H inside the call)
    h_src = [[torch.from_numpy(p).pin_memory() for p in f.src] for f in frames]
    h_rec0 = [f.rec for f in frames]
    h_rec = [[torch.from_numpy(p.copy()).pin_memory() for p in f.rec] for f in frames]
    h_mi = [torch.from_numpy(m.view(np.int32).copy()).pin_memory() for m in mis]
    harr = (abi.ZfFrame * n)()
    for i, f in enumerate(frames):
        harr[i] = abi.make_frame_struct(f, [x.numpy() for x in h_src[i]], [x.numpy() for x in h_rec[i]],
                                        h_mi[i].numpy())
    h2d = sum(x.numel() * x.element_size() for r in h_rec for x in r) * 2 + sum(m.numel() * 4 for m in h_mi)
    e_times = []
    for k in range(2 + args.steps):
        for r, r0 in zip(h_rec, h_rec0):
            for a, b in zip(r, r0):
                a.numpy()[...] = b
        flush.fill_(1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.submit_batch_raw(harr, n, darr, st)
        e1.record(stream)
        e1.synchronize()
        if k >= 2:
            e_times.append(e0.elapsed_time(e1))
    e_ms = float(np.mean(e_times))
    # the autotuner on the same device-resident batch (it times every launch
    # setting on private copies of the recon); the context goes back to the
    # default setting afterwards
    best, cands = ctx.autotune_raw(arr, n, reps=2)
    default = (0, 1, 8, 0, 64, 8)  # graphs, stats_tma, apply_group, stats_tc, trial_tile, db_levels
    keys = ("graphs", "stats_tma", "apply_group", "stats_tc", "trial_tile", "db_levels")
    dflt = [c for c in cands if tuple(c[k] for k in keys) == default]
    ctx.set_tune(*default)
    tune = {"best": best, "default_ms": dflt[0]["ms"] if dflt else None, "candidates": len(cands)}
    peak = _peaks().get("hbm_gbs", 6800.0)
    return {"workload": "256 images, W,H ~ U[64,2048] (~20% odd), 70% 8-bit / 30% 10-bit, qp ~ U[20,50], preset 6",
            "images": n, "luma_mpix": round(px / 1e6, 3),
            "batched_mpix_per_s": round(px / (b_ms / 1e3) / 1e6, 3), "batched_ms": round(b_ms, 3),
            "launches_per_batch": int(b_launches), "kernel_ms": b_kernels,
            "plain_mpix_per_s": round(px / (p_ms / 1e3) / 1e6, 3), "plain_ms": round(p_ms, 3),
            "batched_over_plain": round(p_ms / b_ms, 3),
            "graphs": {"plain_ms": round(pg_ms, 3), "batched_ms": round(bg_ms, 3)},
            "two_contexts": {"batched_ms": round(b2_ms, 3), "batched_mpix_per_s": round(px / (b2_ms / 1e3) / 1e6, 3),
                             "identical": bool(same2)},
            "batched_e2e_mpix_per_s": round(px / (e_ms / 1e3) / 1e6, 3),
            "e2e_h2d_bytes": int(h2d), "e2e_d2h_bytes": int(h2d // 2),
            "identical_to_plain": bool(same), "autotune": tune,
            "stage_frac_of_hbm": round(mand / (b_ms / 1e3) / 1e9 / peak, 5),
            "stage_bytes": int(mand)}


def run_served(args, device, frames):
    """Served requests: Poisson arrivals at 50 / 200 / 800 req/s, sizes
    log-uniform 128^2 .. 6000x4000 (80 % 8-bit), preset 6, through the
    continuous-batching loop (--served-workers contexts, 120 GB HBM budget).
    Requests cycle through a pool of pre-generated images (pinned host
    buffers); latency = completion - scheduled arrival."""
    import copy
    import torch
    pkg = ge._pkg()
    from zenav1_svt_gb300 import serve, synth
    pool = []
    for f in frames:
        src = [torch.from_numpy(p).pin_memory().numpy() for p in f.src]
        pool.append({"f": f, "src": src, "rec0": f.rec, "mi": pkg.pack_geom(f.geom), "slots": []})
    executors = [serve.FilterExecutor(device) for _ in range(args.served_workers)]
    # every worker's arena sized up front for a full batch (48 MP at 10 bits
    # needs < 1 GB), so no arena grows while requests are timed
    srv = serve.Server(executors, hbm_budget_bytes=120 << 30, max_batch=64, max_batch_px=args.served_batch_mpix << 20,
                       reserve_bytes=3 << 29)
    for e in pool:
        r = serve.Request(e["f"], mi=e["mi"])
        e["fp"] = executors[0].footprint(r)

    def take(e):
        for sl in e["slots"]:
            if sl["req"] is None or sl["req"]._done.is_set():
                return sl
        sl = {"rec": [torch.from_numpy(p.copy()).pin_memory().numpy() for p in e["rec0"]], "req": None}
        e["slots"].append(sl)
        return sl

    def request(k):
        e = pool[k % len(pool)]
        sl = take(e)
        for a, b in zip(sl["rec"], e["rec0"]):
            np.copyto(a, b)
        fr = copy.copy(e["f"])
        fr.src, fr.rec = e["src"], sl["rec"]
        r = serve.Request(fr, mi=e["mi"], rid=k)
        r.footprint = e["fp"]
        sl["req"] = r
        return r

    # warm-up: one burst of the whole pool twice (arenas grow to batch size)
    for _ in range(2):
        for k in range(len(pool)):
            srv.submit(request(k))
        srv.drain(timeout=600)
    # pinned recon slots for requests that overlap on one pool image, made
    # here: a page-locked allocation inside a measured window stalls it
    for e in pool:
        while len(e["slots"]) < 4:
            e["slots"].append({"rec": [torch.from_numpy(p.copy()).pin_memory().numpy() for p in e["rec0"]],
                               "req": None})
    out = {}
    import gc
    for rate in args.served_rates:
        arrivals = synth.poisson_arrivals(rate, args.served_seconds, seed=rate)
        reqs = []
        # no collector pauses inside the measured window (a full collection
        # of this process's heap takes tens of ms and holds the interpreter
        # lock the worker threads need between library calls)
        gc.collect()
        gc.disable()
        t0 = time.perf_counter() + 0.02
        for k, off in enumerate(arrivals):
            r = request(k)
            delay = t0 + off - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            reqs.append(srv.submit(r, arrival=t0 + off))
        srv.drain(timeout=600)
        gc.enable()
        s = serve.latency_summary(reqs)
        s["offered_mpix_per_s"] = round(sum(r.luma_px for r in reqs) / args.served_seconds / 1e6, 3)
        s["errors"] = sum(r.error is not None for r in reqs)
        out["%d_req_s" % rate] = s
    srv.close()
    for e in executors:
        e.close()
    return {"workload": ("Poisson arrivals, sizes log-uniform 128^2..6000x4000, 80% 8-bit / 20% 10-bit, "
                         "qp ~ U[18,45], preset 6; requests cycle a pool of {} images").format(len(pool)),
            "seconds_per_rate": args.served_seconds, "workers": args.served_workers,
            "max_batch_mpix": args.served_batch_mpix, "hbm_budget_gb": 120,
            "peak_reserved_gb": round(srv.peak_reserved / 2 ** 30, 3), "arena_grows": srv.arena_grows,
            "rates": out}


def _peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def run_profile(args):
    """Profiler driver (for ncu): device-resident plain path only, no e2e,
    no CPU baseline, no clock sampling. --pw/--ph pick the frame size."""
    import torch
    ge.build()
    pkg = ge._pkg()
    from zenav1_svt_gb300 import abi, synth
    if args.workload == "highres10":
        frames = [synth.workload_10bit_4096()]
    elif args.workload == "batch":
        frames = gen_frames(batch_jobs(args.batch_n))
    else:
        frames = make_workload(args.pw, args.ph)[:args.nframes]  # the timed frames (same seeds)
    ctx = pkg.Context(0)
    if args.stats_tc:
        t = ctx.get_tune()
        ctx.set_tune(t["graphs"], t["stats_tma"], t["apply_group"], 1)
    dev = torch.device("cuda", 0)
    keep, structs, pairs = [], [], []
    for f in frames:
        s = [torch.from_numpy(p.copy()).to(dev) for p in f.src]
        r0 = [torch.from_numpy(p.copy()).to(dev) for p in f.rec]
        r = [x.clone() for x in r0]
        pairs += list(zip(r, r0))
        m = torch.from_numpy(pkg.pack_geom(f.geom).view(np.int32)).to(dev)
        keep += [s, r, r0, m]
        structs.append((abi.make_frame_struct(f, [x.data_ptr() for x in s], [x.data_ptr() for x in r], m.data_ptr(),
                                              on_device=True), abi.Decisions(f.w, f.h, f.true_w, f.true_h),
                        abi.ZfStats()))
    torch.cuda.synchronize()
    n = len(structs)
    arr, darr, sarr = (abi.ZfFrame * n)(), (abi.ZfDecisions * n)(), (abi.ZfStats * n)()
    for i, (s, d, st) in enumerate(structs):
        arr[i], darr[i] = s, d.c
    for _ in range(args.warmup + args.steps):
        for a, b in pairs:  # every pass filters the same pre-deblock recon
            a.copy_(b)
        torch.cuda.synchronize()
        if args.submit_batch:  # the frames as one zf_submit_batch
            ctx.submit_batch_raw(arr, n, darr, sarr)
        else:
            for s, d, st in structs:
                ctx.filter_stage_raw(s, d, st)
        ctx.sync()
    print("profile run done: %d frames %dx%d, %d passes" % (len(frames), args.pw, args.ph, args.warmup + args.steps))
    ctx.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--profile-run", action="store_true", help="plain device path only, for ncu")
    ap.add_argument("--pw", type=int, default=W4K)
    ap.add_argument("--ph", type=int, default=H4K)
    ap.add_argument("--nframes", type=int, default=4)
    ap.add_argument("--stats-tc", action="store_true", help="profile run: tensor-core Wiener statistics")
    ap.add_argument("--workload", default="plain4k", choices=["plain4k", "highres10", "batch"],
                    help="profile run: the frames to run (one zf_filter_stage per frame)")
    ap.add_argument("--submit-batch", action="store_true", help="profile run: the frames as one zf_submit_batch")
    ap.add_argument("--no-batched", action="store_true", help="skip the 256-image batch")
    ap.add_argument("--no-served", action="store_true", help="skip the served request loop")
    ap.add_argument("--batch-n", type=int, default=256)
    ap.add_argument("--served-seconds", type=float, default=4.0, help="arrival window per rate")
    ap.add_argument("--served-rates", type=int, nargs="+", default=[50, 200, 800], help="arrival rates (req/s)")
    ap.add_argument("--served-workers", type=int, default=3, help="worker contexts of the served loop")
    ap.add_argument("--served-batch-mpix", type=int, default=48, help="luma megapixels a served batch holds at most")
    args = ap.parse_args()
    if args.profile_run:
        return run_profile(args)
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
