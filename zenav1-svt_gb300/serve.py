"""Served form of the filter stage: a continuous-batching request loop.

Encode requests (one frame each: source and pre-deblock recon planes in host
memory plus the packed block geometry) arrive at any time. A dispatcher
admits them in arrival order against an HBM budget and hands whatever is
ready, as one batch, to a free worker. Each worker owns one filter context
-- its own CUDA stream and device arena -- so the batches of different
workers overlap on the GPU while later requests wait for the next free
worker. Inside a batch (zf_submit_batch: one launch per pass for all its
frames) a frame's planes stay on the device from the deblock pass through
CDEF and restoration; its filtered recon and decisions come back when the
batch ends. The recon planes are filtered in place, as the reference's
filter stage does with its recon buffers.

Admission. A request's device footprint is zf_query_sizes' device_bytes. A
batch may start on worker k when the arenas the other workers hold plus
worker k's arena grown to the batch stay within the budget. Requests are
served first come, first served: the head of the queue is never overtaken;
when only idle workers' arenas stand in its way they are released
(zf_trim); a request that cannot fit on an otherwise empty GPU fails with
ZF_ERR_ALLOC.

Latency of a request = completion time - arrival time (host clock).

The scheduling core does not depend on CUDA: workers run an executor object
(FilterExecutor here; the CPU tests use a fake with the same methods).
"""
import collections
import threading
import time

# Arena growth rule of the library (ensure_arena: need + need/8, rounded up
# to 1 MiB): what a context holds after running a batch that needs `need`.
_MIB = 1 << 20


def arena_after(need):
    return ((need + need // 8 + _MIB - 1) // _MIB) * _MIB


class Request:
    """One frame to filter. `frame` is a synth.Frame-like object whose rec
    planes are filtered in place; `mi` the packed geometry (zf_pack_geom)."""

    __slots__ = ("frame", "mi", "rid", "arrival", "footprint", "t_start", "t_done", "decisions", "stats",
                 "error", "batch", "worker", "_done")

    def __init__(self, frame, mi=None, rid=None):
        self.frame = frame
        self.mi = mi
        self.rid = rid
        self.arrival = None
        self.footprint = None
        self.t_start = self.t_done = None
        self.decisions = self.stats = self.error = None
        self.batch = self.worker = None
        self._done = threading.Event()

    @property
    def luma_px(self):
        return self.frame.true_w * self.frame.true_h

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.arrival

    def wait(self, timeout=None):
        if not self._done.wait(timeout):
            raise TimeoutError("request %r not finished" % (self.rid,))
        if self.error is not None:
            raise self.error
        return self


class FilterExecutor:
    """Runs batches on one filter context (one CUDA stream + device arena)."""

    def __init__(self, device=0, hbm_budget_bytes=0):
        from . import Context
        self.ctx = Context(device, hbm_budget_bytes)

    def footprint(self, req):
        from . import pack_geom, query_sizes
        if req.mi is None:
            req.mi = pack_geom(req.frame.geom)
        return int(query_sizes(req.frame, req.mi).device_bytes)

    def run(self, reqs):
        import ctypes as C
        from . import abi, stats_dict
        n = len(reqs)
        arr = (abi.ZfFrame * n)()
        darr = (abi.ZfDecisions * n)()
        st = (abi.ZfStats * n)()
        decs = []
        for i, r in enumerate(reqs):
            f = r.frame
            arr[i] = abi.make_frame_struct(f, f.src, f.rec, r.mi)
            d = abi.Decisions(f.w, f.h, f.true_w, f.true_h)
            decs.append(d)
            darr[i] = d.c
        self.ctx.submit_batch_raw(arr, C.c_int32(n), darr, st)
        for i, r in enumerate(reqs):
            decs[i].c = darr[i]
            r.decisions = decs[i].as_dict()
            r.stats = stats_dict(st[i])

    def device_bytes(self):
        return int(self.ctx.device_bytes())

    def reserve(self, device_bytes):
        self.ctx.reserve(device_bytes)

    def trim(self):
        self.ctx.trim()

    def close(self):
        self.ctx.close()


class _Worker:
    def __init__(self, idx, executor):
        self.idx = idx
        self.ex = executor
        self.busy = False
        self.held = 0          # device bytes the executor holds (after its last batch)
        self.reserved = 0      # bytes accounted while a batch runs
        self.batch = None
        self.wake = threading.Condition()
        self.thread = None


class Server:
    """Continuous-batching loop over `executors` (one worker thread each)."""

    def __init__(self, executors, hbm_budget_bytes=120 << 30, max_batch=64, max_batch_px=32 << 20,
                 reserve_bytes=0, clock=time.perf_counter):
        """reserve_bytes > 0: grow every worker's arena to that size up front
        (growing an arena later releases the old one, which synchronises the
        device and stalls every worker)."""
        if not executors:
            raise ValueError("need at least one executor")
        self.budget = int(hbm_budget_bytes)
        self.max_batch = int(max_batch)
        self.max_batch_px = int(max_batch_px)
        self.clock = clock
        self.workers = [_Worker(i, e) for i, e in enumerate(executors)]
        self.queue = collections.deque()
        self.lock = threading.Condition()
        self.stopping = False
        self.batches = 0
        self.peak_reserved = 0
        self.completed = []
        self.arena_grows = 0
        if reserve_bytes * len(executors) > self.budget:
            raise ValueError("reserved arenas exceed the HBM budget")
        self._disp = threading.Thread(target=self._dispatch_loop, name="zf-dispatch", daemon=True)
        for w in self.workers:
            if reserve_bytes:
                w.ex.reserve(reserve_bytes)
            w.held = w.ex.device_bytes()
            w.thread = threading.Thread(target=self._worker_loop, args=(w,), name="zf-worker%d" % w.idx,
                                        daemon=True)
            w.thread.start()
        self._disp.start()

    # -- client side ----------------------------------------------------------
    def submit(self, req, arrival=None):
        """Queue a request; returns it (wait() blocks until it is done)."""
        req.arrival = self.clock() if arrival is None else arrival
        if req.footprint is None:
            # packs the geometry when needed; zf_query_sizes holds no context
            req.footprint = self.workers[0].ex.footprint(req)
        with self.lock:
            if self.stopping:
                raise RuntimeError("server is stopping")
            self.queue.append(req)
            self.lock.notify_all()
        return req

    def drain(self, timeout=None):
        """Block until every queued and running request is done."""
        t_end = None if timeout is None else time.monotonic() + timeout
        with self.lock:
            while self.queue or any(w.busy for w in self.workers):
                left = None if t_end is None else t_end - time.monotonic()
                if left is not None and left <= 0:
                    raise TimeoutError("server did not drain")
                self.lock.wait(left if left is not None else 0.5)

    def close(self):
        with self.lock:
            self.stopping = True
            self.lock.notify_all()
        self._disp.join()
        for w in self.workers:
            with w.wake:
                w.wake.notify_all()
            w.thread.join()

    # -- accounting -------------------------------------------------------------
    def _resident(self, skip=None):
        return sum(max(w.held, w.reserved) for w in self.workers if w is not skip)

    def _fits(self, w, need):
        return self._resident(skip=w) + max(w.held, arena_after(need)) <= self.budget

    # -- dispatcher -------------------------------------------------------------
    def _dispatch_loop(self):
        while True:
            with self.lock:
                while True:
                    if self.stopping and not self.queue:
                        return
                    free = [w for w in self.workers if not w.busy]
                    if self.queue and free:
                        started = self._try_start(free)
                        if started:
                            continue
                    self.lock.wait(0.05)

    def _try_start(self, free):
        """Start one batch on a free worker (lock held). False when nothing
        could start now."""
        head = self.queue[0]
        # the worker whose arena already holds the most (least growth)
        free.sort(key=lambda w: -w.held)
        w = free[0]
        if not self._fits(w, head.footprint):
            # release idle arenas that block the head of the queue
            for o in self.workers:
                if not o.busy and o.held:
                    o.ex.trim()
                    o.held = o.ex.device_bytes()
            if not self._fits(w, head.footprint):
                if not any(o.busy for o in self.workers):
                    self.queue.popleft()
                    head.error = MemoryError("request %r needs %d device bytes, over the %d-byte budget"
                                             % (head.rid, arena_after(head.footprint), self.budget))
                    head.t_done = self.clock()
                    head._done.set()
                    self.lock.notify_all()
                    return True
                return False
        batch, need, px = [], 0, 0
        while self.queue and len(batch) < self.max_batch:
            r = self.queue[0]
            if batch and (px + r.luma_px > self.max_batch_px or not self._fits(w, need + r.footprint)):
                break
            batch.append(self.queue.popleft())
            need += r.footprint
            px += r.luma_px
        w.busy = True
        w.reserved = arena_after(need)
        w.batch = batch
        self.batches += 1
        bid = self.batches
        for r in batch:
            r.batch, r.worker = bid, w.idx
        self.peak_reserved = max(self.peak_reserved, self._resident())
        with w.wake:
            w.wake.notify_all()
        return True

    # -- workers ----------------------------------------------------------------
    def _worker_loop(self, w):
        while True:
            with w.wake:
                while w.batch is None and not self.stopping:
                    w.wake.wait(0.05)
                batch = w.batch
            if batch is None:
                return
            t0 = self.clock()
            err = None
            try:
                w.ex.run(batch)
            except Exception as e:  # the batch fails as a whole
                err = e
            t1 = self.clock()
            held = w.ex.device_bytes()
            with self.lock:
                self.arena_grows += held > w.held
                for r in batch:
                    r.t_start, r.t_done = t0, t1
                    r.error = err
                    self.completed.append(r)
                    r._done.set()
                w.batch = None
                w.held = held
                w.reserved = 0
                w.busy = False
                self.lock.notify_all()


def latency_summary(reqs):
    """p50 / p99 / max latency (ms) and served MPix/s over finished requests."""
    import numpy as np
    done = [r for r in reqs if r.t_done is not None and r.error is None]
    if not done:
        return {"requests": 0}
    lat = np.array([r.latency for r in done]) * 1e3
    wait = np.array([r.t_start - r.arrival for r in done]) * 1e3
    svc = np.array([r.t_done - r.t_start for r in done]) * 1e3
    t0 = min(r.arrival for r in done)
    t1 = max(r.t_done for r in done)
    px = sum(r.luma_px for r in done)
    return {"requests": len(done), "p50_ms": round(float(np.percentile(lat, 50)), 3),
            "p99_ms": round(float(np.percentile(lat, 99)), 3), "max_ms": round(float(lat.max()), 3),
            "p99_queue_ms": round(float(np.percentile(wait, 99)), 3),
            "p99_batch_ms": round(float(np.percentile(svc, 99)), 3),
            "mpix_per_s": round(px / max(t1 - t0, 1e-9) / 1e6, 3),
            "batches": len({(r.worker, r.batch) for r in done})}
