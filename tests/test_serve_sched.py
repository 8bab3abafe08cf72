"""Scheduling core of the served request loop (zenav1-svt_gb300/serve.py),
on the CPU with a fake executor: arrival-order admission, the HBM budget,
overlap of batches across workers (continuous batching), release of idle
arenas, and failure of a request that cannot fit at all."""
import threading
import time

import pytest

from zenav1_svt_gb300 import serve


class FakeFrame:
    def __init__(self, w, h):
        self.w = self.true_w = w
        self.h = self.true_h = h


class FakeExecutor:
    """Sleeps in proportion to the batch's pixels; holds an arena the way
    the library does (grows to the batch, never shrinks until trim)."""

    log = []
    lock = threading.Lock()

    def __init__(self, idx, s_per_px=2e-9, bytes_per_px=8):
        self.idx = idx
        self.s_per_px = s_per_px
        self.bpp = bytes_per_px
        self.held = 0
        self.trims = 0

    def footprint(self, req):
        return req.frame.w * req.frame.h * self.bpp

    def run(self, reqs):
        need = sum(self.footprint(r) for r in reqs)
        self.held = max(self.held, serve.arena_after(need))
        with FakeExecutor.lock:
            FakeExecutor.log.append(("start", self.idx, time.perf_counter(), [r.rid for r in reqs]))
        time.sleep(sum(r.luma_px for r in reqs) * self.s_per_px)
        for r in reqs:
            r.decisions = {"rid": r.rid}
        with FakeExecutor.lock:
            FakeExecutor.log.append(("end", self.idx, time.perf_counter(), [r.rid for r in reqs]))

    def device_bytes(self):
        return self.held

    def trim(self):
        self.trims += 1
        self.held = 0


@pytest.fixture(autouse=True)
def _clear_log():
    FakeExecutor.log = []
    yield


def test_all_requests_complete_in_arrival_order():
    ex = [FakeExecutor(0), FakeExecutor(1)]
    srv = serve.Server(ex, hbm_budget_bytes=1 << 40, max_batch=4)
    reqs = [srv.submit(serve.Request(FakeFrame(64 + 8 * i, 64), rid=i)) for i in range(40)]
    srv.drain(timeout=30)
    srv.close()
    for r in reqs:
        r.wait(0)
        assert r.decisions == {"rid": r.rid}
        assert r.latency >= 0 and r.t_start >= r.arrival - 1e-6
    # first come, first served: dispatch order (batch ids) follows arrival order
    assert [r.batch for r in reqs] == sorted(r.batch for r in reqs)
    assert all(len(b) <= 4 for k, _, _, b in FakeExecutor.log)


def test_batches_overlap_across_workers():
    ex = [FakeExecutor(0, s_per_px=5e-7), FakeExecutor(1, s_per_px=5e-7)]
    srv = serve.Server(ex, hbm_budget_bytes=1 << 40, max_batch=8)
    first = srv.submit(serve.Request(FakeFrame(256, 256), rid="a"))  # ~33 ms
    time.sleep(0.005)
    second = srv.submit(serve.Request(FakeFrame(128, 128), rid="b"))  # arrives while "a" runs
    srv.drain(timeout=10)
    srv.close()
    assert first.worker != second.worker
    assert second.t_start < first.t_done  # admitted while the other batch was on the device


def test_budget_bounds_resident_bytes():
    bpp = 8
    one = serve.arena_after(256 * 256 * bpp)
    budget = 2 * one + one // 2  # room for two single-frame arenas, not three
    ex = [FakeExecutor(i, s_per_px=2e-7, bytes_per_px=bpp) for i in range(3)]
    srv = serve.Server(ex, hbm_budget_bytes=budget, max_batch=1)
    reqs = [srv.submit(serve.Request(FakeFrame(256, 256), rid=i)) for i in range(12)]
    srv.drain(timeout=30)
    srv.close()
    assert all(r.error is None for r in reqs)
    assert srv.peak_reserved <= budget
    # never three batches on the device at once
    events = sorted(FakeExecutor.log, key=lambda e: e[2])
    live = peak = 0
    for kind, *_ in events:
        live += 1 if kind == "start" else -1
        peak = max(peak, live)
    assert peak <= 2


def test_idle_arenas_released_for_the_queue_head():
    gib = 1 << 30
    ex = [FakeExecutor(i, s_per_px=1e-6) for i in range(3)]
    ex[0].held, ex[1].held, ex[2].held = int(0.30 * gib), int(0.25 * gib), int(0.25 * gib)
    srv = serve.Server(ex, hbm_budget_bytes=gib)
    long_req = serve.Request(FakeFrame(256, 256), rid="long")  # ~65 ms on the largest arena (worker 0)
    long_req.footprint = 1 << 20
    srv.submit(long_req)
    time.sleep(0.01)
    big = serve.Request(FakeFrame(64, 64), rid="big")
    big.footprint = int(0.45 * gib)  # fits only once the idle arenas of workers 1 and 2 are released
    srv.submit(big)
    srv.drain(timeout=10)
    srv.close()
    assert long_req.worker == 0 and big.worker in (1, 2)
    assert ex[1].trims + ex[2].trims >= 1
    assert big.t_start < long_req.t_done
    assert srv.peak_reserved <= gib


def test_request_over_budget_fails_alone():
    ex = [FakeExecutor(0)]
    srv = serve.Server(ex, hbm_budget_bytes=1 << 20)
    big = srv.submit(serve.Request(FakeFrame(2048, 2048), rid="big"))
    small = srv.submit(serve.Request(FakeFrame(64, 64), rid="small"))
    srv.drain(timeout=10)
    srv.close()
    with pytest.raises(MemoryError):
        big.wait(0)
    assert small.wait(0).decisions == {"rid": "small"}


def test_latency_summary():
    ex = [FakeExecutor(0)]
    srv = serve.Server(ex, hbm_budget_bytes=1 << 40)
    reqs = [srv.submit(serve.Request(FakeFrame(128, 128), rid=i)) for i in range(10)]
    srv.drain(timeout=10)
    srv.close()
    s = serve.latency_summary(reqs)
    assert s["requests"] == 10 and s["p50_ms"] <= s["p99_ms"] <= s["max_ms"]
    assert s["mpix_per_s"] > 0
