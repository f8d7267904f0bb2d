"""Host logic of the serving loop: the scratch allocator, the arrival trace and the
continuous-batching scheduler driven by a simulated executor (no GPU)."""
import numpy as np
import pytest

from tqpk.serve import DeviceArena, FirstFit, Request, Scheduler, latency_summary, poisson_trace


def test_first_fit_alloc_release_coalesce():
    ff = FirstFit(1 << 20, align=256)
    offs = [ff.alloc(100_000) for _ in range(10)]
    assert all(o is not None for o in offs)
    assert ff.alloc(100_000) is None                  # 10 x 100,096 B used, 48,576 B left
    for o in offs[::2]:
        ff.release(o)
    assert ff.alloc(200_000) is None                  # freed ranges are not adjacent
    for o in offs[1::2]:
        ff.release(o)
    assert ff.free == [(0, 1 << 20)] and ff.used_bytes == 0
    assert ff.alloc(1 << 20) == 0


def test_first_fit_random_invariants():
    rng = np.random.default_rng(1)
    ff = FirstFit(1 << 24, align=512)
    live = []
    for _ in range(3000):
        if live and rng.random() < 0.45:
            ff.release(live.pop(int(rng.integers(0, len(live)))))
        else:
            o = ff.alloc(int(rng.integers(1, 1 << 19)))
            if o is not None:
                live.append(o)
        spans = sorted([(o, ff.used[o]) for o in live] + ff.free)
        pos = 0
        for off, size in spans:                     # used + free tile [0, capacity) exactly
            assert off == pos and off % 512 == 0
            pos += size
        assert pos == ff.capacity
        for (a, sa), (b, _) in zip(ff.free, ff.free[1:]):
            assert a + sa < b                        # free ranges are coalesced


def test_arena_budget_accounting():
    with pytest.raises(MemoryError):
        DeviceArena(10 << 30, 11 << 30)
    a = DeviceArena(150 << 30, 6 << 30, device=None, slab_cap=1 << 30)
    assert a.capacity == 1 << 30
    p = a.alloc(512 << 20)
    assert p is not None and a.alloc(600 << 20) is None
    a.release(p)
    assert a.alloc(600 << 20) is not None


def test_poisson_trace_is_seeded_and_shaped():
    t1 = poisson_trace(20_000, 2000.0, 60_000_000, seed=5)
    t2 = poisson_trace(20_000, 2000.0, 60_000_000, seed=5)
    assert [(r.shape, r.rows, r.consts, r.arrival) for r in t1] == [(r.shape, r.rows, r.consts, r.arrival) for r in t2]
    arr = np.array([r.arrival for r in t1])
    assert arr[0] == 0 and np.all(np.diff(arr) >= 0)
    assert abs(np.diff(arr).mean() - 1 / 2000) < 0.05 / 2000
    rows = np.array([r.rows for r in t1])
    assert rows.min() >= 1_000_000 and rows.max() <= 60_000_000
    assert abs(np.median(np.log(rows)) - (np.log(1e6) + np.log(6e7)) / 2) < 0.1    # log-uniform
    shapes = [r.shape for r in t1]
    for s in ("filter_groupby", "join", "star"):
        assert abs(shapes.count(s) / len(shapes) - 1 / 3) < 0.02


class FakeClock:
    def __init__(self, tick=1e-5):
        self.t, self.tick = 0.0, tick

    def __call__(self):
        self.t += self.tick
        return self.t


class SimExecutor:
    """Each request takes `service(req)` seconds of simulated time once launched."""

    def __init__(self, clock, service, scratch):
        self.clock, self.service, self.scratch = clock, service, scratch
        self.launched, self.running, self.max_running = [], 0, 0

    def scratch_bytes(self, req):
        return self.scratch(req)

    def launch(self, req, slot, ptr):
        self.launched.append((req.rid, slot, ptr))
        self.running += 1
        self.max_running = max(self.max_running, self.running)
        return [req, self.clock.t + self.service(req), False]

    def done(self, h):
        return self.clock.t >= h[1]

    def finish(self, h):
        assert not h[2]
        h[2] = True
        self.running -= 1
        return ("result", h[0].rid)


def _trace(n, gap):
    return [Request(i, "join", 1000, (1,), i * gap) for i in range(n)]


def test_scheduler_one_at_a_time_is_fifo_and_serial():
    clk = FakeClock()
    ex = SimExecutor(clk, lambda r: 1e-3, lambda r: 1 << 20)
    done = Scheduler(ex, DeviceArena(1 << 30, 0), slots=1, clock=clk).run(_trace(20, 1e-4))
    assert [c.req.rid for c in done] == list(range(20))
    assert ex.max_running == 1
    for a, b in zip(done, done[1:]):
        assert b.start >= a.end - 1e-4                  # the next starts only after the previous ended
    assert all(c.result == ("result", c.req.rid) for c in done)


def test_scheduler_overlaps_requests_that_arrive_while_others_run():
    clk = FakeClock()
    ex = SimExecutor(clk, lambda r: 2e-3, lambda r: 1 << 20)
    sched = Scheduler(ex, DeviceArena(1 << 30, 0), slots=4, clock=clk)
    done = sched.run(_trace(40, 2e-4))
    assert sorted(c.req.rid for c in done) == list(range(40))
    assert ex.max_running == 4 and sched.max_inflight == 4
    by = {c.req.rid: c for c in done}
    assert by[1].start < by[0].end                     # admitted while request 0 was still running
    serial = Scheduler(SimExecutor(clk, lambda r: 2e-3, lambda r: 1 << 20), DeviceArena(1 << 30, 0), slots=1,
                       clock=clk).run(_trace(40, 2e-4))
    assert latency_summary(done)["p99_ms"] < latency_summary(serial)["p99_ms"] / 2


def test_scheduler_respects_the_memory_budget():
    clk = FakeClock()
    ex = SimExecutor(clk, lambda r: 1e-3, lambda r: 400 << 20)
    arena = DeviceArena(1 << 30, 0)                    # room for two 400 MB requests at a time
    done = Scheduler(ex, arena, slots=8, clock=clk).run(_trace(12, 0.0))
    assert len(done) == 12 and ex.max_running == 2
    assert arena.ff.used_bytes == 0                    # every scratch range came back


def test_scheduler_rejects_a_request_larger_than_the_arena():
    clk = FakeClock()
    ex = SimExecutor(clk, lambda r: 1e-3, lambda r: 2 << 30)
    with pytest.raises(MemoryError):
        Scheduler(ex, DeviceArena(1 << 30, 0), slots=2, clock=clk).run(_trace(1, 0.0))
