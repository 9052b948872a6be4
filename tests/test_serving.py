"""Request loop: admission by device footprint, FIFO order, failure isolation,
latency statistics (CPU, fake engine), and on the GPU that every request's
radargram is bitwise the same alone and in a concurrent mix (split facet
parts off, so that a lone small call sums its parts as a larger one does)."""
import threading
import time

import numpy as np
import pytest

from helpers import tiny_scene


class FakeEngine:
    """Stands in for the GPU behind the native scheduler: footprint =
    bytes_per_trace * ns; run() sleeps and returns a radargram that is a pure
    function of the traces."""

    def __init__(self, bytes_per_trace=1000, delay=0.02, fail_on_base=None):
        self.bpt = bytes_per_trace
        self.delay = delay
        self.fail_on_base = fail_on_base
        self.nrs = {}
        self.lock = threading.Lock()
        self.live = 0
        self.live_bytes = 0
        self.peak_live = 0
        self.peak_bytes = 0
        self.started = []

    def footprint(self, sid, ns, form):
        return self.bpt * ns

    def run(self, sid, traces, form):
        fp = self.footprint(sid, traces.shape[0], form)
        with self.lock:
            self.started.append(float(traces[0, 0]))
            self.live += 1
            self.live_bytes += fp
            self.peak_live = max(self.peak_live, self.live)
            self.peak_bytes = max(self.peak_bytes, self.live_bytes)
        try:
            time.sleep(self.delay)
            if self.fail_on_base is not None and traces[0, 0] == self.fail_on_base:
                raise RuntimeError("planted failure")
            nr = self.nrs[sid]
            out = np.outer(traces[:, 0], np.arange(nr)).astype(np.complex64)
            counts = np.ones((traces.shape[0], 2), np.int64)
            return out, counts
        finally:
            with self.lock:
                self.live -= 1
                self.live_bytes -= fp


def _server(eng, nr=4, **kw):
    from europaraypaths_gb300.serving import Server
    srv = Server(executor=eng, **kw)
    sid = srv.add_scene({"nr": nr})
    eng.nrs[sid] = nr
    return srv, sid


def _traces(n, base):
    t = np.zeros((n, 9))
    t[:, 0] = base + np.arange(n)
    return t


def test_results_and_stats():
    eng = FakeEngine()
    srv, sid = _server(eng, nr=8, workers=3, mem_budget=10 ** 6, max_batch=1)
    reqs = [srv.submit(sid, _traces(1 + i % 3, 10 * i)) for i in range(12)]
    for i, r in enumerate(reqs):
        out = r.result(timeout=10)
        assert out.shape == (1 + i % 3, 8)
        assert np.array_equal(out[:, 1].real, 10 * i + np.arange(1 + i % 3))
    st = srv.stats()
    assert st["completed"] == 12 and st["p99_ms"] >= st["p50_ms"] > 0
    assert st["pairs"] == sum(3 * (1 + i % 3) for i in range(12))
    assert eng.peak_live > 1          # requests overlapped
    srv.close()


def test_admission_respects_budget():
    eng = FakeEngine(bytes_per_trace=1000, delay=0.03)
    srv, sid = _server(eng, workers=8, mem_budget=2500, max_batch=1)
    reqs = [srv.submit(sid, _traces(1, i)) for i in range(10)]
    for r in reqs:
        r.result(timeout=10)
    assert eng.peak_bytes <= 2500
    assert eng.peak_live == 2          # 2 x 1000 fit, a third does not
    srv.close()


def test_request_over_budget_refused():
    from europaraypaths_gb300.serving import BudgetError
    srv, sid = _server(FakeEngine(), workers=2, mem_budget=1500)
    with pytest.raises(BudgetError):
        srv.submit(sid, _traces(2, 0))
    assert srv.stats()["rejected"] == 1
    srv.close()


def test_fifo_order_single_worker():
    eng = FakeEngine(delay=0.005)
    srv, sid = _server(eng, workers=1, mem_budget=10 ** 6, max_batch=1)
    for i in range(8):
        srv.submit(sid, _traces(1, i))
    srv.drain(timeout=10)
    assert eng.started == [float(i) for i in range(8)]
    srv.close()


def test_head_of_line_waits_for_budget():
    # a big request at the head is not overtaken by smaller ones behind it
    eng = FakeEngine(bytes_per_trace=1000, delay=0.03)
    srv, sid = _server(eng, workers=4, mem_budget=3000, max_batch=1)
    a = srv.submit(sid, _traces(2, 0))
    big = srv.submit(sid, _traces(3, 10))
    small = srv.submit(sid, _traces(1, 20))
    srv.drain(timeout=10)
    assert eng.started.index(10.0) < eng.started.index(20.0)
    assert a.done() and big.done() and small.done()
    srv.close()


def test_failure_is_isolated():
    eng = FakeEngine(fail_on_base=2.0)
    srv, sid = _server(eng, workers=2, mem_budget=10 ** 6, max_batch=1)
    reqs = [srv.submit(sid, _traces(1, i)) for i in range(5)]
    for i, r in enumerate(reqs):
        if i == 2:
            with pytest.raises(RuntimeError, match="failed"):
                r.result(timeout=10)
        else:
            r.result(timeout=10)
    st = srv.stats()
    assert st["completed"] == 4 and st["failed"] == 1
    srv.close()


def test_cancel_queued():
    from europaraypaths_gb300.serving import CancelledError
    eng = FakeEngine(delay=0.2)
    srv, sid = _server(eng, workers=1, mem_budget=10 ** 6, max_batch=1)
    first = srv.submit(sid, _traces(1, 0))
    time.sleep(0.05)
    second = srv.submit(sid, _traces(1, 1))
    assert srv.cancel(second)
    with pytest.raises(CancelledError):
        second.result(timeout=5)
    first.result(timeout=5)
    srv.close()
    assert 1.0 not in eng.started
    assert srv.stats is not None


def test_continuous_batching_takes_queued_requests():
    # one worker busy with a slow request; requests queued meanwhile are
    # taken together by its next call
    eng = FakeEngine(delay=0.1)
    srv, sid = _server(eng, workers=1, mem_budget=10 ** 6, max_batch=8)
    reqs = [srv.submit(sid, _traces(1, 0))]
    time.sleep(0.03)
    reqs += [srv.submit(sid, _traces(2, 10 * k)) for k in range(1, 6)]
    for k, r in enumerate(reqs):
        assert r.result(timeout=10)[0, 1].real == 10 * k
    st = srv.stats()
    assert st["worker_calls"] == 2 and st["max_batch_seen"] == 5
    srv.close()


def test_adopted_scene_survives_close():
    from europaraypaths_gb300.serving import Server
    eng = FakeEngine(delay=0.001)
    srv = Server(executor=eng, workers=2, mem_budget=10 ** 6)
    sid = srv.adopt_scene({"nr": 6})
    eng.nrs[sid] = 6
    assert srv.submit(sid, _traces(2, 5)).result(timeout=5).shape == (2, 6)
    srv.close(keep_scenes=True)
    assert sid in srv.scenes


def test_steps_round_robin_results():
    # requests cut into 2-trace steps: every step lands at its offset, and
    # one call takes steps of several requests
    eng = FakeEngine(delay=0.01)
    srv, sid = _server(eng, nr=5, workers=1, mem_budget=10 ** 6, max_batch=4, step_traces=2)
    a = srv.submit(sid, _traces(7, 100))
    b = srv.submit(sid, _traces(3, 200))
    c = srv.submit(sid, _traces(1, 300))
    for r, n, base in ((a, 7, 100), (b, 3, 200), (c, 1, 300)):
        out = r.result(timeout=10)
        assert out.shape == (n, 5)
        assert np.array_equal(out[:, 1].real, base + np.arange(n))
        assert np.array_equal(r.counts, np.ones((n, 2)))
    st = srv.stats()
    assert st["steps"] == 4 + 2 + 1 and st["max_batch_seen"] >= 2 and st["completed"] == 3
    srv.close()


def test_short_request_not_blocked_by_long_one():
    # step-level scheduling: a 1-trace request that arrives while a 30-trace
    # request runs finishes long before it
    eng = FakeEngine(delay=0.02)
    srv, sid = _server(eng, workers=1, mem_budget=10 ** 6, max_batch=2, step_traces=1)
    t0 = time.perf_counter()
    big = srv.submit(sid, _traces(30, 0))
    time.sleep(0.05)
    small = srv.submit(sid, _traces(1, 1000))
    small.result(timeout=10)
    t_small = time.perf_counter() - t0
    big.result(timeout=10)
    t_big = time.perf_counter() - t0
    assert t_small < 0.5 * t_big
    srv.close()


def test_active_limit_and_queue_wait_bound():
    from europaraypaths_gb300.serving import ShedError
    eng = FakeEngine(delay=0.05)
    srv, sid = _server(eng, workers=2, mem_budget=10 ** 6, max_batch=4, step_traces=1, max_active=1,
                       max_wait=0.15)
    first = srv.submit(sid, _traces(8, 0))          # ~0.4 s of steps
    time.sleep(0.02)
    late = [srv.submit(sid, _traces(1, 100 + k)) for k in range(3)]
    assert first.result(timeout=10).shape == (8, 4)
    for r in late:
        with pytest.raises(ShedError):
            r.result(timeout=10)
    st = srv.stats()
    assert st["shed"] == 3 and st["max_active_seen"] == 1 and st["completed"] == 1
    srv.close()


def test_step_failure_drops_the_rest_of_its_request_only():
    eng = FakeEngine(delay=0.005, fail_on_base=2.0)
    srv, sid = _server(eng, workers=2, mem_budget=10 ** 6, max_batch=4, step_traces=2)
    bad = srv.submit(sid, _traces(6, 0))           # steps at 0, 2 (fails), 4
    good = srv.submit(sid, _traces(4, 50))
    with pytest.raises(RuntimeError, match="failed"):
        bad.result(timeout=10)
    assert np.array_equal(good.result(timeout=10)[:, 1].real, 50 + np.arange(4))
    st = srv.stats()
    assert st["failed"] == 1 and st["completed"] == 1
    srv.close()


def test_configure_after_submit_refused():
    from europaraypaths_gb300 import _abi
    eng = FakeEngine(delay=0.2)
    srv, sid = _server(eng, workers=1, mem_budget=10 ** 6)
    srv.submit(sid, _traces(1, 0))
    assert _abi.lib().rp_server_configure(srv._h, 2, 0, 0) == -1
    srv.close()


@pytest.mark.gpu
@pytest.mark.parametrize("step", [0, 2])
def test_gpu_same_alone_and_mixed(built_lib, step, no_split_parts):
    from europaraypaths_gb300 import param_gen, simulator, traces as tr_mod
    from europaraypaths_gb300.serving import Server
    from europaraypaths_gb300 import scenes as scn
    scs = [tiny_scene(nside=40, ntside=4, ns=6),
           tiny_scene(nside=30, ntside=3, ns=5, eps_2=4.0, rx_window_m=scn.rx_window_for_bins(1024, 4e6))]
    srv = Server(workers=3, mem_budget=2 << 30, step_traces=step)
    sids = [srv.add_scene(sc["params"], sc["facets"], sc["targets"]) for sc in scs]
    jobs = []
    for k in range(12):
        which = k % 2
        p = param_gen.to_rp_params(scs[which]["params"])
        tr = tr_mod.linear_track(p)
        lo = k % 3
        jobs.append((which, lo, tr[lo:lo + 1 + k % 4]))
    reqs = [srv.submit(sids[w], tr) for w, _lo, tr in jobs]
    mixed = [r.result(timeout=120) for r in reqs]
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(jobs) and st["p99_ms"] > 0
    scenes = [simulator.Scene(sc["params"], sc["facets"], sc["targets"]) for sc in scs]
    try:
        full = [s.simulate() for s in scenes]
        for (w, lo, tr), got in zip(jobs, mixed):
            alone = scenes[w].simulate(tr)
            assert np.array_equal(alone.view(np.uint32), got.view(np.uint32))
            # a trace's radargram does not depend on the other traces of its request
            assert np.array_equal(full[w][lo:lo + tr.shape[0]].view(np.uint32), got.view(np.uint32))
    finally:
        for s in scenes:
            s.close()
