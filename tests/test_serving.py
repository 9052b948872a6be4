"""Request loop: admission by device footprint, FIFO order, failure isolation,
latency statistics (CPU, fake engine), and on the GPU that every request's
radargram is bitwise the same alone and in a concurrent mix."""
import threading
import time

import numpy as np
import pytest

from helpers import tiny_scene


class FakeEngine:
    """Stands in for the GPU: footprint = bytes_per_trace * ns, run() sleeps
    and returns a radargram that is a pure function of the traces."""

    def __init__(self, bytes_per_trace=1000, delay=0.02, fail_on=None):
        self.bpt = bytes_per_trace
        self.delay = delay
        self.fail_on = fail_on
        self.scenes = {}
        self.lock = threading.Lock()
        self.live = 0
        self.live_bytes = 0
        self.peak_live = 0
        self.peak_bytes = 0
        self.started = []

    def free_memory(self):
        return 10 ** 9

    def add_scene(self, sid, params, facets, targets, prisms):
        self.scenes[sid] = int(params["nr"])

    def adopt_scene(self, sid, scene):
        self.scenes[sid] = int(scene["nr"])

    def remove_scene(self, sid):
        self.scenes.pop(sid)

    def footprint(self, sid, ns, form):
        return self.bpt * ns

    def make_slot(self):
        return {}

    def close_slot(self, slot):
        pass

    def run(self, slot, req):
        fp = self.footprint(req.scene_id, req.traces.shape[0], req.form)
        with self.lock:
            self.started.append(req.id)
            self.live += 1
            self.live_bytes += fp
            self.peak_live = max(self.peak_live, self.live)
            self.peak_bytes = max(self.peak_bytes, self.live_bytes)
        try:
            time.sleep(self.delay)
            if self.fail_on is not None and req.id == self.fail_on:
                raise RuntimeError("planted failure")
            nr = self.scenes[req.scene_id]
            out = np.outer(req.traces[:, 0], np.arange(nr)).astype(np.complex64)
            counts = np.ones((req.traces.shape[0], 2), np.int64)
            return out, counts
        finally:
            with self.lock:
                self.live -= 1
                self.live_bytes -= fp


def _traces(n, base):
    t = np.zeros((n, 9))
    t[:, 0] = base + np.arange(n)
    return t


def test_results_and_stats():
    from europaraypaths_gb300.serving import Server
    eng = FakeEngine()
    srv = Server(engine=eng, workers=3, mem_budget=10 ** 6)
    sid = srv.add_scene({"nr": 8}, None)
    reqs = [srv.submit(sid, _traces(1 + i % 3, 10 * i)) for i in range(12)]
    for i, r in enumerate(reqs):
        out = r.result(timeout=10)
        assert out.shape == (1 + i % 3, 8)
        assert np.array_equal(out[:, 1].real, 10 * i + np.arange(1 + i % 3))
    st = srv.stats()
    assert st["completed"] == 12 and st["p99_ms"] >= st["p50_ms"] > 0
    assert eng.peak_live > 1          # requests overlapped
    srv.close()


def test_admission_respects_budget():
    from europaraypaths_gb300.serving import Server
    eng = FakeEngine(bytes_per_trace=1000, delay=0.03)
    srv = Server(engine=eng, workers=8, mem_budget=2500)
    sid = srv.add_scene({"nr": 4}, None)
    reqs = [srv.submit(sid, _traces(1, i)) for i in range(10)]
    for r in reqs:
        r.result(timeout=10)
    assert eng.peak_bytes <= 2500
    assert eng.peak_live == 2          # 2 x 1000 fit, a third does not
    srv.close()


def test_request_over_budget_refused():
    from europaraypaths_gb300.serving import BudgetError, Server
    srv = Server(engine=FakeEngine(), workers=2, mem_budget=1500)
    sid = srv.add_scene({"nr": 4}, None)
    with pytest.raises(BudgetError):
        srv.submit(sid, _traces(2, 0))
    assert srv.stats()["rejected"] == 1
    srv.close()


def test_fifo_order_single_worker():
    from europaraypaths_gb300.serving import Server
    eng = FakeEngine(delay=0.005)
    srv = Server(engine=eng, workers=1, mem_budget=10 ** 6)
    sid = srv.add_scene({"nr": 4}, None)
    reqs = [srv.submit(sid, _traces(1, i)) for i in range(8)]
    srv.drain(timeout=10)
    assert eng.started == [r.id for r in reqs]
    srv.close()


def test_head_of_line_waits_for_budget():
    # a big request at the head is not overtaken by smaller ones behind it
    from europaraypaths_gb300.serving import Server
    eng = FakeEngine(bytes_per_trace=1000, delay=0.03)
    srv = Server(engine=eng, workers=4, mem_budget=3000)
    sid = srv.add_scene({"nr": 4}, None)
    a = srv.submit(sid, _traces(2, 0))
    big = srv.submit(sid, _traces(3, 10))
    small = srv.submit(sid, _traces(1, 20))
    srv.drain(timeout=10)
    assert eng.started.index(big.id) < eng.started.index(small.id)
    assert a.done() and big.done() and small.done()
    srv.close()


def test_failure_is_isolated():
    from europaraypaths_gb300.serving import Server
    eng = FakeEngine(fail_on=2)
    srv = Server(engine=eng, workers=2, mem_budget=10 ** 6)
    sid = srv.add_scene({"nr": 4}, None)
    reqs = [srv.submit(sid, _traces(1, i)) for i in range(5)]
    for r in reqs:
        if r.id == 2:
            with pytest.raises(RuntimeError, match="planted"):
                r.result(timeout=10)
        else:
            r.result(timeout=10)
    assert srv.stats()["completed"] == 4
    srv.close()


def test_cancel_queued():
    from europaraypaths_gb300.serving import Server
    eng = FakeEngine(delay=0.05)
    srv = Server(engine=eng, workers=1, mem_budget=10 ** 6)
    sid = srv.add_scene({"nr": 4}, None)
    first = srv.submit(sid, _traces(1, 0))
    second = srv.submit(sid, _traces(1, 1))
    time.sleep(0.01)
    assert srv.cancel(second)
    with pytest.raises(RuntimeError, match="cancelled"):
        second.result(timeout=5)
    first.result(timeout=5)
    srv.close()
    assert second.id not in eng.started


def test_adopted_scene_survives_close():
    from europaraypaths_gb300.serving import Server
    eng = FakeEngine(delay=0.001)
    srv = Server(engine=eng, workers=2, mem_budget=10 ** 6)
    sid = srv.adopt_scene({"nr": 6})
    assert srv.submit(sid, _traces(2, 5)).result(timeout=5).shape == (2, 6)
    srv.close(keep_scenes=True)
    assert sid in eng.scenes


@pytest.mark.gpu
def test_gpu_same_alone_and_mixed(built_lib):
    from europaraypaths_gb300 import param_gen, simulator, traces as tr_mod
    from europaraypaths_gb300.serving import Server
    from europaraypaths_gb300 import scenes as scn
    scs = [tiny_scene(nside=40, ntside=4, ns=6),
           tiny_scene(nside=30, ntside=3, ns=5, eps_2=4.0, rx_window_m=scn.rx_window_for_bins(1024, 4e6))]
    srv = Server(workers=3, mem_budget=2 << 30)
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
