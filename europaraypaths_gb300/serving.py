"""Resident request loop: many flyby simulations served concurrently on one GPU.

* Scenes are registered once and stay resident on the device (facet store,
  targets, spectral tables); requests name a scene and carry a trace table.
* Admission: a request's device footprint (scratch from rp_query_footprint,
  plus its trace table and output) must fit in the memory budget together
  with every request already running; requests wait in FIFO order until a
  worker slot and enough budget are free.  A request larger than the whole
  budget is refused (``BudgetError``).
* Continuous batching: each worker slot owns a CUDA stream and an
  ``rp_workspace``; admitted requests run at once on their own streams, so
  work of requests that arrive while others are on the GPU overlaps on the
  device.  Results do not depend on what else is running: every kernel's sum
  order is fixed by the request's own data.
* ``stats()`` reports p50/p99 latency (submit to result) and aggregate
  pairs/s.

The engine is pluggable: ``GpuEngine`` drives libraraypath; tests of the
scheduling logic use a fake engine on the CPU.
"""
import collections
import ctypes
import threading
import time

import numpy as np

from . import _abi, opcount


class BudgetError(RuntimeError):
    """The request can never fit in the admission budget."""


class Request:
    def __init__(self, rid, scene_id, traces, form):
        self.id = rid
        self.scene_id = scene_id
        self.traces = np.ascontiguousarray(traces, dtype=np.float64).reshape(-1, 9)
        self.form = form
        self.footprint = 0
        self.t_submit = time.perf_counter()
        self.t_start = None
        self.t_end = None
        self.out = None
        self.counts = None
        self.error = None
        self.cancelled = False
        self._done = threading.Event()

    def done(self):
        return self._done.is_set()

    def result(self, timeout=None):
        if not self._done.wait(timeout):
            raise TimeoutError(f"request {self.id} not finished after {timeout} s")
        if self.error is not None:
            raise self.error
        return self.out

    @property
    def latency(self):
        return None if self.t_end is None else self.t_end - self.t_submit


class GpuEngine:
    """libraypath engine: resident scenes, one workspace + stream per slot."""

    def __init__(self, device=0):
        import torch
        self.torch = torch
        self.device = device
        torch.cuda.set_device(device)
        self.scenes = {}

    def free_memory(self):
        free, _total = self.torch.cuda.mem_get_info(self.device)
        return free

    def add_scene(self, sid, params, facets, targets, prisms):
        from .simulator import Scene
        self.scenes[sid] = Scene(params, facets, targets, prisms=prisms, device=self.device)
        return self.scenes[sid].footprint()

    def adopt_scene(self, sid, scene):
        self.scenes[sid] = scene

    def remove_scene(self, sid):
        self.scenes.pop(sid).close()

    def footprint(self, sid, ns, form):
        sc = self.scenes[sid]
        return sc.scratch_bytes(ns, form) + ns * (72 + 8 * sc.nr)

    def nr(self, sid):
        return self.scenes[sid].nr

    def make_slot(self):
        ws = ctypes.c_void_p()
        _abi.check("rp_workspace_create", _abi.lib().rp_workspace_create(self.device, ctypes.byref(ws)))
        return {"ws": ws, "stream": self.torch.cuda.Stream(device=self.device)}

    def close_slot(self, slot):
        _abi.lib().rp_workspace_destroy(slot["ws"])

    def run(self, slot, req):
        torch = self.torch
        torch.cuda.set_device(self.device)
        sc = self.scenes[req.scene_id]
        ns = req.traces.shape[0]
        counts = np.zeros((ns, 2), np.int64)
        with torch.cuda.stream(slot["stream"]):
            d_tr = torch.from_numpy(req.traces).to(f"cuda:{self.device}", non_blocking=True)
            d_out = torch.empty((ns, sc.nr), dtype=torch.complex64, device=f"cuda:{self.device}")
            from .simulator import FORMS
            rc = _abi.lib().rp_simulate_ws(ctypes.c_void_p(sc.handle), slot["ws"],
                                           ctypes.c_void_p(d_tr.data_ptr()), ns, FORMS[req.form],
                                           ctypes.c_void_p(d_out.data_ptr()), counts.ctypes.data,
                                           ctypes.c_void_p(slot["stream"].cuda_stream))
            _abi.check("rp_simulate_ws", rc)
            out = d_out.cpu()
        return out.numpy(), counts


class Server:
    """Concurrent, memory-budgeted request loop over resident scenes."""

    def __init__(self, engine=None, workers=3, mem_budget=None, device=0):
        self.engine = engine if engine is not None else GpuEngine(device)
        if mem_budget is None:
            mem_budget = int(0.6 * self.engine.free_memory())
        self.budget = int(mem_budget)
        self.in_flight = 0
        self.queue = collections.deque()
        self.cv = threading.Condition()
        self.closed = False
        self.next_id = 0
        self.next_scene = 0
        self.completed = []
        self.rejected = 0
        self.slots = [self.engine.make_slot() for _ in range(workers)]
        self.free_slots = list(range(workers))
        self.threads = []
        self.dispatcher = threading.Thread(target=self._dispatch, daemon=True)
        self.dispatcher.start()

    # ---------------------------------------------------------------- scenes
    def add_scene(self, params, facets, targets=None, prisms=None):
        with self.cv:
            sid = self.next_scene
            self.next_scene += 1
        self.engine.add_scene(sid, params, facets, targets, prisms)
        return sid

    def adopt_scene(self, scene):
        """Serve an existing resident Scene (the caller keeps ownership)."""
        with self.cv:
            sid = self.next_scene
            self.next_scene += 1
        self.engine.adopt_scene(sid, scene)
        return sid

    def remove_scene(self, sid):
        self.engine.remove_scene(sid)

    # -------------------------------------------------------------- requests
    def submit(self, scene_id, traces, form="fast"):
        with self.cv:
            if self.closed:
                raise RuntimeError("server is closed")
            req = Request(self.next_id, scene_id, traces, form)
            self.next_id += 1
        req.footprint = self.engine.footprint(scene_id, req.traces.shape[0], form)
        if req.footprint > self.budget:
            self.rejected += 1
            raise BudgetError(f"request {req.id} needs {req.footprint} bytes, budget is {self.budget}")
        with self.cv:
            self.queue.append(req)
            self.cv.notify_all()
        return req

    def cancel(self, req):
        """Cancel a request that has not started; returns whether it was."""
        with self.cv:
            if req in self.queue:
                self.queue.remove(req)
                req.cancelled = True
                req.error = RuntimeError(f"request {req.id} cancelled")
                req.t_end = time.perf_counter()
                req._done.set()
                self.cv.notify_all()
                return True
        return False

    def _dispatch(self):
        while True:
            with self.cv:
                while not self.closed and not (
                        self.queue and self.free_slots and
                        self.in_flight + self.queue[0].footprint <= self.budget):
                    self.cv.wait(0.05)
                if self.closed and not self.queue:
                    return
                if not (self.queue and self.free_slots and
                        self.in_flight + self.queue[0].footprint <= self.budget):
                    continue
                req = self.queue.popleft()          # FIFO: the head waits for budget
                slot_id = self.free_slots.pop()
                self.in_flight += req.footprint
            t = threading.Thread(target=self._work, args=(slot_id, req), daemon=True)
            t.start()
            self.threads.append(t)

    def _work(self, slot_id, req):
        req.t_start = time.perf_counter()
        try:
            req.out, req.counts = self.engine.run(self.slots[slot_id], req)
        except Exception as e:   # a failing request must not take the server down
            req.error = e
        req.t_end = time.perf_counter()
        with self.cv:
            self.in_flight -= req.footprint
            self.free_slots.append(slot_id)
            if req.error is None:
                self.completed.append(req)
            self.cv.notify_all()
        req._done.set()

    # ----------------------------------------------------------------- stats
    def stats(self):
        with self.cv:
            done = list(self.completed)
        if not done:
            return {"completed": 0, "rejected": self.rejected}
        lat = np.array([r.latency for r in done]) * 1e3
        t0 = min(r.t_submit for r in done)
        t1 = max(r.t_end for r in done)
        pairs = sum(opcount.pairs(r.counts) for r in done if r.counts is not None)
        return {"completed": len(done), "rejected": self.rejected,
                "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "mean_ms": float(lat.mean()), "pairs": int(pairs),
                "pairs_per_s": pairs / (t1 - t0) if t1 > t0 else None, "wall_s": t1 - t0}

    def drain(self, timeout=None):
        t_end = None if timeout is None else time.perf_counter() + timeout
        with self.cv:
            while self.queue or self.in_flight > 0 or len(self.free_slots) < len(self.slots):
                left = None if t_end is None else t_end - time.perf_counter()
                if left is not None and left <= 0:
                    raise TimeoutError("drain timed out")
                self.cv.wait(0.05 if left is None else min(0.05, left))

    def close(self, keep_scenes=False):
        """Drain, stop the dispatcher and free the slots (and, unless
        keep_scenes, the scenes)."""
        self.drain()
        with self.cv:
            self.closed = True
            self.cv.notify_all()
        self.dispatcher.join(timeout=5)
        for s in self.slots:
            self.engine.close_slot(s)
        if not keep_scenes:
            for sid in list(getattr(self.engine, "scenes", {}).keys()):
                self.engine.remove_scene(sid)
