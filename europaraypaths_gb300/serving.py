"""Resident request loop: many flyby simulations served concurrently on one GPU.

A thin wrapper over the native server of libraypath (rp_server_create,
rp_submit, rp_poll, rp_cancel, rp_server_stats):

* scenes are registered once and stay resident on the device; requests name
  a scene and carry a trace table;
* admission: a request's device footprint (rp_query_footprint plus its trace
  table and output) must fit the memory budget next to everything running;
  requests wait in FIFO order; a request larger than the whole budget is
  refused (``BudgetError``);
* continuous batching: worker threads, each with its own CUDA stream and
  workspace, take the queue head plus the following fast-form requests that
  fit and run them as one multi-scene call, so requests arriving while others
  run are admitted as workers and memory free up and overlap on the device.
  A result does not depend on what it was batched or overlapped with;
* ``stats()`` reports p50/p99 latency (submit to result), queue wait and
  aggregate pairs/s.

``executor=`` replaces the GPU by a Python object with ``run(scene, traces,
form) -> (out, counts)`` and ``footprint(scene, ns, form) -> bytes``: the
same native scheduler then runs without CUDA (used by the CPU tests).
"""
import ctypes

import numpy as np

from . import _abi

RP_PENDING = 1
RP_ERR_BUDGET = -7
RP_ERR_CANCELLED = -10
STAT_KEYS = ("completed", "failed", "rejected", "cancelled", "p50_ms", "p99_ms", "mean_ms", "mean_wait_ms",
             "pairs", "pairs_per_s", "worker_calls", "max_batch_seen", "in_flight_bytes", "shed", "steps",
             "max_active_seen", "max_calls_running", "p90_ms")
RP_ERR_TIMEOUT = -8


class BudgetError(RuntimeError):
    """The request can never fit in the admission budget."""


class CancelledError(RuntimeError):
    """The request was cancelled before it started."""


class ShedError(RuntimeError):
    """The request waited in the queue longer than the server's bound."""


class Request:
    def __init__(self, server, ticket, out, counts, traces):
        self.server = server
        self.id = ticket
        self.out = out
        self.counts = counts
        self.traces = traces          # kept alive until the request is finished
        self.status = None
        self.error_text = ""

    def _finish(self, rc):
        self.status = rc
        self.traces = None
        if rc != 0:
            self.error_text = _abi.last_error()

    def done(self):
        if self.status is None:
            rc = _abi.lib().rp_poll(self.server._h, self.id, 0)
            if rc != RP_PENDING:
                self._finish(rc)
        return self.status is not None

    def result(self, timeout=None):
        """The complex64 (ns, nr) radargram; raises on failure or timeout."""
        if self.status is None:
            ms = -1 if timeout is None else max(1, int(timeout * 1000))
            rc = _abi.lib().rp_poll(self.server._h, self.id, ms)
            if rc == RP_PENDING:
                raise TimeoutError(f"request {self.id} not finished after {timeout} s")
            self._finish(rc)
        if self.status == RP_ERR_CANCELLED:
            raise CancelledError(f"request {self.id} cancelled")
        if self.status == RP_ERR_TIMEOUT:
            raise ShedError(f"request {self.id} shed: {self.error_text}")
        if self.status != 0:
            raise RuntimeError(f"request {self.id} failed ({_abi.ERRORS.get(self.status, self.status)}): "
                               f"{self.error_text}")
        return self.out


_RUN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                        ctypes.c_int64, ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64))
_FOOT = ctypes.CFUNCTYPE(ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int)
_BINS = ctypes.CFUNCTYPE(ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p)


class _Executor(ctypes.Structure):
    _fields_ = [("run", _RUN), ("footprint", _FOOT), ("user", ctypes.c_void_p), ("bins", _BINS)]


class Server:
    """Concurrent, memory-budgeted request loop over resident scenes."""

    FORMS = {"plain": 0, "fast": 1}

    def __init__(self, workers=3, mem_budget=None, device=0, max_batch=8, executor=None, step_traces=0,
                 max_active=0, max_wait=None):
        """``step_traces`` > 0 cuts requests into steps of that many traces,
        scheduled round robin across the active requests (continuous batching
        at step granularity); ``max_active`` bounds the requests active at
        once (0: the memory budget alone); ``max_wait`` (seconds) sheds
        queued requests that waited longer (``ShedError``)."""
        self.device = device
        self.scenes = {}          # sid -> (handle, nr, owned Scene or None)
        self._next_sid = 1
        self._ex = None
        exp = None
        if executor is not None:
            def run(_user, scene, traces, ns, form, out, counts):
                try:
                    tr = np.ctypeslib.as_array(traces, shape=(ns, 9)).copy()
                    o, c = executor.run(int(scene or 0), tr, form)
                    o = np.ascontiguousarray(o, dtype=np.complex64)
                    ctypes.memmove(out, o.ctypes.data, o.nbytes)
                    c = np.ascontiguousarray(c, dtype=np.int64).reshape(-1)
                    ctypes.memmove(counts, c.ctypes.data, c.nbytes)
                    return 0
                except Exception:
                    return -9

            def foot(_user, scene, ns, form):
                return int(executor.footprint(int(scene or 0), ns, form))

            def bins(_user, scene):
                return int(self.scenes[int(scene or 0)][1])

            self._ex = _Executor(_RUN(run), _FOOT(foot), None, _BINS(bins))
            exp = ctypes.byref(self._ex)
        self._h = ctypes.c_void_p()
        _abi.check("rp_server_create", _abi.lib().rp_server_create(
            int(device), int(workers), int(mem_budget or 0), int(max_batch), exp, ctypes.byref(self._h)))
        if step_traces or max_active or max_wait:
            _abi.check("rp_server_configure", _abi.lib().rp_server_configure(
                self._h, int(step_traces), int(max_active), int(round(1000 * (max_wait or 0)))))

    # ---------------------------------------------------------------- scenes
    def add_scene(self, params, facets=None, targets=None, prisms=None):
        """Create a resident scene owned by the server (an executor-backed
        server takes any mapping with an ``nr`` entry instead)."""
        if self._ex is not None:
            return self._register(None, int(params["nr"]), None)
        from .simulator import Scene
        sc = Scene(params, facets, targets, prisms=prisms, device=self.device)
        return self._register(sc.handle, sc.nr, sc)

    def adopt_scene(self, scene):
        """Serve an existing resident Scene (the caller keeps ownership)."""
        if self._ex is not None:
            return self._register(None, int(scene["nr"]), None)
        return self._register(scene.handle, scene.nr, None)

    def _register(self, handle, nr, owned):
        sid = self._next_sid
        self._next_sid += 1
        # an executor-backed server passes the scene id as the scene handle
        self.scenes[sid] = (handle if handle is not None else sid, nr, owned)
        return sid

    def remove_scene(self, sid):
        _h, _nr, owned = self.scenes.pop(sid)
        if owned is not None:
            owned.close()

    # -------------------------------------------------------------- requests
    def submit(self, sid, traces, form="fast"):
        handle, nr, _ = self.scenes[sid]
        tr = np.ascontiguousarray(traces, dtype=np.float64).reshape(-1, 9)
        ns = tr.shape[0]
        out = np.zeros((ns, nr), np.complex64)
        counts = np.zeros((ns, 2), np.int64)
        t = ctypes.c_int64()
        rc = _abi.lib().rp_submit(self._h, ctypes.c_void_p(handle), tr.ctypes.data, ns, self.FORMS[form],
                                  out.ctypes.data, counts.ctypes.data, ctypes.byref(t))
        if rc == RP_ERR_BUDGET:
            raise BudgetError(_abi.last_error())
        _abi.check("rp_submit", rc)
        return Request(self, t.value, out, counts, tr)

    def cancel(self, req):
        """Cancel a request that has not started; returns whether it was."""
        return _abi.lib().rp_cancel(self._h, req.id) == 0

    # ----------------------------------------------------------------- stats
    def stats(self):
        buf = (ctypes.c_double * len(STAT_KEYS))()
        _abi.check("rp_server_stats", _abi.lib().rp_server_stats(self._h, buf, len(STAT_KEYS)))
        d = dict(zip(STAT_KEYS, list(buf)))
        for k in ("completed", "failed", "rejected", "cancelled", "worker_calls", "max_batch_seen",
                  "in_flight_bytes", "shed", "steps", "max_active_seen", "max_calls_running"):
            d[k] = int(d[k])
        return d

    def drain(self, timeout=None):
        ms = -1 if timeout is None else int(timeout * 1000)
        rc = _abi.lib().rp_server_drain(self._h, ms)
        if rc == -8:
            raise TimeoutError("drain timed out")
        _abi.check("rp_server_drain", rc)

    def close(self, keep_scenes=False):
        """Drain, stop the workers and (unless keep_scenes) free owned scenes."""
        if self._h and self._h.value:
            _abi.lib().rp_server_destroy(self._h)
            self._h = ctypes.c_void_p()
        if not keep_scenes:
            for sid in list(self.scenes):
                self.remove_scene(sid)

    def __del__(self):
        try:
            self.close(keep_scenes=True)
        except Exception:
            pass
