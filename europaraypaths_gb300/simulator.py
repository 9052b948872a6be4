"""Resident-scene simulation API over the C ABI (libraypath.so).

``Scene`` owns a device-resident facet store (created once, reused by every
call), and ``Scene.simulate`` runs any number of traces in one call -- the
trace loop of ``src/CUDA/sim.cu:615-1008`` without its per-trace files.
``simulate(params, facets, targets)`` is the one-shot convenience form and
returns a complex64 radargram shaped like ``compile_rdrgrm``'s (nr, ns).

Forms: ``"fast"`` (fused FP32 split-precision kernels) and ``"plain"`` (the
FP64 restatement of the reference trace loop).  There is no CPU fallback:
without the library, or without a GPU, calls raise.
"""
import ctypes

import numpy as np

from . import _abi
from . import param_gen
from . import traces as _traces

FORMS = {"plain": _abi.RP_FORM_PLAIN_F64, "fast": _abi.RP_FORM_FAST_F32}
OUT_COMPLEX128 = 0x100


# cudaStreamLegacy: the legacy default stream as an explicit handle.  A NULL
# stream handle means "the library's own stream" in the C ABI, so torch's
# default stream (handle 0) is passed as this value instead.
CUDA_STREAM_LEGACY = 0x1


def stream_handle(stream=None, device=None):
    """The cudaStream_t to hand to the C ABI for a torch stream.

    ``None`` selects torch's current stream on ``device``, so the call is
    ordered after the torch work that produced its inputs (and before the
    work that reads its outputs).  Torch's default stream has handle 0,
    which the C ABI would read as "the library's own stream"; it is passed
    as cudaStreamLegacy instead."""
    import torch
    if stream is None:
        stream = torch.cuda.current_stream(device)
    h = int(stream.cuda_stream)
    return ctypes.c_void_p(h if h != 0 else CUDA_STREAM_LEGACY)


def _as_params(params):
    if isinstance(params, _abi.RpParams):
        return params
    return param_gen.to_rp_params(params)


def prisms_from_conductivity(p, prisms_cond):
    """(7, P) prisms with a conductivity row -> alpha row (rp_prism_alpha)."""
    pr = np.array(prisms_cond, dtype=np.float64).reshape(7, -1).copy()
    lib = _abi.lib()
    for k in range(pr.shape[1]):
        a = ctypes.c_double()
        _abi.check("rp_prism_alpha", lib.rp_prism_alpha(ctypes.byref(p), float(pr[0, k]), ctypes.byref(a)))
        pr[0, k] = a.value
    return pr


class Scene:
    """A resident scene: facets (12, N), targets (7, T), prisms (7, P) with alpha.

    The library copies what it needs at creation; the scene keeps no
    reference to the host arrays (which may be a store's memory mapping)."""

    def __init__(self, params, facets, targets=None, prisms=None, device=0):
        self.params = _as_params(params)
        facets = np.ascontiguousarray(facets, dtype=np.float64).reshape(12, -1)
        if targets is None:
            targets = np.zeros((7, 0))
        targets = np.ascontiguousarray(targets, dtype=np.float64).reshape(7, -1)
        if prisms is None:
            prisms = np.zeros((7, 0))
        prisms = np.ascontiguousarray(prisms, dtype=np.float64).reshape(7, -1)
        self.nf, self.nt, self.np = facets.shape[1], targets.shape[1], prisms.shape[1]
        self.nr = int(self.params.nr)
        self.device = int(device)
        self._h = ctypes.c_void_p()
        lib = _abi.lib()
        rc = lib.rp_scene_create(ctypes.byref(self.params), facets.ctypes.data, self.nf, targets.ctypes.data,
                                 self.nt, prisms.ctypes.data, self.np, int(device), ctypes.byref(self._h))
        _abi.check("rp_scene_create", rc)

    @property
    def handle(self):
        return self._h.value

    def close(self):
        if self._h and self._h.value:
            _abi.lib().rp_scene_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def footprint(self):
        b = ctypes.c_int64()
        _abi.check("rp_scene_footprint", _abi.lib().rp_scene_footprint(self._h, ctypes.byref(b)))
        return b.value

    def scratch_bytes(self, ns, form="fast"):
        b = ctypes.c_int64()
        _abi.check("rp_query_footprint",
                   _abi.lib().rp_query_footprint(self._h, int(ns), FORMS[form], ctypes.byref(b)))
        return b.value

    def default_traces(self):
        return _traces.linear_track(self.params)

    def simulate(self, traces=None, form="fast", complex128=False, return_counts=False):
        """Simulate traces (ns, 9) on host memory; returns complex (ns, nr)."""
        tr = self.default_traces() if traces is None else traces
        tr = np.ascontiguousarray(tr, dtype=np.float64).reshape(-1, 9)
        ns = tr.shape[0]
        out = np.zeros((ns, self.nr), np.complex128 if complex128 else np.complex64)
        counts = np.zeros((ns, 2), np.int64)
        f = FORMS[form] | (OUT_COMPLEX128 if complex128 else 0)
        rc = _abi.lib().rp_simulate(self._h, tr.ctypes.data, ns, f, out.ctypes.data, 0,
                                    counts.ctypes.data, None)
        _abi.check("rp_simulate", rc)
        return (out, counts) if return_counts else out

    def simulate_device(self, d_traces, d_out, form="fast", stream=None, complex128=False,
                        counts=None):
        """Resident-input path: d_traces (ns, 9) float64 and d_out (ns, nr)
        complex64 torch CUDA tensors; runs on ``stream`` (a torch stream;
        default: torch's current stream on the scene's device, so the call is
        ordered after the torch work that filled its inputs).
        ``counts``: optional int64 numpy array (ns, 2) filled with N_ill, N_t."""
        ns = int(d_traces.shape[0])
        f = FORMS[form] | (OUT_COMPLEX128 if complex128 else 0)
        sp = stream_handle(stream, self.device)
        cp = None if counts is None else counts.ctypes.data
        rc = _abi.lib().rp_simulate_device(self._h, ctypes.c_void_p(d_traces.data_ptr()), ns, f,
                                           ctypes.c_void_p(d_out.data_ptr()), cp, sp)
        _abi.check("rp_simulate_device", rc)

    def capture(self, traces, d_traces, d_out):
        """Record one fast-form call as a CUDA graph (rp_graph_create):
        ``traces`` (ns, 9) float64 on the host plan it; ``d_traces`` (ns, 9)
        float64 and ``d_out`` (ns, nr) complex64 torch CUDA tensors are the
        buffers every replay reads and writes.  The inputs must hold the
        traces when this is called (the call runs once eagerly first).
        Returns a :class:`Graph`."""
        import torch
        tr = np.ascontiguousarray(traces, dtype=np.float64).reshape(-1, 9)
        ns = tr.shape[0]
        if tuple(d_traces.shape) != (ns, 9) or tuple(d_out.shape) != (ns, self.nr):
            raise ValueError("capture: d_traces must be (ns, 9) and d_out (ns, nr)")
        torch.cuda.current_stream(d_traces.device).synchronize()     # inputs written before the eager run
        g = ctypes.c_void_p()
        rc = _abi.lib().rp_graph_create(self._h, tr.ctypes.data, ctypes.c_void_p(d_traces.data_ptr()), ns,
                                        ctypes.c_void_p(d_out.data_ptr()), ctypes.byref(g))
        _abi.check("rp_graph_create", rc)
        return Graph(g.value, ns, (self, d_traces, d_out), d_traces.device)

    def simulate_host_ptrs(self, traces_ptr, ns, out_ptr, form="fast", stream=None, counts=None):
        """rp_simulate on raw host pointers (e.g. pinned torch tensors); runs
        on ``stream`` (default: torch's current stream on the scene's device)."""
        f = FORMS[form]
        sp = stream_handle(stream, self.device)
        cp = None if counts is None else counts.ctypes.data
        rc = _abi.lib().rp_simulate(self._h, ctypes.c_void_p(traces_ptr), int(ns), f,
                                    ctypes.c_void_p(out_ptr), 0, cp, sp)
        _abi.check("rp_simulate", rc)


class Graph:
    """A captured fast-form call (Scene.capture) or batch (capture_batch):
    launch() replays the whole call on a stream with one graph launch; check()
    after the replay has finished returns the counts (ns, 2; a batch's jobs
    stacked in job order) or raises the status a direct call would have
    raised."""

    def __init__(self, handle, ns, keep, device):
        self._h = handle
        self.ns = ns
        self._keep = keep          # the scenes and the device buffers the graph uses
        self.device = device

    def launch(self, stream=None):
        _abi.check("rp_graph_launch", _abi.lib().rp_graph_launch(ctypes.c_void_p(self._h),
                                                                 stream_handle(stream, self.device.index)))

    def check(self, stream=None):
        """Waits for ``stream`` (default: torch's current stream), then reads
        the replay's flags and counts."""
        import torch
        (stream if stream is not None else torch.cuda.current_stream(self.device)).synchronize()
        counts = np.zeros((self.ns, 2), np.int64)
        _abi.check("rp_graph_check", _abi.lib().rp_graph_check(ctypes.c_void_p(self._h), counts.ctypes.data))
        return counts

    def close(self):
        if self._h:
            _abi.lib().rp_graph_destroy(ctypes.c_void_p(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_timing(enable=True):
    """Per-stage CUDA-event timing of this thread's calls (rp_set_timing)."""
    _abi.lib().rp_set_timing(1 if enable else 0)


def last_timing():
    """Stage times (ms) of this thread's last call: setup, pairs, compression,
    surface+sum, and the pair-kernel launch count."""
    buf = (ctypes.c_double * 5)()
    _abi.lib().rp_last_timing(buf, 5)
    return {"setup_ms": buf[0], "pairs_ms": buf[1], "compress_ms": buf[2], "tail_ms": buf[3],
            "pair_launches": int(buf[4])}


def last_launch_count():
    n = ctypes.c_int64()
    _abi.lib().rp_last_launch_count(ctypes.byref(n))
    return n.value


def simulate(params, facets, targets=None, traces=None, form="fast", prisms=None, device=0):
    """One-shot simulation; returns the complex64 radargram (nr, ns)."""
    with Scene(params, facets, targets, prisms, device) as sc:
        return sc.simulate(traces, form=form).T


class Workspace:
    """Device scratch for calls on one stream (rp_workspace)."""

    def __init__(self, device=0):
        self.device = device
        self._h = ctypes.c_void_p()
        _abi.check("rp_workspace_create", _abi.lib().rp_workspace_create(int(device), ctypes.byref(self._h)))

    @property
    def handle(self):
        return self._h

    def bytes(self):
        b = ctypes.c_int64()
        _abi.check("rp_workspace_bytes", _abi.lib().rp_workspace_bytes(self._h, ctypes.byref(b)))
        return b.value

    def close(self):
        if self._h and self._h.value:
            _abi.lib().rp_workspace_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def simulate_batch(jobs, workspace=None, stream=None, return_counts=False):
    """Fast form over many scenes in one call (rp_simulate_batch).

    ``jobs``: a list of (Scene, traces (ns, 9)) pairs, scenes of any sizes and
    bands on one device.  The pair stage of all of them runs as one persistent
    launch.  Returns one complex64 (ns, nr) array per job (and the (ns, 2)
    counts per job with ``return_counts``)."""
    import torch
    if not jobs:
        return []
    dev = jobs[0][0].device
    ws = workspace if workspace is not None else Workspace(dev)
    d_tr, d_out, counts = [], [], []
    arr = (_abi.RpJob * len(jobs))()
    for i, (sc, tr) in enumerate(jobs):
        tr = np.ascontiguousarray(tr, dtype=np.float64).reshape(-1, 9)
        t = torch.from_numpy(tr).to(f"cuda:{dev}")
        o = torch.empty((tr.shape[0], sc.nr), dtype=torch.complex64, device=f"cuda:{dev}")
        c = np.zeros((tr.shape[0], 2), np.int64)
        d_tr.append(t)
        d_out.append(o)
        counts.append(c)
        arr[i] = _abi.RpJob(sc.handle, t.data_ptr(), tr.shape[0], o.data_ptr(), c.ctypes.data)
    rc = _abi.lib().rp_simulate_batch(arr, len(jobs), ws.handle, stream_handle(stream, dev))
    _abi.check("rp_simulate_batch", rc)
    outs = [o.cpu().numpy() for o in d_out]
    return (outs, counts) if return_counts else outs


def capture_batch(jobs, d_traces, d_outs):
    """Record one simulate_batch call as a CUDA graph (rp_graph_create_batch).

    ``jobs``: (Scene, traces (ns, 9) float64 on the host) pairs that plan the
    call; ``d_traces[j]`` (ns_j, 9) float64 and ``d_outs[j]`` (ns_j, nr_j)
    complex64 torch CUDA tensors are the buffers every replay reads and
    writes, and must hold the traces when this is called (the call runs once
    eagerly first).  Returns a :class:`Graph`; its check() stacks the jobs'
    counts in job order."""
    import torch
    if not jobs or len(jobs) != len(d_traces) or len(jobs) != len(d_outs):
        raise ValueError("capture_batch: one trace buffer and one output buffer per job")
    arr = (_abi.RpJob * len(jobs))()
    hs = []
    for j, ((sc, tr), dt, do) in enumerate(zip(jobs, d_traces, d_outs)):
        tr = np.ascontiguousarray(tr, dtype=np.float64).reshape(-1, 9)
        ns = tr.shape[0]
        if tuple(dt.shape) != (ns, 9) or tuple(do.shape) != (ns, sc.nr):
            raise ValueError(f"capture_batch: job {j}: d_traces must be (ns, 9) and d_out (ns, nr)")
        hs.append(tr)
        arr[j] = _abi.RpJob(sc.handle, dt.data_ptr(), ns, do.data_ptr(), None)
    ptrs = (ctypes.c_void_p * len(hs))(*[h.ctypes.data for h in hs])
    torch.cuda.current_stream(d_traces[0].device).synchronize()     # inputs written before the eager run
    g = ctypes.c_void_p()
    rc = _abi.lib().rp_graph_create_batch(arr, len(jobs), ptrs, ctypes.byref(g))
    _abi.check("rp_graph_create_batch", rc)
    return Graph(g.value, sum(h.shape[0] for h in hs), (jobs, d_traces, d_outs, hs), d_traces[0].device)


def split_parts(enable=True):
    """Split the facet parts of small calls (rp_split_parts; on by default).
    Off: every trace's result is bitwise independent of the call's shape."""
    _abi.lib().rp_split_parts(1 if enable else 0)


def autotune(enable=True):
    """Switch the pair-kernel autotuner on or off (rp_autotune)."""
    _abi.lib().rp_autotune(1 if enable else 0)


def autotune_query(multi, degree=0, specular=False):
    """The tuned pair-kernel configuration (0-3; 0-1 for the specular-mode
    kernel) or -1 when not tuned yet."""
    c = ctypes.c_int()
    kind = 2 if specular else int(bool(multi))
    _abi.check("rp_autotune_query", _abi.lib().rp_autotune_query(kind, int(degree), ctypes.byref(c)))
    return c.value
