"""Per-trace state tables (the inputs of one trace-loop iteration).

A trace row is ``sx,sy,sz, snx,sny,snz, rst, grefl_lin, grefr_lin`` -- the
values ``src/CUDA/sim.cu:621-651`` sets before each iteration: the source
position (linear track ``sx0 + is*sdx`` or the source-path file), the source
normal times ``source_normal_multiplier``, the receive-window start (static
offset or the rx-window position file) and the linear gains (static or the
gain-pattern file, ``powf(10, g/10)``).
"""
import numpy as np


def linear_track(p, ns=None, start=0):
    """Trace table of the linear source track of an ``RpParams`` (sim.cu:641-644, 547-552)."""
    ns = p.ns if ns is None else ns
    idx = np.arange(start, start + ns, dtype=np.float64)
    tr = np.zeros((ns, 9))
    tr[:, 0] = p.sx0 + idx * p.sdx
    tr[:, 1] = p.sy
    tr[:, 2] = p.sz
    tr[:, 5] = 1.0 * p.source_normal_multiplier
    tr[:, 6] = p.rx_window_offset_m
    tr[:, 7] = p.grefl_lin
    tr[:, 8] = p.grefr_lin
    return tr


def from_sources(p, sources, rx_window=None, gains_db=None):
    """Trace table from a source-path array (ns, 3 or 6), optional per-trace
    receive-window starts (ns,) and gains in dB (ns, 2) (sim.cu:625-651)."""
    src = np.asarray(sources, dtype=np.float64)
    if src.ndim == 1:
        src = src[None, :]
    ns = src.shape[0]
    tr = np.zeros((ns, 9))
    tr[:, 0:3] = src[:, 0:3]
    if src.shape[1] >= 6:
        tr[:, 3:6] = src[:, 3:6] * p.source_normal_multiplier
    else:
        tr[:, 5] = 1.0 * p.source_normal_multiplier
    if rx_window is None:
        tr[:, 6] = p.rx_window_offset_m
    else:
        rw = np.asarray(rx_window, dtype=np.float64)
        if rw.shape[0] != ns:
            raise ValueError(f"rx window positions: {rw.shape[0]} entries, expected exactly {ns}")
        tr[:, 6] = rw
    if gains_db is None:
        tr[:, 7] = p.grefl_lin
        tr[:, 8] = p.grefr_lin
    else:
        g = np.asarray(gains_db, dtype=np.float64).reshape(-1, 2)
        tr[:, 7] = np.power(10.0, g[:ns, 0] / 10.0)
        tr[:, 8] = np.power(10.0, g[:ns, 1] / 10.0)
    return tr
