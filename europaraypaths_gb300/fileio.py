"""The reference's text file formats through the library's C parsers.

Facet (.fct), target, source-path, gain-pattern, receive-window and
attenuation-prism files are read into the SoA / row arrays of the C ABI;
traces are written as "%e %e" per bin, one s%06d.txt per trace
(src/CUDA/file_io.cu:284-624).
"""
import ctypes

import numpy as np

from . import _abi


def _b(path):
    return str(path).encode()


def count_records(path):
    n = ctypes.c_int64()
    _abi.check("rp_count_records", _abi.lib().rp_count_records(_b(path), ctypes.byref(n)))
    return n.value


def _read_soa(func, path, rows, *extra):
    cap = count_records(path)
    soa = np.zeros((rows, max(cap, 1)), np.float64)
    n = ctypes.c_int64()
    args = [_b(path)] + list(extra) + [soa.ctypes.data, cap, ctypes.byref(n)]
    _abi.check(func, getattr(_abi.lib(), func)(*args))
    return np.ascontiguousarray(soa[:, :n.value])


def read_facets(path):
    """(12, N) facets of a .fct file (loadFacetFile)."""
    return _read_soa("rp_read_facets", path, 12)


def read_targets(path):
    """(7, T) targets of a 3/4/6/7-column target file (loadTargetFile)."""
    return _read_soa("rp_read_targets", path, 7)


def read_prisms(path, p):
    """(7, P) prisms with alpha from a conductivity file (loadAttenPrismFile)."""
    return _read_soa("rp_read_prisms", path, 7, ctypes.byref(p))


def _read_rows(func, path, width):
    cap = count_records(path)
    rows = np.zeros((max(cap, 1), width), np.float64)
    n = ctypes.c_int64()
    _abi.check(func, getattr(_abi.lib(), func)(_b(path), rows.ctypes.data, cap, ctypes.byref(n)))
    return rows[:n.value]


def read_sources(path):
    """(ns, 6) source positions and normals (loadSourceFile)."""
    return _read_rows("rp_read_sources", path, 6)


def read_gains(path):
    """(ns, 2) surface/subsurface gains in dB (loadGainFile)."""
    return _read_rows("rp_read_gains", path, 2)


def read_rx_window(path, ns):
    """(ns,) receive-window starts; exactly ns entries (loadRxWindowPositions)."""
    out = np.zeros(max(ns, 1), np.float64)
    _abi.check("rp_read_rx_window", _abi.lib().rp_read_rx_window(_b(path), out.ctypes.data, ns))
    return out[:ns]


def write_trace(path, col):
    """Write one complex column as "%e %e" lines (saveSignalToFile)."""
    c = np.ascontiguousarray(np.asarray(col, dtype=np.complex64))
    _abi.check("rp_write_trace", _abi.lib().rp_write_trace(_b(path), c.ctypes.data, c.shape[0]))


def check_directory(path):
    _abi.check("rp_check_directory", _abi.lib().rp_check_directory(_b(path)))


def clear_traces(path):
    n = ctypes.c_int64()
    _abi.check("rp_clear_traces", _abi.lib().rp_clear_traces(_b(path), ctypes.byref(n)))
    return n.value
