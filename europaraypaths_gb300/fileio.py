"""The reference's text file formats through the library's C parsers, and
their binary replacements.

Facet (.fct), target, source-path, gain-pattern, receive-window and
attenuation-prism files are read into the SoA / row arrays of the C ABI;
traces are written as "%e %e" per bin, one s%06d.txt per trace
(src/CUDA/file_io.cu:284-624).

Binary stores (no counterpart in the reference): facet and target stores
hold the C ABI's float64 SoA behind a 32-byte header and are memory-mapped
(no parsing); a radargram file holds every trace, trace-major.  Convert a
text file with ``python -m europaraypaths_gb300.fileio facets.fct facets.rpf``.
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


# ------------------------------------------------------------ binary store --
STORE_FACETS, STORE_TARGETS, STORE_RADARGRAM = 0, 1, 2
_COLS = {STORE_FACETS: 12, STORE_TARGETS: 7}


def store_kind(path):
    """0 facet store, 1 target store, 2 radargram, -1 a text file."""
    k = ctypes.c_int()
    _abi.check("rp_store_kind", _abi.lib().rp_store_kind(_b(path), ctypes.byref(k)))
    return k.value


def write_store(path, soa, kind):
    """Write a (12, N) facet or (7, T) target SoA as a binary store."""
    a = np.ascontiguousarray(np.asarray(soa, dtype=np.float64).reshape(_COLS[kind], -1))
    _abi.check("rp_write_store", _abi.lib().rp_write_store(_b(path), kind, a.ctypes.data, a.shape[1]))


class MappedStore:
    """A read-only memory mapping of a facet or target store; ``soa`` is a
    (cols, n) float64 view of it, valid until ``close()``."""

    def __init__(self, path, kind):
        ptr = ctypes.c_void_p()
        n = ctypes.c_int64()
        self._h = ctypes.c_void_p()
        _abi.check("rp_map_store", _abi.lib().rp_map_store(_b(path), kind, ctypes.byref(ptr), ctypes.byref(n),
                                                            ctypes.byref(self._h)))
        cols = _COLS[kind]
        if n.value > 0:
            buf = (ctypes.c_double * (cols * n.value)).from_address(ptr.value)
            self.soa = np.frombuffer(buf, dtype=np.float64).reshape(cols, n.value)
        else:
            self.soa = np.zeros((cols, 0))
        self.soa.flags.writeable = False

    def close(self):
        if self._h:
            self.soa = None
            _abi.lib().rp_unmap_store(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def load_facets(path):
    """(12, N) facets from a .fct text file or a facet store (detected by its
    header; the store is copied out of its mapping)."""
    if store_kind(path) == STORE_FACETS:
        with MappedStore(path, STORE_FACETS) as m:
            return np.array(m.soa)
    return read_facets(path)


def load_targets(path):
    """(7, T) targets from a target text file or a target store."""
    if store_kind(path) == STORE_TARGETS:
        with MappedStore(path, STORE_TARGETS) as m:
            return np.array(m.soa)
    return read_targets(path)


def write_radargram(path, rdr):
    """Write an (ns, nr) complex64 or complex128 radargram as one file."""
    a = np.ascontiguousarray(rdr)
    if a.dtype not in (np.complex64, np.complex128):
        a = a.astype(np.complex64)
    wide = 1 if a.dtype == np.complex128 else 0
    ns, nr = a.shape
    _abi.check("rp_write_radargram", _abi.lib().rp_write_radargram(_b(path), a.ctypes.data, ns, nr, wide))


def read_radargram(path):
    """(ns, nr) radargram of a radargram file, in its stored precision."""
    ns, nr, wide = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int()
    _abi.check("rp_radargram_info", _abi.lib().rp_radargram_info(_b(path), ctypes.byref(ns), ctypes.byref(nr),
                                                                  ctypes.byref(wide)))
    out = np.zeros((ns.value, nr.value), np.complex128 if wide.value else np.complex64)
    _abi.check("rp_read_radargram", _abi.lib().rp_read_radargram(_b(path), out.ctypes.data, ns.value, nr.value,
                                                                  wide.value))
    return out


def main(argv=None):
    """Convert a facet (.fct) or target text file into a binary store."""
    import argparse
    ap = argparse.ArgumentParser(prog="europaraypaths_gb300.fileio", description=main.__doc__)
    ap.add_argument("src")
    ap.add_argument("dst")
    ap.add_argument("--kind", choices=["facets", "targets"], default="facets")
    a = ap.parse_args(argv)
    if a.kind == "facets":
        write_store(a.dst, read_facets(a.src), STORE_FACETS)
    else:
        write_store(a.dst, read_targets(a.src), STORE_TARGETS)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
