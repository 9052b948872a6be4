"""Azimuth focusing on the GPU: drop-in for ``src/PYTHON/simple_focusing.py``.

Same functions and arguments as the reference:

* ``focus_rdrgrm(rdrgrm, par, st=None, en=None, return_shifts=False,
  return_match_filter=False)`` (simple_focusing.py:310-404): every pixel
  focused over its range row's synthetic aperture.  The per-row geometry
  (range-bin shifts, matched filter) and all pixels run in libraypath
  (``rp_focus_geometry`` / ``rp_focus_aperture``);
* ``full_focus_at_center(rdrgrm, par, c1=299792458)``
  (simple_focusing.py:115-185): range-cell-migration correction for a point
  target under trace ns // 2 and one azimuth matched filter.  Its per-trace
  Snell geometry (one root per trace) is found on the host as in the
  reference; the correction and the filter run in ``rp_focus_center``;
* the geometry helpers ``snell_intersection``, ``est_slant_range``,
  ``get_target_phase`` and ``slantrange_to_rangebin`` with the reference's
  arguments.

``rdrgrm`` is (range bins, traces), complex.  Results come back in the
input's precision (complex64 or complex128); the sums run in FP32.  The
reference's plots and progress prints are not reproduced.
"""
import ctypes

import numpy as np

from . import _abi

C1 = 299792458


class FocusParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("rx_window_m", "rx_window_offset_m", "rx_sample_rate",
                                               "sin_aperture", "spacing", "altitude", "eps_2", "lam", "c1",
                                               "bracket_hi")]


def _lam(par):
    return par["lam"] if "lam" in par else C1 / par["frequency"]


def _focus_params(par):
    return FocusParams(float(par["rx_window_m"]), float(par["rx_window_offset_m"]), float(par["rx_sample_rate"]),
                       float(np.sin(np.radians(par["aperture"]))), float(par["spacing"]), float(par["altitude"]),
                       float(par["eps_2"]), float(_lam(par)), float(C1), float(np.radians(20)))


def _complex_in(rdrgrm):
    a = np.ascontiguousarray(rdrgrm)
    if a.dtype == np.complex128:
        return a, 1
    return np.ascontiguousarray(a, dtype=np.complex64), 0


# -------------------------------------------------------------- geometry --
def slantrange_to_rangebin(sltrng, params, c1=C1):
    """unit_convs.py:22-24."""
    dm = c1 / params["rx_sample_rate"]
    return ((sltrng - params["rx_window_offset_m"]) // dm).astype(int)


def snell_intersection(xA, zA, xB, zB, v1, v2):
    """simple_focusing.py:10-44: interface crossing of the Snell ray A -> B."""
    from scipy.optimize import brentq

    def f(x):
        return (x - xA) / (v1 * np.sqrt((x - xA) ** 2 + zA ** 2)) - (xB - x) / (v2 * np.sqrt((xB - x) ** 2 + zB ** 2))
    return brentq(f, min(xA, xB) - abs(xB - xA), max(xA, xB) + abs(xB - xA))


def est_slant_range(sx, sz, tx, tz, c1, c2, trim=True, clutter=False):
    """simple_focusing.py:48-79."""
    if tz > 0 or clutter:
        return np.sqrt((sx - tx) ** 2 + (sz - tz) ** 2)
    est = []
    for x in sx:
        ix = snell_intersection(x, sz, tx, tz, c1, c2)
        est.append(np.sqrt((x - ix) ** 2 + sz ** 2) + np.sqrt((ix - tx) ** 2 + tz ** 2) * (c1 / c2))
    est = np.array(est)
    if not trim:
        return est
    m, h = int(np.argmin(est)), len(est) // 2
    return est[:-2 * (h - m)] if m < h else est[2 * (m - h):]


def get_target_phase(params, h, d, xoff, cmplx_out=False):
    """simple_focusing.py:89-112: two-way phase through the refraction point."""
    from scipy.optimize import brentq
    eps = params["eps_2"]

    def ang(th, x):
        return h * np.tan(np.arcsin(np.sqrt(eps) * np.sin(th))) + d * np.tan(th) - x
    xoff = np.asarray(xoff, dtype=float)
    th_r = np.array([brentq(ang, 0.0, np.radians(20), args=(abs(x),)) for x in xoff])
    th_i = np.arcsin(np.sqrt(eps) * np.sin(th_r))
    cmplx = np.exp(((-4j * np.pi) / _lam(params)) * (h / np.cos(th_i) + d / np.cos(th_r) * np.sqrt(eps)))
    return cmplx if cmplx_out else np.degrees(np.angle(cmplx))


# -------------------------------------------------------------- focusing --
def focus_rdrgrm(rdrgrm, par, st=None, en=None, return_shifts=False, return_match_filter=False):
    """simple_focusing.py:310-404 on the GPU.  Rows outside [st, en] are zero
    when both are given (and non-zero, as in the reference)."""
    a, in128 = _complex_in(rdrgrm)
    Nr, Na = a.shape
    P = _focus_params(par)
    lo, hi = (int(st), int(en)) if (st and en) else (0, Nr - 1)
    hi = min(hi, Nr - 1)
    if return_shifts or return_match_filter:     # the reference returns the first processed row's
        rng = par["rx_window_m"] * (lo / Nr) + par["rx_window_offset_m"]
        maxA = int(2 * rng * P.sin_aperture / par["spacing"]) + 2
        apt = np.zeros(2, np.int32)
        rb = np.zeros(maxA, np.int32)
        mf = np.zeros(2 * maxA, np.float32)
        _abi.check("rp_focus_geometry", _abi.lib().rp_focus_geometry(
            ctypes.byref(P), Nr, lo, 1, maxA, apt.ctypes.data, rb.ctypes.data, mf.ctypes.data))
        n = int(apt[0])
        if return_shifts:
            return rb[:n].astype(int)
        return (mf[0:2 * n:2] + 1j * mf[1:2 * n:2]).astype(np.complex128)
    out = np.zeros((Nr, Na), a.dtype)
    if lo <= hi:
        _abi.check("rp_focus_aperture", _abi.lib().rp_focus_aperture(
            ctypes.byref(P), a.ctypes.data, Nr, Na, in128, lo, hi, out.ctypes.data, in128, None))
    return out


def full_focus_at_center(rdrgrm, par, c1=C1, sx_linspace=True):
    """simple_focusing.py:115-185 on the GPU (the shifts and matched filter
    from the reference's host geometry; the correction and filter on the
    device).  The target must lie under trace ns // 2."""
    if not sx_linspace:
        raise NotImplementedError("Irregular source spacing is not yet supported.")
    a, in128 = _complex_in(rdrgrm)
    Nr, Na = a.shape
    sx = par["sx0"] + par["sdx"] * np.arange(par["ns"])
    c2 = c1 / np.sqrt(par["eps_2"])
    sl = est_slant_range(sx, par["sz"], par["tx"], par["tz"], c1, c2)
    if sl.shape[0] != Na:
        raise ValueError(f"the slant-range curve keeps {sl.shape[0]} of {Na} traces: "
                         "the target must lie under trace ns // 2")
    rb = slantrange_to_rangebin(sl, par, c1=c1)
    shifts = np.ascontiguousarray(rb - np.min(rb), dtype=np.int64)
    mf = np.conj(get_target_phase(par, par["sz"], par["tz"], sx - par["tx"], cmplx_out=True))
    mf32 = np.ascontiguousarray(mf.astype(np.complex64))
    out = np.zeros((Nr, Na), np.complex128 if in128 else np.complex64)
    _abi.check("rp_focus_center", _abi.lib().rp_focus_center(
        a.ctypes.data, Nr, Na, in128, shifts.ctypes.data, mf32.ctypes.data, out.ctypes.data, in128, None))
    return out
