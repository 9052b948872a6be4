"""Test infrastructure: a NumPy restatement of the reference's azimuth
focusing (src/PYTHON/simple_focusing.py, unit_convs.py), the checker for the
CUDA focusing in europaraypaths_gb300.focusing.

Pinned against the reference itself: tests/golden/focus_small.npz holds the
reference's outputs on seeded inputs (tests/golden/make_focus_golden.py) and
tests/test_oracle.py compares this module with them.  Roots are found with
scipy.optimize.brentq on the reference's brackets, as the reference does
(root_scalar(method='brentq')); no plotting.
"""
import numpy as np
from scipy.optimize import brentq

C1 = 299792458


def c2(params, c1=C1):
    """unit_convs.py:16-17."""
    return c1 / np.sqrt(params["eps_2"])


def slantrange_to_rangebin(sltrng, params, c1=C1):
    """unit_convs.py:22-24: floor division by the range-sample length."""
    dm = c1 / params["rx_sample_rate"]
    return ((sltrng - params["rx_window_offset_m"]) // dm).astype(int)


def snell_intersection(xA, zA, xB, zB, v1, v2):
    """simple_focusing.py:10-44: the interface crossing (z = 0) of the
    Snell ray from A (medium 1) to B (medium 2), as the zero of d(time)/dx."""
    def f(x):
        return (x - xA) / (v1 * np.sqrt((x - xA) ** 2 + zA ** 2)) - (xB - x) / (v2 * np.sqrt((xB - x) ** 2 + zB ** 2))
    x_min = min(xA, xB) - abs(xB - xA)
    x_max = max(xA, xB) + abs(xB - xA)
    return brentq(f, x_min, x_max)


def est_slant_range(sx, sz, tx, tz, c1, c2_, trim=True, clutter=False):
    """simple_focusing.py:48-79: one-way slant range per source, through the
    Snell crossing for a buried target, trimmed so its minimum is centred."""
    if tz > 0 or clutter:
        return np.sqrt((sx - tx) ** 2 + (sz - tz) ** 2)
    est = []
    for x in sx:
        ix = snell_intersection(x, sz, tx, tz, c1, c2_)
        est.append(np.sqrt((x - ix) ** 2 + sz ** 2) + np.sqrt((ix - tx) ** 2 + tz ** 2) * (c1 / c2_))
    est = np.array(est)
    if not trim:
        return est
    m = np.argmin(est)
    h = len(est) // 2
    if m < h:
        return est[:-2 * int(h - m)]
    return est[2 * int(m - h):]


def refracted_angle(th_r, xoff, h, d, eps_2):
    """simple_focusing.py:82-86."""
    y = np.arcsin(np.sqrt(eps_2) * np.sin(th_r))
    return h * np.tan(y) + d * np.tan(th_r) - xoff


def get_target_phase(params, h, d, xoff, cmplx_out=False):
    """simple_focusing.py:89-112: two-way phase of a buried point through the
    refraction point (root of refracted_angle on [0, 20 deg])."""
    lam = params["lam"] if "lam" in params else C1 / params["frequency"]
    th_r = np.zeros_like(xoff, dtype=float)
    for i, dx in enumerate(xoff):
        th_r[i] = brentq(refracted_angle, 0.0, np.radians(20), args=(np.abs(dx), h, d, params["eps_2"]))
    th_i = np.arcsin(np.sqrt(params["eps_2"]) * np.sin(th_r))
    corrected_rng = h / np.cos(th_i) + d / np.cos(th_r) * np.sqrt(params["eps_2"])
    cmplx = np.exp(((-4j * np.pi) / lam) * corrected_rng)
    if cmplx_out:
        return cmplx
    return np.degrees(np.angle(cmplx))


def full_focus_at_center(rdrgrm, par, c1=C1):
    """simple_focusing.py:115-185 without its plots: range-cell-migration
    correction by integer rolls, then the azimuth matched filter by FFT at
    twice the trace count, cropped from pad // 2."""
    sx = par["sx0"] + par["sdx"] * np.arange(par["ns"])
    Nr, Na = rdrgrm.shape
    sltrng = est_slant_range(sx, par["sz"], par["tx"], par["tz"], c1, c2(par, c1=c1))
    sltrng_rb = slantrange_to_rangebin(sltrng, par, c1=c1)
    mf = np.conj(get_target_phase(par, par["sz"], par["tz"], sx - par["tx"], cmplx_out=True))
    shift = sltrng_rb - np.min(sltrng_rb)
    rolled = np.array([np.roll(rdrgrm[:, i], -int(shift[i])) for i in range(Na)]).T
    L = 2 * Na
    pad = L - Na
    rolled = np.pad(rolled, ((0, 0), (0, pad)))
    mf = np.pad(mf, (0, pad))
    focused = np.fft.ifft(np.fft.fft(rolled, axis=1, n=L) * np.fft.fft(mf, n=L)[np.newaxis, :], axis=1)
    return focused[:, pad // 2:pad // 2 + Na]


def aperture_row(par, i, Nr):
    """The per-range-row geometry of focus_rdrgrm (simple_focusing.py:328-351):
    (apt_smpl, apt_hsmpl, sltrng_rb, mth_filt)."""
    rng = par["rx_window_m"] * (i / Nr) + par["rx_window_offset_m"]
    apt_m = rng * np.sin(np.radians(par["aperture"]))
    apt_smpl = int(2 * apt_m / par["spacing"])
    apt_hsmpl = int(apt_m / par["spacing"])
    sx = np.linspace(-1 * apt_m, 1 * apt_m, apt_smpl)
    sz = par["altitude"]
    tx = 0
    tz = par["altitude"] - rng
    sltrng = est_slant_range(sx, sz, tx, tz, par["eps_1"], par["eps_2"], trim=False, clutter=True)
    sltrng_rb = slantrange_to_rangebin(sltrng, par)
    mth = np.conj(get_target_phase(par, sz, tz, sx - tx, cmplx_out=True))
    return apt_smpl, apt_hsmpl, sltrng_rb, mth


def focus_rdrgrm(rdrgrm, par, st=None, en=None, return_shifts=False, return_match_filter=False):
    """simple_focusing.py:310-404 without its progress prints: every pixel
    focused over its range row's synthetic aperture (a rolled window, an FFT
    matched filter of length 2 * apt_smpl, one output sample kept)."""
    Nr, Na = rdrgrm.shape
    out = np.zeros_like(rdrgrm)
    for i in range(Nr):
        if st and en and (i < st or i > en):
            continue
        apt_smpl, apt_hsmpl, sltrng_rb, mth = aperture_row(par, i, Nr)
        if return_shifts:
            return sltrng_rb
        if return_match_filter:
            return mth
        L = int(2 * apt_smpl)
        ft = np.fft.fft(np.pad(mth, (0, L - apt_smpl)), n=L)      # the filter's zero padding, cut to L
        for j in range(Na):
            a0, a1 = max(0, j - apt_hsmpl), min(Na, j + apt_hsmpl)
            w = a1 - a0
            # row i of each column rolled by sltrng_rb[k] - i is element sltrng_rb[k] mod Nr
            row = np.array([rdrgrm[sltrng_rb[k] % Nr, a0 + k] for k in range(w)])
            pad = L - w
            f = np.fft.ifft(np.fft.fft(np.pad(row, (0, pad)), n=L) * ft)
            out[i, j] = f[(j - a0) + pad // 2]
    return out
