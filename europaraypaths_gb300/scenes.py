"""Seeded synthetic scenes for the benchmark and test workloads.

No public dataset is involved: every surface, target layer and trace table is
generated here in FP64 from ``numpy.random.default_rng(seed)``.

* Gaussian-correlated heights: white noise filtered in the Fourier domain with
  amplitude sqrt(PSD), PSD(k) proportional to exp(-k^2 l^2 / 4).
* Fractal heights: PSD(k) proportional to k^-(2H+2) (DC removed).
* Heights are rescaled to the requested RMS; normals and tangents come from
  ``simple_surfaces.gen_normals`` exactly as the reference computes them.
* Target layers are ``make_target_array`` grids (ttype 1) on the interface.

Workloads (named by what they are):

``small_plain``  200x200 facets at 10 m, Gaussian RMS 2 m / l = 50 m; flat
                 reflector 1 km deep (40x40 targets at 50 m), eps 3.15,
                 10 dB/km loss; 100 traces at 25 km, 50 m spacing; 9 MHz /
                 1 MHz, 4 MHz sampling, 2048 bins; aperture 10 deg.
``large_scene``  2000x2000 facets at 5 m, fractal H 0.8 / RMS 5 m; rough
                 interface 1.5 km deep (RMS 10 m, l = 200 m) as 200x200
                 targets at 50 m; 2000 traces at 50 km, 5 m spacing;
                 9 MHz / 1 MHz, 4 MHz sampling, 4096 bins; aperture 3 deg.
"""
import numpy as np

from . import simple_surfaces as ss

C_NR = 299792480.0     # the constant of the reference's nr expression (file_io.cu:212)
PI_FRIIS = 3.14159     # the pi of the reference's attenuation formula (file_io.cu:196-206)


def rx_window_for_bins(nr, smpl):
    """rx_window_m for which the reference's nr expression yields exactly nr."""
    return (nr + 0.5) * C_NR / smpl


def sigma_for_loss(db_per_km, f0, eps):
    """Conductivity giving a one-way power loss of db_per_km through the
    reference's alpha formula (file_io.cu:202-206), by bisection."""
    # power loss dB/m = 10 log10(e^2) * alpha = 8.686 * alpha
    alpha_target = db_per_km / 1000.0 / 8.685889638065037
    lam = 299792458.0 / f0

    def alpha(sig):
        epp = sig / (2 * PI_FRIIS * f0 * 8.85e-12)
        a = np.sqrt(1 + (epp / eps) ** 2) - 1
        a = np.sqrt(0.5 * eps * a)
        return a * 2 * PI_FRIIS / lam

    lo, hi = 0.0, 1.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if alpha(mid) < alpha_target:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def _filtered_field(nx, ny, fs, psd, rms, seed):
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((ny, nx))
    kx = 2 * np.pi * np.fft.fftfreq(nx, d=fs)
    ky = 2 * np.pi * np.fft.fftfreq(ny, d=fs)
    KX, KY = np.meshgrid(kx, ky)
    K = np.sqrt(KX ** 2 + KY ** 2)
    amp = np.sqrt(psd(K))
    h = np.real(np.fft.ifft2(np.fft.fft2(w) * amp))
    h -= h.mean()
    s = h.std()
    return h * (rms / s) if s > 0 else h


def gaussian_field(nx, ny, fs, rms, corr_len, seed):
    """Heights with Gaussian correlation: PSD ~ exp(-k^2 l^2 / 4)."""
    return _filtered_field(nx, ny, fs, lambda k: np.exp(-(k * corr_len) ** 2 / 4.0), rms, seed)


def fractal_field(nx, ny, fs, rms, hurst, seed):
    """Self-affine heights: PSD ~ k^-(2H+2), DC removed."""
    def psd(k):
        out = np.zeros_like(k)
        m = k > 0
        out[m] = k[m] ** (-(2 * hurst + 2))
        return out
    return _filtered_field(nx, ny, fs, psd, rms, seed)


def base_params(f0, B, smpl, nr, aperture, eps2, sig2, rms, fs, alt, ns, sdx, gain_db):
    """A gen_params-style dictionary for a linear along-x source track."""
    return {
        "eps_1": 1.0, "sig_1": 0.0, "mu_1": 1.0, "mu_2": 1.0,
        "convolution": True, "convolution_linear": True, "specular": False,
        "lossless": False, "incoherent": False, "debug_surface": False,
        "rerad_funct": 1, "buff": 1.1,
        "power": 100, "frequency": f0, "bandwidth": B,
        "surface_gain": gain_db, "subsurface_gain": gain_db, "polarization": "HH",
        "eps_2": eps2, "sig_2": sig2, "rms_height": rms, "fs": fs,
        "rx_window_m": rx_window_for_bins(nr, smpl), "rx_sample_rate": smpl,
        "rx_window_offset_m": alt - 1000.0,
        "ns": ns, "aperture": aperture,
        "sx0": -(ns - 1) * sdx / 2.0, "sy": 0.0, "sz": alt, "sdx": sdx,
        "altitude": alt,
        "lam": 299792458 / f0, "k": 2 * np.pi * f0 / 299792458,
    }


def small_plain(seed=1, n_facets_side=200, n_targets_side=40, ns=100):
    """The small plain-form scene (CPU-runnable); sizes can be reduced for tests."""
    fs = 10.0 * 200 / n_facets_side
    p = base_params(9e6, 1e6, 4e6, 2048, 10.0, 3.15, sigma_for_loss(10.0, 9e6, 3.15),
                    2.0, fs, 25e3, ns, 50.0, 4.0)
    side = 2000.0
    dom = {"fs": fs, "nx": n_facets_side, "ny": n_facets_side, "ox": -side / 2, "oy": -side / 2}
    h = gaussian_field(n_facets_side, n_facets_side, fs, 2.0, 50.0, seed)
    facets = ss.surface_arrays(dom, "flat", heights=h)
    tfs = side / n_targets_side
    tdom = {"fs": tfs, "nx": n_targets_side, "ny": n_targets_side, "ox": -side / 2, "oy": -side / 2}
    targets = ss.target_arrays(tdom, "flat", zoffset=-1000.0)
    return {"name": "small_plain", "params": p, "facets": facets, "targets": targets}


def large_scene(seed=2, n_facets_side=2000, n_targets_side=200, ns=2000):
    """The single large scene (4M facets, 40k targets, 2000 traces at 50 km)."""
    fs = 5.0 * 2000 / n_facets_side
    p = base_params(9e6, 1e6, 4e6, 4096, 3.0, 3.15, 1e-6, 5.0, fs, 50e3, ns, 5.0, 4.0)
    side = n_facets_side * fs
    dom = {"fs": fs, "nx": n_facets_side, "ny": n_facets_side, "ox": -side / 2, "oy": -side / 2}
    h = fractal_field(n_facets_side, n_facets_side, fs, 5.0, 0.8, seed)
    facets = ss.surface_arrays(dom, "flat", heights=h)
    tfs = 50.0
    tside = n_targets_side * tfs
    tdom = {"fs": tfs, "nx": n_targets_side, "ny": n_targets_side,
            "ox": -tside / 2, "oy": -tside / 2}
    th = gaussian_field(n_targets_side, n_targets_side, tfs, 10.0, 200.0, seed + 1000)
    targets = ss.target_arrays(tdom, "flat", zoffset=-1500.0, heights=th)
    return {"name": "large_scene", "params": p, "facets": facets, "targets": targets}
