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
``flyby``        8000x8000 facets at 2.5 m, fractal H 0.75 / RMS 8 m; rough
                 interfaces 1 km and 3 km deep as 400x400 targets at 50 m
                 each; 10,000 traces at 25 km, 2 m spacing; 60 MHz /
                 10 MHz, 24 MHz sampling, 16384 bins; aperture 3 deg.
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


def flyby(seed=5, n_facets_side=8000, fs=2.5, target_spacing=50.0, trace_spacing=2.0):
    """The flyby-scale scene (64M facets, two rough layers, 10,000 traces at
    25 km, 60 MHz / 10 MHz sampled at 24 MHz into 16384 bins).

    * surface: 8000x8000 facets at 2.5 m (20 km square), fractal heights
      (Hurst 0.75, RMS 8 m);
    * two rough interfaces 1 km and 3 km deep (RMS 10 m, l = 200 m), each
      sampled as a target grid at 50 m (2 x 400x400 = 320k targets, ttype 1);
    * traces along x at 25 km altitude every 2 m across the scene (10,000),
      aperture 3 deg;
    * eps 3.15 above the first interface, sigma 1e-6.  The permittivities
      below the interfaces (3.2, 6.0) have no counterpart in the reference's
      physics (targets carry no Fresnel term) and are not used.
    A smaller ``n_facets_side`` keeps the spacings and band and shrinks the
    square (2000 facets: 5 km, 4M facets, 2 x 100x100 targets, 2,500 traces;
    the aperture footprint still fits inside)."""
    side = n_facets_side * fs
    ns = int(round(side / trace_spacing))
    p = base_params(60e6, 10e6, 24e6, 16384, 3.0, 3.15, 1e-6, 8.0, fs, 25e3, ns, trace_spacing, 7.3)
    dom = {"fs": fs, "nx": n_facets_side, "ny": n_facets_side, "ox": -side / 2, "oy": -side / 2}
    h = fractal_field(n_facets_side, n_facets_side, fs, 8.0, 0.75, seed)
    facets = ss.surface_arrays_blocked(dom, h)
    del h
    n_targets_side = max(1, int(round(side / target_spacing)))
    tdom = {"fs": target_spacing, "nx": n_targets_side, "ny": n_targets_side, "ox": -side / 2, "oy": -side / 2}
    layers = []
    for k, depth in enumerate((1000.0, 3000.0)):
        th = gaussian_field(n_targets_side, n_targets_side, target_spacing, 10.0, 200.0, seed * 1000 + k)
        layers.append(ss.target_arrays(tdom, "flat", zoffset=-depth, heights=th))
    targets = np.concatenate(layers, axis=1)
    return {"name": "flyby", "params": p, "facets": facets, "targets": targets}


def uneven_batch(seed=3, n_scenes=64, min_facets=10_000, max_facets=4_000_000, alt=25e3):
    """Many independent scenes of uneven size (the batched-scenes workload).

    Per scene (all drawn from ``default_rng(seed)``):
    * facet count log-uniform in [min_facets, max_facets] (a square grid);
    * band: 9 MHz / 1 MHz chirp sampled at 4 MHz with fs = 10 m, or 60 MHz /
      10 MHz sampled at 24 MHz with fs = 2.5 m (equal odds);
    * bins: 2048, 4096 or 8192;
    * surface: Gaussian field, RMS U(1, 10) m, l = 50 m;
    * one or two target layers at U(0.5, 3) km depth, 50 m sampling, each a
      Gaussian interface (RMS 5 m, l = 200 m), eps 3.15, sigma 1e-6;
    * trace count U{50..2000}, linear along x across the scene at 25 km,
      aperture 3 deg.
    Returns a list of scene dictionaries (name, params, facets, targets)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_scenes):
        nfac = float(np.exp(rng.uniform(np.log(min_facets), np.log(max_facets))))
        n_side = max(8, int(round(np.sqrt(nfac))))
        vhf = bool(rng.integers(0, 2))
        f0, B, smpl, fs, gain = (60e6, 10e6, 24e6, 2.5, 7.3) if vhf else (9e6, 1e6, 4e6, 10.0, 4.0)
        nr = int(rng.choice([2048, 4096, 8192]))
        rms = float(rng.uniform(1.0, 10.0))
        nlay = int(rng.integers(1, 3))
        depths = sorted(float(d) for d in rng.uniform(500.0, 3000.0, nlay))
        ns = int(rng.integers(50, 2001))
        side = n_side * fs
        sdx = side / ns
        p = base_params(f0, B, smpl, nr, 3.0, 3.15, 1e-6, rms, fs, alt, ns, sdx, gain)
        dom = {"fs": fs, "nx": n_side, "ny": n_side, "ox": -side / 2, "oy": -side / 2}
        h = gaussian_field(n_side, n_side, fs, rms, 50.0, seed * 1000 + i)
        facets = ss.surface_arrays(dom, "flat", heights=h)
        tn = max(1, int(side // 50.0))
        tdom = {"fs": 50.0, "nx": tn, "ny": tn, "ox": -tn * 25.0, "oy": -tn * 25.0}
        layers = []
        for k, d in enumerate(depths):
            th = gaussian_field(tn, tn, 50.0, 5.0, 200.0, seed * 1000 + 500 + 2 * i + k)
            layers.append(ss.target_arrays(tdom, "flat", zoffset=-d, heights=th))
        targets = np.concatenate(layers, axis=1)
        out.append({"name": f"uneven_{i}", "params": p, "facets": facets, "targets": targets,
                    "band": "60/10 MHz" if vhf else "9/1 MHz", "layers": nlay})
    return out
