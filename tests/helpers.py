"""Shared test helpers: scenes at test sizes and the comparison metrics."""
import numpy as np


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def phase_err_max(a, b, floor_db=-40.0):
    """Max |angle(a/b)| over bins where |b| is above floor_db of the peak."""
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    mag = np.abs(b)
    m = mag > mag.max() * 10 ** (floor_db / 20.0)
    return float(np.max(np.abs(np.angle(a[m] / b[m])))) if m.any() else 0.0


def peak_bins(x):
    return np.argmax(np.abs(np.asarray(x)), axis=-1)


def tiny_scene(nside=30, ntside=4, ns=3, **over):
    from europaraypaths_gb300 import scenes
    sc = scenes.small_plain(n_facets_side=nside, n_targets_side=ntside, ns=ns)
    sc["params"].update(over)
    return sc


def vhf_scene(nr, n_side=120, fs=2.5, nt_side=4, ns=2, seed=5):
    # 60 MHz / 10 MHz chirp sampled at 24 MHz, 2.5 m facets (the VHF band of
    # the batched and flyby workloads), a rough layer 1 km deep
    from europaraypaths_gb300 import scenes, simple_surfaces as ss
    p = scenes.base_params(60e6, 10e6, 24e6, nr, 3.0, 3.15, 1e-6, 1.0, fs, 25e3, ns, 20.0, 7.3)
    side = n_side * fs
    dom = {"fs": fs, "nx": n_side, "ny": n_side, "ox": -side / 2, "oy": -side / 2}
    h = scenes.gaussian_field(n_side, n_side, fs, 1.0, 20.0, seed)
    facets = ss.surface_arrays(dom, "flat", heights=h)
    tfs = side / nt_side
    tdom = {"fs": tfs, "nx": nt_side, "ny": nt_side, "ox": -side / 2, "oy": -side / 2}
    th = scenes.gaussian_field(nt_side, nt_side, tfs, 2.0, 50.0, seed + 1)
    targets = ss.target_arrays(tdom, "flat", zoffset=-1000.0, heights=th)
    return {"params": p, "facets": facets, "targets": targets}
