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
