"""Azimuth focusing (simple_focusing.py: focus_rdrgrm, full_focus_at_center).

CPU: the NumPy oracle (oracle/np_focus.py) against the reference's own
outputs on seeded radargrams (tests/golden/focus_small.npz, made by
tests/golden/make_focus_golden.py).  GPU: the CUDA focusing through the C ABI
against the oracle and the same golden outputs."""
import importlib.util
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
G = os.path.join(HERE, "golden")
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))


def _golden_module():
    spec = importlib.util.spec_from_file_location("make_focus_golden", os.path.join(G, "make_focus_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


@pytest.fixture(scope="module")
def golden():
    m = _golden_module()
    ap, cf = m.inputs()
    return m, ap, cf, np.load(os.path.join(G, "focus_small.npz"))


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_oracle_focus_rdrgrm_matches_reference(golden):
    import np_focus as nf
    m, ap, _, g = golden
    assert np.array_equal(nf.focus_rdrgrm(ap, dict(m.AP_PAR), return_shifts=True), g["ap_shifts"])
    assert np.array_equal(nf.focus_rdrgrm(ap, dict(m.AP_PAR), return_match_filter=True), g["ap_mf"])
    assert rel(nf.focus_rdrgrm(ap, dict(m.AP_PAR)), g["ap_all"]) < 1e-12
    win = nf.focus_rdrgrm(ap, dict(m.AP_PAR), st=5, en=20)
    assert rel(win, g["ap_win"]) < 1e-12
    assert not win[:5].any() and not win[21:].any() and win[5:21].all()


def test_oracle_full_focus_at_center_matches_reference(golden):
    import np_focus as nf
    m, _, cf, g = golden
    assert rel(nf.full_focus_at_center(cf, dict(m.CF_PAR)), g["cf_out"]) < 1e-12


# ---------------------------------------------------------------- GPU -----
@pytest.mark.gpu
def test_gpu_focus_rdrgrm_matches_reference(built_lib, golden):
    from europaraypaths_gb300 import focusing
    m, ap, _, g = golden
    par = dict(m.AP_PAR)
    assert np.array_equal(focusing.focus_rdrgrm(ap, par, return_shifts=True), g["ap_shifts"])
    mf = focusing.focus_rdrgrm(ap, par, return_match_filter=True)
    assert np.abs(mf - g["ap_mf"]).max() < 1e-6
    got = focusing.focus_rdrgrm(ap, par)
    assert got.dtype == np.complex128 and rel(got, g["ap_all"]) < 1e-5
    win = focusing.focus_rdrgrm(ap, par, st=5, en=20)
    assert rel(win, g["ap_win"]) < 1e-5 and not win[:5].any() and not win[21:].any()
    got32 = focusing.focus_rdrgrm(ap.astype(np.complex64), par)
    assert got32.dtype == np.complex64 and rel(got32, g["ap_all"]) < 1e-5


@pytest.mark.gpu
def test_gpu_full_focus_at_center_matches_reference(built_lib, golden):
    from europaraypaths_gb300 import focusing
    m, _, cf, g = golden
    got = focusing.full_focus_at_center(cf, dict(m.CF_PAR))
    assert got.shape == cf.shape and rel(got, g["cf_out"]) < 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("Nr,Na,spacing", [(300, 257, 60.0), (128, 64, 25.0)])
def test_gpu_focus_rdrgrm_vs_oracle_larger(built_lib, Nr, Na, spacing):
    # apertures of ~50 and ~130 traces, windows clipped at both track ends
    import np_focus as nf
    from europaraypaths_gb300 import focusing
    rng = np.random.default_rng(Nr + Na)
    rdr = (rng.standard_normal((Nr, Na)) + 1j * rng.standard_normal((Nr, Na))).astype(np.complex64)
    par = {"rx_window_m": 9000.0, "rx_window_offset_m": 24000.0, "rx_sample_rate": 4e6, "aperture": 3.0,
           "spacing": spacing, "altitude": 25000.0, "eps_1": 1.0, "eps_2": 3.15, "frequency": 9e6}
    st, en = Nr // 3, Nr // 3 + 6
    ref = nf.focus_rdrgrm(rdr.astype(np.complex128), dict(par), st=st, en=en)
    got = focusing.focus_rdrgrm(rdr, dict(par), st=st, en=en)
    assert rel(got, ref) < 1e-5
    assert np.array_equal(focusing.focus_rdrgrm(rdr, dict(par), st=st, en=en, return_shifts=True),
                          nf.focus_rdrgrm(rdr, dict(par), st=st, en=en, return_shifts=True))


@pytest.mark.gpu
def test_gpu_focus_refused_without_root(built_lib):
    # no refraction angle in [0, 20 deg]: the reference's brentq raises; the
    # library reports RP_ERR_ARG with the row
    from europaraypaths_gb300 import _abi, focusing
    rdr = np.ones((16, 8), np.complex64)
    par = {"rx_window_m": 100.0, "rx_window_offset_m": 24000.0, "rx_sample_rate": 4e6, "aperture": 60.0,
           "spacing": 1000.0, "altitude": 25000.0, "eps_1": 1.0, "eps_2": 3.15, "frequency": 9e6}
    with pytest.raises(_abi.RaypathError) as e:
        focusing.focus_rdrgrm(rdr, par)
    assert e.value.rc == -1 and "refraction angle" in str(e.value)
