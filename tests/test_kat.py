"""Known-answer tests: the reference's own validation scenes
(examples/UNIT_TESTS/*/code) at reduced sizes, checked against the analytic
radar equations of their output.py scripts with the reference's error bands.

* fresnel_zone (output.py:32-36, plot band 0-5 %): a flat first-Fresnel-zone
  disk returns P G^2 lam^2 / ((4 pi)^2 h^2).
* image_theory (output.py:18-28, band 0-5 %): an unbounded flat surface
  returns P G^2 lam^2 / ((4 pi)^2 (2h)^2).
* subsurface_target (output.py:13-36): a nadir facet target at depth d
  returns P G^2 lam^4 G_T^2 g_r^4 / ((4 pi)^4 (h+d)^4 n^2) with phase
  angle(exp(-j 4 pi (h + sqrt(eps) d) / lam)).
* subsurface_layer (output.py:32-45, band 0-10 %): a reflector layer of
  targets returns P G^2 lam^2 g_r^2 / ((4 pi)^2 (2(h+d))^2)  (GPU only:
  90,000 targets x 90,000 facets per trace).

The CPU tests run the FP64 oracle; the gpu-marked ones run both GPU forms
through the C ABI on the same scenes.
"""
import contextlib
import io

import numpy as np
import pytest

from europaraypaths_gb300 import param_gen as pg, simple_surfaces as ss, traces as tr_mod


def quiet():
    return contextlib.redirect_stdout(io.StringIO())


def _fresnel(h):
    with quiet():
        dom = {"ox": -1e3, "oy": -1e3, "oz": 0, "fs": 10, "nx": 200, "ny": 200}
        rec = {"rx_window_offset_m": h - 250, "rx_window_m": 0.75e3, "rx_sample_rate": 120e6}
        src = {"sy": 0, "sz": h, "sdx": 10, "sx0": 0, "ns": 1, "aperture": 70}
        prm = pg.gen_params("REASON_VHF", "planetary_ice", dom, rec, src, par={"lossless": True})
    fac = ss.surface_arrays(prm, "fresnel")
    G = 10 ** (prm["surface_gain"] / 10)
    Pr = prm["power"] * G ** 2 * prm["lam"] ** 2 / ((4 * np.pi) ** 2 * h ** 2)
    return prm, fac, np.zeros((7, 0)), Pr


def _image(h):
    with quiet():
        dom = {"ox": -5e3, "oy": -5e3, "oz": 0, "fs": 20, "nx": 500, "ny": 500}
        rec = {"rx_window_m": 0.75e3, "rx_sample_rate": 120e6, "rx_window_offset_m": h - 250}
        src = {"ns": 1, "sx0": 0, "sy": 0, "sz": h, "sdx": 0, "aperture": 70}
        prm = pg.gen_params("REASON_VHF", "planetary_ice", dom, rec, src, par={"lossless": True})
    fac = ss.surface_arrays(prm, "flat")
    G = 10 ** (prm["surface_gain"] / 10)
    Pr = prm["power"] * G ** 2 * prm["lam"] ** 2 / ((4 * np.pi) ** 2 * (2 * h) ** 2)
    return prm, fac, np.zeros((7, 0)), Pr


def _subsurface(h, d):
    with quiet():
        dom = {"ox": -1e3, "oy": -1e3, "oz": 0, "fs": 2.5, "nx": 800, "ny": 800}
        n = np.sqrt(3.15)
        rec = {"rx_window_m": 1.25e3, "rx_sample_rate": 60e6, "rx_window_offset_m": h + d * n - 500}
        src = {"ns": 1, "sx0": 0, "sy": 0, "sz": h, "sdx": 0, "aperture": 70}
        prm = pg.gen_params("REASON_VHF", "planetary_ice", dom, rec, src,
                            par={"lossless": True, "disable_surface": True})
    fac = ss.surface_arrays(prm, "flat")
    tg = np.array([[0.0], [0.0], [-d], [0.0], [0.0], [1.0], [1.0]])
    G = 10 ** (prm["surface_gain"] / 10)
    lam = prm["lam"]
    gr = (h + d) / (h + d / n)
    GT = 4 * np.pi * prm["fs"] ** 2 / lam ** 2
    Pr = prm["power"] * G ** 2 * lam ** 4 * GT ** 2 / ((4 * np.pi) ** 4 * (h + d) ** 4) * gr ** 4 / n ** 2
    phase = np.angle(np.exp(-4j * np.pi / lam * (h + n * d)))
    return prm, fac, tg, Pr, phase


# The reference's plots band these scenes at 0-5 % (power) and the phase is
# compared in degrees.  The oracle's measured errors on the scenes below are
# at most 1.7 % in power (fresnel 0.7-1.2 %, image 0.05-1.5 %, subsurface
# target 0.28-1.7 %) and 4.5 degrees in phase (0.4 degrees at 5 km depth), so
# the bars are tightened to 2.5 % and 6 degrees; the GPU forms agree with the
# oracle to ~1e-7 and are held to the same bars.
POWER_TOL = 2.5
PHASE_TOL = 6.0


def _check_power(out, Pr, tol_pct):
    Pnum = float(np.max(np.abs(out) ** 2))
    err = abs(Pnum - Pr) / Pr * 100
    assert err < tol_pct, f"power error {err:.2f} % (numerical {Pnum:.4e}, analytic {Pr:.4e})"


def _check_phase(out, phase, tol_deg):
    k = int(np.argmax(np.abs(out[0])))
    e = np.degrees(np.angle(out[0, k] * np.exp(-1j * phase)))
    assert abs(e) < tol_deg, f"phase error {e:.2f} deg"


def _oracle_run(oracle, prm, fac, tg):
    p = pg.to_rp_params(prm, derive=False)
    oracle.derive(p)
    out, _ = oracle.simulate(p, fac, tg, tr_mod.linear_track(p, 1))
    return out


@pytest.mark.parametrize("h", [200e3, 50e3])
def test_kat_fresnel_zone_oracle(oracle, h):
    prm, fac, tg, Pr = _fresnel(h)
    _check_power(_oracle_run(oracle, prm, fac, tg), Pr, POWER_TOL)


@pytest.mark.parametrize("h", [100e3, 25e3])
def test_kat_image_theory_oracle(oracle, h):
    prm, fac, tg, Pr = _image(h)
    _check_power(_oracle_run(oracle, prm, fac, tg), Pr, POWER_TOL)


@pytest.mark.parametrize("h,d", [(300e3, 250.0), (19e3, 250.0), (100e3, 5000.0)])
def test_kat_subsurface_target_oracle(oracle, h, d):
    prm, fac, tg, Pr, ph = _subsurface(h, d)
    out = _oracle_run(oracle, prm, fac, tg)
    _check_power(out, Pr, POWER_TOL)
    _check_phase(out, ph, PHASE_TOL)


# ------------------------------------------------------------------ GPU --
def _gpu_run(prm, fac, tg, form):
    from europaraypaths_gb300 import simulator
    with simulator.Scene(prm, fac, tg) as sc:
        return sc.simulate(tr_mod.linear_track(sc.params, 1), form=form)


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["fast", "plain"])
def test_kat_fresnel_and_image_gpu(built_lib, form):
    prm, fac, tg, Pr = _fresnel(125e3)
    _check_power(_gpu_run(prm, fac, tg, form), Pr, POWER_TOL)
    prm, fac, tg, Pr = _image(50e3)
    _check_power(_gpu_run(prm, fac, tg, form), Pr, POWER_TOL)


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["fast", "plain"])
def test_kat_subsurface_target_gpu(built_lib, form):
    for h, d in ((300e3, 250.0), (19e3, 5000.0)):
        prm, fac, tg, Pr, ph = _subsurface(h, d)
        out = _gpu_run(prm, fac, tg, form)
        _check_power(out, Pr, POWER_TOL)
        _check_phase(out, ph, PHASE_TOL)


@pytest.mark.gpu
def test_kat_subsurface_layer_gpu(built_lib):
    """subsurface_layer/code/params.py: vacuum, 20 km deep layer of 300x300
    targets under 300x300 facets of 13.3 m, source at altitude h, receive
    window tracking the layer; P of a mirror at 2(h+d) (output.py:32-45, 72).

    Checked at h = 40 and 20 km, where the 4 km wide layer spans several
    Fresnel radii of the two-way path.  Towards h = 100 km (the top of the
    reference's altitude range) it spans only about two, and the reference's
    model -- in the FP64 plain form as in the fast form -- falls below the
    infinite-layer formula (0.70 of it at h = 100 km)."""
    depth = 20e3
    with quiet():
        dom = {"ox": -2e3, "oy": -2e3, "oz": 0, "fs": 20 / 1.5, "nx": 300, "ny": 300}
        rec = {"rx_window_m": 1.25e3, "rx_sample_rate": 60e6, "rx_window_offset_m": 0}
        src = {"ns": 1, "sx0": 0, "sy": 0, "sz": 100e3, "sdx": 0, "aperture": 70}
        prm = pg.gen_params("REASON_VHF", "vacuum", dom, rec, src,
                            par={"lossless": False, "disable_surface": True})
    fac = ss.surface_arrays(prm, "flat")
    tg = ss.target_arrays(prm, "flat", zoffset=-depth)
    from europaraypaths_gb300 import simulator
    G = 10 ** (prm["surface_gain"] / 10)
    lam = prm["lam"]
    with simulator.Scene(prm, fac, tg) as sc:
        for h in (40e3, 20e3):
            tr = tr_mod.linear_track(sc.params, 1)
            tr[0, 2] = h
            tr[0, 6] = h + depth - 500.0           # track_Z_rxwin(sz, -d sqrt(eps2) + 500), eps2 = 1
            out = sc.simulate(tr, form="fast")
            Pr = prm["power"] * G ** 2 * lam ** 2 / ((4 * np.pi) ** 2 * (2 * (h + depth)) ** 2)
            _check_power(out, Pr, 10.0)
