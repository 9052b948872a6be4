"""The Python entry points reproduce the reference's own outputs byte for byte
(fixtures generated by tests/golden/make_golden.py from the reference's
src/PYTHON modules)."""
import contextlib
import io
import json
import os

import numpy as np
import pytest

from europaraypaths_gb300 import output_handling as oh
from europaraypaths_gb300 import param_gen as pg
from europaraypaths_gb300 import simple_surfaces as ss

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DOM = {"ox": -100.0, "oy": -80.0, "oz": 0, "fs": 10.0, "nx": 12, "ny": 9}
REC = {"rx_window_m": 1.25e3, "rx_sample_rate": 60e6, "rx_window_offset_m": 9e3}
SRC = {"ns": 7, "sx0": -30.0, "sy": 0.0, "sz": 10e3, "sdx": 10.0, "aperture": 10}


def quiet():
    return contextlib.redirect_stdout(io.StringIO())


@pytest.mark.parametrize("plat", ["REASON_VHF", "REASON_HF", "1MHz"])
@pytest.mark.parametrize("media", ["planetary_ice", "vacuum"])
def test_gen_params_matches_reference(plat, media):
    with quiet():
        p = pg.gen_params(plat, media, DOM, REC, SRC, par={"lossless": True})
    with open(os.path.join(G, f"params_{plat}_{media}.json")) as f:
        ref = json.load(f)
    assert json.loads(json.dumps(p, sort_keys=True)) == ref


def test_gen_params_errors():
    with pytest.raises(ValueError):
        pg.gen_params("NOPE", "vacuum", DOM, REC, SRC)
    with pytest.raises(ValueError):
        pg.gen_params("REASON_HF", "nope", DOM, REC, SRC)
    with pytest.raises(ValueError):
        pg.gen_params("REASON_HF", "vacuum", {"ox": 0}, REC, SRC)
    with pytest.raises(ValueError):
        pg.gen_params("REASON_HF", "vacuum", DOM, {"rx_window_m": 1, "rx_sample_rate": 1}, SRC)


@pytest.mark.parametrize("stype", ["flat", "concave", "fresnel", "fresnel-convex"])
def test_make_surface_matches_reference(stype, tmp_path):
    with quiet():
        p = pg.gen_params("REASON_VHF", "planetary_ice", DOM, REC, SRC)
    p["lam"] = 299792458 / p["frequency"]
    if stype.startswith("fresnel"):
        p.update({"ox": -60.0, "oy": -60.0, "nx": 13, "ny": 13, "sz": 500.0})
    out = tmp_path / "s.fct"
    with quiet():
        ss.make_surface(p, stype, str(out))
    assert out.read_bytes() == open(os.path.join(G, f"surface_{stype}.fct"), "rb").read()


def test_make_target_array_matches_reference(tmp_path):
    with quiet():
        p = pg.gen_params("REASON_VHF", "planetary_ice", DOM, REC, SRC)
        out = tmp_path / "t.txt"
        ss.make_target_array(p, "flat", str(out), zoffset=-500.0)
    assert out.read_bytes() == open(os.path.join(G, "targets_flat.txt"), "rb").read()


def test_source_path_and_rx_window_files(tmp_path):
    sz = pg.vert_source_path({"ns": 5}, 20e3, 10e3, "source_path", direct=str(tmp_path))
    pg.track_Z_rxwin(sz, 250.0, "rxwin", direct=str(tmp_path))
    for name in ("source_path.txt", "rxwin.txt"):
        assert (tmp_path / name).read_bytes() == open(os.path.join(G, name), "rb").read()


def test_compile_rdrgrm_matches_reference():
    with quiet():
        r = oh.compile_rdrgrm(os.path.join(G, "rdr"), {"ns": 4})
    assert np.array_equal(r, np.load(os.path.join(G, "rdrgrm.npy")))


def test_compile_rdrgrm_empty_dir(tmp_path):
    with pytest.raises(ValueError):
        oh.compile_rdrgrm(str(tmp_path), {"ns": 1})


def test_surface_arrays_match_file_writer(tmp_path):
    with quiet():
        p = pg.gen_params("REASON_VHF", "planetary_ice", DOM, REC, SRC)
    soa = ss.surface_arrays(p, "concave")
    rows = [list(map(float, ln.replace(":", ",").split(","))) for ln in
            open(os.path.join(G, "surface_concave.fct")).read().splitlines()]
    assert np.allclose(np.array(rows).T, soa, atol=5e-7)
