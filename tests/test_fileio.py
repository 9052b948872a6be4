"""The reference's text formats through the library's C parsers and writer
(no GPU work): facets, targets (3/4/6/7 columns), sources, gains, receive
window, prisms, trace output and directory handling."""
import contextlib
import io
import os

import numpy as np
import pytest

from europaraypaths_gb300 import _abi, fileio, param_gen as pg, simple_surfaces as ss
from helpers import tiny_scene

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_read_facets_golden(built_lib):
    f = fileio.read_facets(os.path.join(G, "surface_concave.fct"))
    dom = {"ox": -100.0, "oy": -80.0, "oz": 0, "fs": 10.0, "nx": 12, "ny": 9, "sz": 10e3}
    ref = ss.surface_arrays(dom, "concave")
    assert f.shape == (12, 108)
    assert np.allclose(f, ref, atol=5e-7)


def test_read_targets_golden_and_column_variants(built_lib, tmp_path):
    t = fileio.read_targets(os.path.join(G, "targets_flat.txt"))
    assert t.shape == (7, 108) and np.all(t[6] == 1) and np.allclose(t[2], -500.0)
    p = tmp_path / "t.txt"
    p.write_text("1,2,3\n4,5,6,7\n1,1,1,0.1,0.2,0.97\n0,0,-1500,0,0,1,1\n")
    t = fileio.read_targets(str(p))
    assert t.shape == (7, 4)
    assert list(t[:, 0]) == [1, 2, 3, 0, 0, 1, 0]            # 3 columns: +z normal, ttype 0
    assert list(t[:, 1]) == [4, 5, 6, 0, 0, 1, 7]            # 4 columns: ttype
    assert np.allclose(t[:, 2], [1, 1, 1, 0.1, 0.2, 0.97, 0])
    assert list(t[:, 3]) == [0, 0, -1500, 0, 0, 1, 1]
    p.write_text("1,2\n")
    with pytest.raises(_abi.RaypathError) as e:
        fileio.read_targets(str(p))
    assert e.value.rc == -3 and "incorrect number of entries" in str(e.value)


def test_read_sources_rx_gains(built_lib, tmp_path):
    s = fileio.read_sources(os.path.join(G, "source_path.txt"))
    assert s.shape == (5, 6) and np.allclose(s[:, 2], np.linspace(20e3, 10e3, 5)) and np.all(s[:, 5] == 1)
    rx = fileio.read_rx_window(os.path.join(G, "rxwin.txt"), 5)
    assert np.allclose(rx, np.linspace(20e3, 10e3, 5) - 250.0)
    with pytest.raises(_abi.RaypathError) as e:
        fileio.read_rx_window(os.path.join(G, "rxwin.txt"), 4)
    assert "MORE entries" in str(e.value)
    with pytest.raises(_abi.RaypathError) as e:
        fileio.read_rx_window(os.path.join(G, "rxwin.txt"), 6)
    assert "expected exactly 6" in str(e.value)
    g = tmp_path / "g.txt"
    g.write_text("7.3,7.3\n\n6.0,5.5\n")
    assert np.allclose(fileio.read_gains(str(g)), [[7.3, 7.3], [6.0, 5.5]])


def test_read_prisms_alpha(built_lib, tmp_path):
    from oracle import np_oracle
    sc = tiny_scene()
    p = pg.to_rp_params(sc["params"])
    f = tmp_path / "prisms.txt"
    f.write_text("1e-05,-5000.0,-2500.0,-500.0,-1000.0,2500.0,0\n2e-05,1000.0,-2500.0,-500.0,5000.0,2500.0,0\n")
    pr = fileio.read_prisms(str(f), p)
    pd = np_oracle.derive(sc["params"])
    assert pr.shape == (7, 2)
    assert abs(pr[0, 0] - np_oracle.prism_alpha(1e-5, pd)) < 1e-15
    assert list(pr[1:, 1]) == [1000.0, -2500.0, -500.0, 5000.0, 2500.0, 0.0]


def test_write_trace_format_and_clear(built_lib, tmp_path):
    col = np.array([1.5 - 2.25j, -3.0e-9 + 4.0e-12j], np.complex64)
    f = tmp_path / "s000000.txt"
    fileio.write_trace(str(f), col)
    assert f.read_text() == "%e %e\n%e %e\n" % (1.5, -2.25, np.float32(-3.0e-9), np.float32(4.0e-12))
    (tmp_path / "s000001.txt").write_text("x")
    (tmp_path / "keep.txt").write_text("x")
    assert fileio.clear_traces(str(tmp_path)) == 2
    assert os.listdir(tmp_path) == ["keep.txt"]
    with pytest.raises(_abi.RaypathError):
        fileio.check_directory(str(tmp_path / "keep.txt"))
    with pytest.raises(_abi.RaypathError):
        fileio.read_facets(str(tmp_path / "missing.fct"))


def test_cli_input_loading(built_lib, tmp_path):
    """sim.load_inputs builds the same trace table the reference's main() does."""
    from europaraypaths_gb300 import sim, traces as tr_mod
    with contextlib.redirect_stdout(io.StringIO()):
        prm = pg.gen_params("REASON_HF", "planetary_ice",
                            {"ox": -100.0, "oy": -100.0, "oz": 0, "fs": 10.0, "nx": 20, "ny": 20},
                            {"rx_window_m": 1.25e3, "rx_sample_rate": 60e6, "rx_window_offset_m": 9e3},
                            {"ns": 4, "sx0": -20.0, "sy": 0.0, "sz": 10e3, "sdx": 10.0, "aperture": 10})
    prm["source_normal_multiplier"] = 1.0
    d = str(tmp_path)
    pg.export_params(prm, "params", directory=d)
    with contextlib.redirect_stdout(io.StringIO()):
        ss.make_surface(prm, "flat", os.path.join(d, "f.fct"))
        ss.make_target_array(prm, "flat", os.path.join(d, "t.txt"), zoffset=-300.0)
    p, facets, targets, prisms, tr = sim.load_inputs(os.path.join(d, "params.json"), os.path.join(d, "f.fct"),
                                                     os.path.join(d, "t.txt"))
    assert facets.shape == (12, 400) and targets.shape == (7, 400) and prisms is None
    assert np.allclose(tr, tr_mod.linear_track(p))


def test_binary_store_round_trip_and_kind(built_lib, tmp_path):
    sc = tiny_scene()
    fp, tp, xp = str(tmp_path / "f.rpf"), str(tmp_path / "t.rpt"), str(tmp_path / "x.txt")
    fileio.write_store(fp, sc["facets"], fileio.STORE_FACETS)
    fileio.write_store(tp, sc["targets"], fileio.STORE_TARGETS)
    open(xp, "w").write("1,2,3\n")
    assert [fileio.store_kind(p) for p in (fp, tp, xp)] == [0, 1, -1]
    assert os.path.getsize(fp) == 32 + 8 * sc["facets"].size
    with fileio.MappedStore(fp, fileio.STORE_FACETS) as m:
        assert m.soa.shape == sc["facets"].shape and not m.soa.flags.writeable
        assert np.array_equal(m.soa, sc["facets"])
    assert np.array_equal(fileio.load_targets(tp), sc["targets"])
    assert np.array_equal(fileio.load_targets(xp), fileio.read_targets(xp))


def test_text_to_store_conversion_is_exact(built_lib, tmp_path):
    txt = os.path.join(G, "surface_concave.fct")
    dst = str(tmp_path / "c.rpf")
    assert fileio.main([txt, dst]) == 0
    assert np.array_equal(fileio.load_facets(dst), fileio.read_facets(txt))
    tdst = str(tmp_path / "c.rpt")
    assert fileio.main([os.path.join(G, "targets_flat.txt"), tdst, "--kind", "targets"]) == 0
    assert np.array_equal(fileio.load_targets(tdst), fileio.read_targets(os.path.join(G, "targets_flat.txt")))


def test_binary_store_errors(built_lib, tmp_path):
    sc = tiny_scene()
    fp = str(tmp_path / "f.rpf")
    fileio.write_store(fp, sc["facets"], fileio.STORE_FACETS)
    with pytest.raises(_abi.RaypathError) as e:          # a facet store is not a target store
        fileio.MappedStore(fp, fileio.STORE_TARGETS)
    assert e.value.rc == -3
    data = open(fp, "rb").read()
    open(fp, "wb").write(data[:-8])                       # truncated
    with pytest.raises(_abi.RaypathError) as e:
        fileio.MappedStore(fp, fileio.STORE_FACETS)
    assert e.value.rc == -3 and "file size" in str(e.value)
    with pytest.raises(_abi.RaypathError) as e:
        fileio.MappedStore(str(tmp_path / "missing.rpf"), fileio.STORE_FACETS)
    assert e.value.rc == -2


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_radargram_file_round_trip(built_lib, tmp_path, dtype):
    rng = np.random.default_rng(4)
    rdr = (rng.standard_normal((5, 33)) + 1j * rng.standard_normal((5, 33))).astype(dtype)
    p = str(tmp_path / "r.rdr")
    fileio.write_radargram(p, rdr)
    assert fileio.store_kind(p) == fileio.STORE_RADARGRAM
    got = fileio.read_radargram(p)
    assert got.dtype == dtype and np.array_equal(got, rdr)
    empty = str(tmp_path / "e.rdr")
    fileio.write_radargram(empty, np.zeros((0, 8), np.complex64))
    assert fileio.read_radargram(empty).shape == (0, 8)
