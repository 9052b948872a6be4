"""The sim-compatible CLI end to end: reference-format input files in,
outdir/s%06d.txt out, read back with compile_rdrgrm and compared with the FP64
oracle run on the same parsed inputs."""
import contextlib
import io
import os

import numpy as np
import pytest

from europaraypaths_gb300 import param_gen as pg, simple_surfaces as ss, output_handling as oh
from helpers import rel_l2

pytestmark = pytest.mark.gpu


def _scene_files(d, with_files=False):
    q = contextlib.redirect_stdout(io.StringIO())
    dom = {"ox": -1e3, "oy": -1e3, "oz": 0, "fs": 50.0, "nx": 40, "ny": 40}
    rec = {"rx_window_m": 153534.0, "rx_sample_rate": 4e6, "rx_window_offset_m": 24e3}
    src = {"ns": 4, "sx0": -75.0, "sy": 0.0, "sz": 25e3, "sdx": 50.0, "aperture": 10}
    with q:
        prm = pg.gen_params("REASON_HF", "planetary_ice", dom, rec, src, par={"rerad_funct": 1})
    if with_files:
        sp = os.path.join(d, "source_path.txt")
        with open(sp, "w") as f:
            for k in range(4):
                f.write(f"{-75.0 + 50 * k},0.0,{25e3 - 100 * k}\n")
        prm["source_path_file"] = sp
        rx = os.path.join(d, "rx.txt")
        with open(rx, "w") as f:
            for k in range(4):
                f.write(f"{24e3 - 100 * k}\n")
        prm["rx_window_position_file"] = rx
        gf = os.path.join(d, "gain.txt")
        with open(gf, "w") as f:
            for k in range(4):
                f.write(f"{4.0 + k},{4.0 - k}\n")
        prm["gain_pattern_file"] = gf
        prm["altitude"] = 25e3
    pg.export_params(prm, "params", directory=d)
    with q:
        ss.make_surface(prm, "flat", os.path.join(d, "facets.fct"))
        tdom = dict(prm, fs=200.0, nx=10, ny=10)
        ss.make_target_array(tdom, "flat", os.path.join(d, "targets.txt"), zoffset=-800.0)
    return prm


@pytest.mark.parametrize("with_files,form,tol", [(False, "fast", 1e-3), (True, "fast", 1e-3),
                                                  (False, "plain", 1e-5)])
def test_cli_matches_oracle(built_lib, oracle, tmp_path, with_files, form, tol):
    from europaraypaths_gb300 import sim
    d = str(tmp_path)
    out = os.path.join(d, "rdrgrm")
    os.makedirs(out)
    with open(os.path.join(out, "s999999.txt"), "w") as f:
        f.write("stale")
    _scene_files(d, with_files)
    args = [os.path.join(d, "params.json"), os.path.join(d, "facets.fct"), os.path.join(d, "targets.txt")]
    with contextlib.redirect_stdout(io.StringIO()):
        n = sim.run(*args, out, form=form)
    assert n == 4 and not os.path.exists(os.path.join(out, "s999999.txt"))
    with contextlib.redirect_stdout(io.StringIO()):
        rdr = oh.compile_rdrgrm(out, {"ns": 4})
    p, facets, targets, prisms, tr = sim.load_inputs(*args)
    ref, _ = oracle.simulate(p, facets, targets, tr)
    # files carry 7 significant digits ("%e")
    assert rel_l2(rdr.T, ref) < tol


def test_cli_main_errors(built_lib, tmp_path):
    from europaraypaths_gb300 import sim
    with contextlib.redirect_stderr(io.StringIO()):
        assert sim.main([str(tmp_path / "nope.json"), "f", "t", str(tmp_path)]) == 1
        assert sim.main(["p", "f", "t", str(tmp_path / "missing_dir")]) == 1


def test_cli_binary_stores_and_radargram_file(built_lib, tmp_path):
    # the same run from binary stores into one radargram file gives the
    # traces the text path writes (to their 7 significant digits)
    from europaraypaths_gb300 import fileio, sim
    d = str(tmp_path)
    _scene_files(d)
    txt = os.path.join(d, "txt")
    os.makedirs(txt)
    args = [os.path.join(d, "params.json"), os.path.join(d, "facets.fct"), os.path.join(d, "targets.txt")]
    with contextlib.redirect_stdout(io.StringIO()):
        sim.run(*args, txt, form="fast")
        rdr_txt = oh.compile_rdrgrm(txt, {"ns": 4})
    assert fileio.main([args[1], os.path.join(d, "facets.rpf")]) == 0
    assert fileio.main([args[2], os.path.join(d, "targets.rpt"), "--kind", "targets"]) == 0
    rfile = os.path.join(d, "all.rdr")
    with contextlib.redirect_stdout(io.StringIO()):
        n = sim.run(args[0], os.path.join(d, "facets.rpf"), os.path.join(d, "targets.rpt"), d, form="fast",
                    radargram=rfile)
    assert n == 4
    rdr = fileio.read_radargram(rfile)
    assert rdr.shape == (4, rdr_txt.shape[0]) and rdr.dtype == np.complex64
    assert rel_l2(rdr, rdr_txt.T) < 1e-6
