"""Generate golden fixtures from the reference's own Python entry points.

Runs only where a reference checkout is available: its root is the first
argument or the REFERENCE_ROOT environment variable (there is no default).
The fixtures it writes are committed next to this script and are all the
tests read.

    python tests/golden/make_golden.py <reference checkout root>

Fixtures:
  params_<platform>_<media>.json   gen_params(...) for each preset
  surface_<stype>.fct              make_surface(...) on a small grid
  targets_flat.txt                 make_target_array(..., zoffset=-500)
  source_path.txt, rxwin.txt       vert_source_path / track_Z_rxwin
  rdrgrm.npy (+ rdr/s*.txt)        compile_rdrgrm on synthetic trace files
"""
import contextlib
import io
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
def reference_root():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("REFERENCE_ROOT")
    if not ref:
        sys.exit("usage: make_golden.py <reference checkout root>  (or set REFERENCE_ROOT)")
    return ref


def main():
    REF = reference_root()
    sys.path.insert(0, os.path.join(REF, "src", "PYTHON"))
    import param_gen as pg
    import simple_surfaces as ss
    import output_handling as oh

    quiet = contextlib.redirect_stdout(io.StringIO())
    dom = {"ox": -100.0, "oy": -80.0, "oz": 0, "fs": 10.0, "nx": 12, "ny": 9}
    rec = {"rx_window_m": 1.25e3, "rx_sample_rate": 60e6, "rx_window_offset_m": 9e3}
    src = {"ns": 7, "sx0": -30.0, "sy": 0.0, "sz": 10e3, "sdx": 10.0, "aperture": 10}
    for plat in ("REASON_VHF", "REASON_HF", "1MHz"):
        for media in ("planetary_ice", "vacuum"):
            with quiet:
                p = pg.gen_params(plat, media, dom, rec, src, par={"lossless": True})
            with open(os.path.join(HERE, f"params_{plat}_{media}.json"), "w") as f:
                json.dump(p, f, indent=1, sort_keys=True)
    with quiet:
        p = pg.gen_params("REASON_VHF", "planetary_ice", dom, rec, src)
    p["lam"] = 299792458 / p["frequency"]
    for stype in ("flat", "concave", "fresnel", "fresnel-convex"):
        q = dict(p)
        if stype.startswith("fresnel"):
            q.update({"ox": -60.0, "oy": -60.0, "nx": 13, "ny": 13, "sz": 500.0})
        with quiet:
            ss.make_surface(q, stype, os.path.join(HERE, f"surface_{stype}.fct"))
    with quiet:
        ss.make_target_array(p, "flat", os.path.join(HERE, "targets_flat.txt"), zoffset=-500.0)
    cwd = os.getcwd()
    os.chdir(HERE)
    try:
        sz = pg.vert_source_path({"ns": 5}, 20e3, 10e3, "source_path", direct=".")
        pg.track_Z_rxwin(sz, 250.0, "rxwin", direct=".")
    finally:
        os.chdir(cwd)
    # compile_rdrgrm on synthetic trace files (the format saveSignalToFile writes)
    rdir = os.path.join(HERE, "rdr")
    os.makedirs(rdir, exist_ok=True)
    rng = np.random.default_rng(7)
    for i in range(4):
        z = rng.standard_normal((6, 2))
        with open(os.path.join(rdir, f"s{i:06d}.txt"), "w") as f:
            for re_, im_ in z:
                f.write("%e %e\n" % (re_, im_))
    with quiet:
        r = oh.compile_rdrgrm(rdir, {"ns": 4})
    np.save(os.path.join(HERE, "rdrgrm.npy"), r)


if __name__ == "__main__":
    main()
