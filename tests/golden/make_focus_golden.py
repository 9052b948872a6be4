"""Golden vectors of the reference's azimuth focusing (simple_focusing.py:
full_focus_at_center 115-185, focus_rdrgrm 310-404) on small seeded
radargrams.  Run where the reference sources are present, with the path of
their src/PYTHON directory as the argument (or REFERENCE_ROOT set to the
checkout root); there is no default:

    python tests/golden/make_focus_golden.py <reference checkout>/src/PYTHON

Writes tests/golden/focus_small.npz (parameters and outputs; the input
radargrams are regenerated from their seed by inputs()).  matplotlib is not
installed, so a stub module takes its place (full_focus_at_center only plots
with it).
"""
import os
import sys
import types

import numpy as np


AP_PAR = {"rx_window_m": 3200.0, "rx_window_offset_m": 24000.0, "rx_sample_rate": 4e6, "aperture": 3.0,
          "spacing": 150.0, "altitude": 25000.0, "eps_1": 1.0, "eps_2": 3.15, "frequency": 9e6}
# a point target under trace ns // 2 (the reference trims the slant-range
# curve to centre its minimum and fails otherwise); more than 200 range bins
# (it takes an argmax over rows 200 and on)
CF_PAR = {"sx0": -1600.0, "sdx": 100.0, "ns": 32, "sz": 25000.0, "tx": 0.0, "tz": -800.0, "eps_2": 3.15,
          "rx_sample_rate": 4e6, "rx_window_offset_m": 24000.0, "frequency": 9e6}


def inputs():
    """The seeded input radargrams: (64, 40) for focus_rdrgrm, (216, 32) for
    full_focus_at_center, complex128."""
    rng = np.random.default_rng(11)
    ap = rng.standard_normal((64, 40)) + 1j * rng.standard_normal((64, 40))
    cf = rng.standard_normal((216, 32)) + 1j * rng.standard_normal((216, 32))
    return ap, cf


def main(ref_dir):
    plt = types.ModuleType("matplotlib.pyplot")
    for name in ("plot", "show", "imshow", "axhline", "figure", "title", "legend", "colorbar"):
        setattr(plt, name, lambda *a, **k: None)
    mpl = types.ModuleType("matplotlib")
    mpl.pyplot = plt
    sys.modules["matplotlib"] = mpl
    sys.modules["matplotlib.pyplot"] = plt
    sys.path.insert(0, ref_dir)
    import io
    import contextlib
    import simple_focusing as sf

    rdr, rdr2 = inputs()
    par, par2 = dict(AP_PAR), dict(CF_PAR)
    out = {}
    with contextlib.redirect_stdout(io.StringIO()):
        f_all = sf.focus_rdrgrm(rdr, dict(par))
        f_win = sf.focus_rdrgrm(rdr, dict(par), st=5, en=20)
        shifts = sf.focus_rdrgrm(rdr, dict(par), return_shifts=True)
        mf = sf.focus_rdrgrm(rdr, dict(par), return_match_filter=True)
        f_c = sf.full_focus_at_center(rdr2, dict(par2))
    out.update(ap_all=f_all, ap_win=f_win, ap_shifts=shifts, ap_mf=mf, cf_out=f_c)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "focus_small.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    if len(sys.argv) > 1:
        main(sys.argv[1])
    elif os.environ.get("REFERENCE_ROOT"):
        main(os.path.join(os.environ["REFERENCE_ROOT"], "src", "PYTHON"))
    else:
        sys.exit("usage: make_focus_golden.py <reference checkout>/src/PYTHON  (or set REFERENCE_ROOT)")
