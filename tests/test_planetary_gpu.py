"""Planetary-scale coordinates: the fast form at Mars-radius offsets.

Orbit geometry in a body-centred frame puts the surface about 3.39e6 m from
the origin (the reference's Mars example writes its source path that way).
The fast form keeps FP64 only for the spacecraft and trace-level anchors and
evaluates every pair as an FP32 offset from them, so a scene moved far from
the origin must give the same radargram.  The same scene, facets, targets
and track translated by 3.39e6 m (along x, and along z as on top of a planet)
is compared with the FP64 CPU oracle at the fast form's bar, at 9 MHz
(2048 bins) and 60 MHz (4096 bins), and with the untranslated fast result.
"""
import json

import numpy as np
import pytest

from helpers import tiny_scene, vhf_scene

pytestmark = pytest.mark.gpu

R_MARS = 3.3895e6


def _translate(sc, v):
    out = dict(sc)
    v = np.asarray(v, np.float64)
    out["facets"] = sc["facets"].copy()
    out["facets"][0:3] += v[:, None]
    out["targets"] = sc["targets"].copy()
    out["targets"][0:3] += v[:, None]
    return out


@pytest.mark.parametrize("band", ["9MHz", "60MHz"])
@pytest.mark.parametrize("axis", ["x", "z"])
def test_fast_form_at_planetary_offsets(built_lib, oracle, band, axis):
    from europaraypaths_gb300 import accuracy, simulator
    if band == "9MHz":
        sc = tiny_scene(nside=60, ntside=4, ns=3)
    else:
        sc = vhf_scene(4096, n_side=120, nt_side=4, ns=3)
    v = np.array([R_MARS, 0.0, 0.0]) if axis == "x" else np.array([0.0, 0.0, R_MARS])
    moved = _translate(sc, v)
    with simulator.Scene(sc["params"], sc["facets"], sc["targets"]) as scene:
        tr = scene.default_traces()
        home = scene.simulate(tr, form="fast")
    tr_m = tr.copy()
    tr_m[:, 0:3] += v
    with simulator.Scene(moved["params"], moved["facets"], moved["targets"]) as scene:
        got, cnt = scene.simulate(tr_m, form="fast", return_counts=True)
        ref, rcnt = oracle.simulate(scene.params, moved["facets"], moved["targets"], tr_m)
    assert np.array_equal(cnt, rcnt) and cnt[:, 0].min() > 0 and cnt[:, 1].min() > 0
    res = accuracy.compare(got, ref)
    moved_vs_home = accuracy.rel_l2(got, home)
    print(json.dumps({"test": f"planetary_{band}_{axis}", "vs_oracle": res, "vs_untranslated": moved_vs_home}))
    assert accuracy.within_bar(res), res
    assert res["rel_l2"] <= accuracy.REL_L2_BAR
    assert moved_vs_home <= accuracy.REL_L2_BAR, moved_vs_home
