"""Accuracy on the full-size workloads, through the C ABI.

Chain of trust, from the CPU oracle to the benchmarked scene:

1. the plain FP64 GPU form against the FP64 CPU oracle on every trace of
   the small plain scene (200x200 facets, 1600 targets, 100 traces at
   25 km), at <= 1e-10 relative L2 -- and the fast form against the same
   oracle output at the fast form's bar;
2. both forms against the oracle on the large scene's 4M facets, with a
   target subset the oracle finishes in seconds, on every 125th trace of
   the 2000 (16 traces);
3. the fast form against the plain FP64 form on the benchmarked large scene
   itself -- all 4M facets and all 40k targets -- on four interior traces.

The fast form's bar: relative L2 <= 1e-3 of the complex radargram (whole and
per trace), phase error <= 0.01 rad at bins above -40 dB of each trace's
peak, every trace's peak range bin exact, and the illuminated-facet and
in-aperture-target counts exact.  Each test prints its figures as one JSON
line (``pytest -s`` shows them).
"""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PLAIN_REL = 1e-10


def _report(name, **kv):
    print(json.dumps({"test": name, **kv}, default=float), flush=True)


def _check_fast(res):
    from europaraypaths_gb300 import accuracy
    assert res["rel_l2"] <= accuracy.REL_L2_BAR, res
    assert accuracy.within_bar(res), res


@pytest.fixture(scope="module")
def large():
    from europaraypaths_gb300 import scenes
    return scenes.large_scene()


def test_small_plain_scene_every_trace(built_lib, oracle):
    from europaraypaths_gb300 import accuracy, scenes, simulator
    sc = scenes.small_plain()
    with simulator.Scene(sc["params"], sc["facets"], sc["targets"]) as scene:
        tr = scene.default_traces()
        assert tr.shape[0] == 100
        ref, rcnt = oracle.simulate(scene.params, sc["facets"], sc["targets"], tr)
        plain, pcnt = scene.simulate(tr, form="plain", complex128=True, return_counts=True)
        fast, fcnt = scene.simulate(tr, form="fast", return_counts=True)
    assert np.array_equal(pcnt, rcnt) and np.array_equal(fcnt, rcnt)
    assert (rcnt[:, 0] == 40000).all() and (rcnt[:, 1] == 1600).all()
    rp = accuracy.rel_l2(plain, ref)
    rf = accuracy.compare(fast, ref)
    _report("small_plain_every_trace", plain_rel_l2=rp, fast=rf)
    assert rp <= PLAIN_REL, rp
    _check_fast(rf)


def test_large_scene_facets_target_subset_vs_oracle(built_lib, oracle, large):
    # the large scene's 4M facets with the targets of the three rows nearest
    # the track (|y| <= 75 m), every 8th along it: ~40 in the aperture of an
    # interior trace, so the FP64 oracle runs 16 traces in seconds
    from europaraypaths_gb300 import accuracy, simulator
    tg = large["targets"]
    xi = np.rint((tg[0] - tg[0].min()) / 50.0).astype(int)
    sub = tg[:, (np.abs(tg[1]) <= 75.0) & (xi % 8 == 0)]
    assert sub.shape[1] == 75
    with simulator.Scene(large["params"], large["facets"], sub) as scene:
        tr = scene.default_traces()[::125]
        assert tr.shape[0] == 16
        ref, rcnt = oracle.simulate(scene.params, large["facets"], sub, tr)
        plain, pcnt = scene.simulate(tr, form="plain", complex128=True, return_counts=True)
        fast, fcnt = scene.simulate(tr, form="fast", return_counts=True)
    assert np.array_equal(pcnt, rcnt) and np.array_equal(fcnt, rcnt)
    assert rcnt[8, 0] > 800000 and rcnt[8, 1] > 30       # trace 1000: interior
    rp = accuracy.rel_l2(plain, ref)
    rf = accuracy.compare(fast, ref)
    _report("large_scene_target_subset_vs_oracle", counts=rcnt.tolist(), plain_rel_l2=rp, fast=rf)
    assert rp <= PLAIN_REL, rp
    _check_fast(rf)


def test_large_scene_fast_vs_plain_interior_traces(built_lib, large):
    # the benchmarked scene in full: 4M facets, 40k targets (~9,100 in the
    # aperture of an interior trace, 1.58e10 pairs per trace)
    from europaraypaths_gb300 import accuracy, simulator
    with simulator.Scene(large["params"], large["facets"], large["targets"]) as scene:
        tr = scene.default_traces()[[500, 833, 1166, 1499]]
        fast, fcnt = scene.simulate(tr, form="fast", return_counts=True)
        plain, pcnt = scene.simulate(tr, form="plain", complex128=True, return_counts=True)
    assert np.array_equal(fcnt, pcnt)
    assert (pcnt[:, 0] > 850000).all() and (pcnt[:, 1] > 9000).all()
    rf = accuracy.compare(fast, plain)
    per = [accuracy.compare(fast[i], plain[i]) for i in range(tr.shape[0])]
    _report("large_scene_fast_vs_plain", counts=pcnt.tolist(), fast=rf,
            per_trace=[{"rel_l2": r["rel_l2"], "phase_max_rad": r["phase_max_rad"]} for r in per])
    _check_fast(rf)
