"""ttype-0 targets in the fused FP32 form vs the FP64 CPU oracle: the
genRefrPhasor path (sim.cu:940-966; radar_kernels.cu:351-448) that the
reference takes for every target of a 3- or 6-column target file, in the
default mode and in specular mode, alone or mixed with ttype-1 targets.

Tolerances are the fast form's: relative L2 <= 1e-3 of the complex
radargram, max phase error <= 0.01 rad at bins above -40 dB of the peak, an
exact match of every trace's peak range bin, and relative L2 <= 1e-3 of the
target contribution alone (the radargram minus the surface-only radargram).
"""
import os

import numpy as np
import pytest

from helpers import rel_l2, tiny_scene
from test_specular_fast_gpu import _bits, _run, check_targets

pytestmark = pytest.mark.gpu


def _t0(sc, every=1, **over):
    sc["targets"][6, ::every] = 0.0
    sc["params"].update(over)
    return sc


def test_fast_ttype0_all_targets(built_lib, oracle):
    check_targets(_t0(tiny_scene()), oracle)


def test_fast_ttype0_mixed_with_ttype1(built_lib, oracle):
    check_targets(_t0(tiny_scene(), every=2), oracle)


def test_fast_ttype0_specular_mixed(built_lib, oracle):
    check_targets(_t0(tiny_scene(), every=2, specular=True), oracle)


def test_fast_ttype0_small_scene_subset(built_lib, oracle):
    from europaraypaths_gb300 import scenes, traces as tr_mod, param_gen
    sc = _t0(scenes.small_plain(), every=3)
    tr = tr_mod.linear_track(param_gen.to_rp_params(sc["params"]))[[0, 50, 99]]
    check_targets(sc, oracle, traces=tr)


@pytest.mark.parametrize("rf", [3, 4])
def test_fast_ttype0_rerad_functions(built_lib, oracle, rf):
    # rerad_funct 3 keeps every angle below 3 * 180 / pi_F radians (the
    # reference's unit slip), 4 is a 1-degree Gaussian of TargetTh
    check_targets(_t0(tiny_scene(), rerad_funct=rf), oracle)


def test_fast_ttype0_rerad_threshold(built_lib, oracle):
    # rerad_funct 1 keeps TargetTh below 1 degree: a step in the angle, taken
    # here on cos(TargetTh) in FP32 against the oracle's FP64 acos, so a pair
    # within ~1e-5 rad of the step may fall on the other side; the target
    # contribution is compared at 1e-2
    sc = _t0(tiny_scene(nside=40, ntside=6), rerad_funct=1)
    got, ref, cnt, rcnt = _run(sc, oracle, complex128=True)
    assert np.array_equal(cnt, rcnt)
    got0, ref0, _, _ = _run(sc, oracle, targets=np.zeros((7, 0)), complex128=True)
    dg, dr = got - got0, ref - ref0
    assert np.abs(dr).max() > 0
    assert rel_l2(dg, dr) <= 1e-2, rel_l2(dg, dr)


def test_fast_ttype0_prisms(built_lib, oracle):
    prisms = np.array([[2e-3], [-500.0], [-500.0], [-1200.0], [300.0], [400.0], [-100.0]])
    check_targets(_t0(tiny_scene(), every=2), oracle, prisms=prisms)


def test_fast_ttype0_ignores_lossless(built_lib, oracle):
    # lossless drops fEI/fEO for ttype-1 targets only; genRefrPhasor applies them
    check_targets(_t0(tiny_scene(), every=2, lossless=True), oracle)


def test_fast_ttype0_non_pow2_bins(built_lib, oracle):
    from europaraypaths_gb300 import scenes
    sc = _t0(tiny_scene(rx_window_m=scenes.rx_window_for_bins(250, 4e6), rx_window_offset_m=24000.0), every=2)
    got, ref = check_targets(sc, oracle)
    assert got.shape[1] == 250


def test_fast_ttype0_vhf_band(built_lib, oracle):
    from helpers import vhf_scene
    sc = vhf_scene(8192)
    sc["targets"][6, ::2] = 0.0
    got, ref = check_targets(sc, oracle)
    assert got.shape[1] == 8192


def test_fast_ttype0_configurations_and_batching_bitwise(built_lib):
    # the ttype-1 kernel's configurations and batched calls leave every
    # radargram bitwise unchanged
    from europaraypaths_gb300 import simulator, traces as tr_mod
    s = _t0(tiny_scene(nside=40, ntside=4, ns=3), every=2)
    outs = []
    simulator.autotune(False)
    try:
        for cfg in range(4):
            os.environ["RP_PAIR_CFG"] = str(cfg)
            with simulator.Scene(s["params"], s["facets"], s["targets"]) as sc:
                outs.append(sc.simulate(form="fast"))
    finally:
        os.environ.pop("RP_PAIR_CFG", None)
        simulator.autotune(True)
    for o in outs[1:]:
        assert np.array_equal(_bits(o), _bits(outs[0]))
    other = tiny_scene(nside=24, ntside=3, ns=2)
    scenes = [simulator.Scene(x["params"], x["facets"], x["targets"]) for x in (other, s)]
    try:
        trs = [tr_mod.linear_track(sc.params) for sc in scenes]
        single = [sc.simulate(tr, form="fast") for sc, tr in zip(scenes, trs)]
        for a, b in zip(single, simulator.simulate_batch(list(zip(scenes, trs)))):
            assert np.array_equal(_bits(a), _bits(b))
    finally:
        for sc in scenes:
            sc.close()


def test_sim_auto_picks_fast_form_for_ttype0(built_lib):
    from europaraypaths_gb300 import param_gen, sim
    sc = _t0(tiny_scene(nside=12, ntside=2, ns=1))
    p = param_gen.to_rp_params(sc["params"])
    assert sim.pick_form(p, sc["targets"]) == "fast"
    sc["params"]["specular"] = True
    sc["params"]["convolution_linear"] = False       # circular convolution
    assert sim.pick_form(param_gen.to_rp_params(sc["params"]), sc["targets"]) == "fast"
    sc["params"]["convolution"] = False              # direct sums
    assert sim.pick_form(param_gen.to_rp_params(sc["params"]), sc["targets"]) == "fast"
