"""Specular mode with linear convolution in the fused FP32 form vs the FP64
CPU oracle (sim.cu:733-986 with specular=true, convolution_linear=true):
genReflPhasor's one-bin surface phasor of the specular energy, the
facetReradiation factors of both refraction legs (binned as separate traces),
and the surface chirp for the targets.

Tolerances are the fast form's: relative L2 <= 1e-3 of the complex
radargram, max phase error <= 0.01 rad at bins above -40 dB of the peak, and
an exact match of every trace's peak range bin.  The target legs are also
checked on their own (the radargram minus the same scene's surface-only
radargram), so a strong specular surface cannot hide them.
"""
import os

import numpy as np
import pytest

from helpers import peak_bins, phase_err_max, rel_l2, tiny_scene

pytestmark = pytest.mark.gpu

REL_L2 = 1e-3
PHASE = 0.01


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _spec(sc, **over):
    sc["params"].update({"specular": True, "rerad_funct": 0})
    sc["params"].update(over)
    return sc


def _run(sc, oracle, traces=None, prisms=None, targets=None, complex128=False):
    from europaraypaths_gb300 import simulator, traces as tr_mod
    tg = sc["targets"] if targets is None else targets
    scene = simulator.Scene(sc["params"], sc["facets"], tg, prisms=prisms)
    tr = tr_mod.linear_track(scene.params) if traces is None else traces
    got, cnt = scene.simulate(tr, form="fast", complex128=complex128, return_counts=True)
    ref, rcnt = oracle.simulate(scene.params, sc["facets"], tg, tr, prisms_soa=prisms)
    scene.close()
    return got, ref, cnt, rcnt


def check(got, ref):
    assert np.abs(ref).max() > 0
    assert rel_l2(got, ref) <= REL_L2, rel_l2(got, ref)
    assert phase_err_max(got, ref) <= PHASE, phase_err_max(got, ref)
    assert np.array_equal(peak_bins(got), peak_bins(ref))


def check_targets(sc, oracle, traces=None, prisms=None):
    """The whole radargram and the target legs alone against the oracle.  The
    target part is the difference of two complex128 radargrams (the fast
    form's final sum is FP64 and its surface part is the same bits in both
    runs), so targets far weaker than the surface keep their precision."""
    got, ref, cnt, rcnt = _run(sc, oracle, traces=traces, prisms=prisms)
    assert np.array_equal(cnt, rcnt)
    check(got, ref)
    empty = np.zeros((7, 0))
    g1, _, _, _ = _run(sc, oracle, traces=traces, prisms=prisms, complex128=True)
    got0, ref0, _, _ = _run(sc, oracle, traces=traces, prisms=prisms, targets=empty, complex128=True)
    dg, dr = g1 - got0, ref - ref0
    assert np.abs(dr).max() > 0
    assert rel_l2(dg, dr) <= REL_L2, rel_l2(dg, dr)
    return got, ref


def test_fast_specular_matches_oracle_tiny(built_lib, oracle):
    check_targets(_spec(tiny_scene()), oracle)


def test_fast_specular_small_scene_subset(built_lib, oracle):
    from europaraypaths_gb300 import scenes, traces as tr_mod, param_gen
    sc = _spec(scenes.small_plain())
    tr = tr_mod.linear_track(param_gen.to_rp_params(sc["params"]))[[0, 50, 99]]
    check_targets(sc, oracle, traces=tr)


def test_fast_specular_prisms(built_lib, oracle):
    prisms = np.array([[2e-3], [-500.0], [-500.0], [-1200.0], [300.0], [400.0], [-100.0]])
    check_targets(_spec(tiny_scene()), oracle, prisms=prisms)


def test_fast_specular_lossless(built_lib, oracle):
    # lossless drops compRefrEnergyIn/Out's factors, reradiation included
    check_targets(_spec(tiny_scene(), lossless=True), oracle)


def test_fast_specular_non_pow2_bins(built_lib, oracle):
    # nr = 250: the Bluestein compression kernel with the outbound trace
    from europaraypaths_gb300 import scenes
    sc = _spec(tiny_scene(rx_window_m=scenes.rx_window_for_bins(250, 4e6), rx_window_offset_m=24000.0))
    got, ref = check_targets(sc, oracle)
    assert got.shape[1] == 250


@pytest.mark.parametrize("nr", [4096, 8192, 16384])
def test_fast_specular_vhf_band(built_lib, oracle, nr):
    # 60 MHz, 2.5 m facets: degree-6 gain polynomial, reradiation arguments up
    # to pi/2; 8192 bins: one transform buffer in shared memory, 16384: the
    # transforms in global scratch by shared-memory sub-blocks
    from helpers import vhf_scene
    sc = vhf_scene(nr)
    sc["params"].update({"specular": True, "rerad_funct": 0})
    got, ref = check_targets(sc, oracle)
    assert got.shape[1] == nr


def test_fast_specular_special_function_path(built_lib, oracle, monkeypatch):
    # RP_PAIR_VARIANT=1: every sinc from the special-function unit
    monkeypatch.setenv("RP_PAIR_VARIANT", "1")
    check_targets(_spec(tiny_scene()), oracle)


def test_fast_specular_disable_surface_has_no_effect(built_lib):
    # specular mode ignores disable_surface (sim.cu:740-772), as the plain form
    from europaraypaths_gb300 import simulator
    a_sc = _spec(tiny_scene(nside=24, ntside=3, ns=2))
    b_sc = _spec(tiny_scene(nside=24, ntside=3, ns=2), disable_surface=True)
    with simulator.Scene(a_sc["params"], a_sc["facets"], a_sc["targets"]) as sa:
        a = sa.simulate(form="fast")
    with simulator.Scene(b_sc["params"], b_sc["facets"], b_sc["targets"]) as sb:
        b = sb.simulate(form="fast")
    assert np.array_equal(_bits(a), _bits(b))


def test_fast_specular_configurations_bitwise_equal(built_lib):
    from europaraypaths_gb300 import simulator
    s = _spec(tiny_scene(nside=40, ntside=4, ns=3))
    outs = []
    simulator.autotune(False)
    try:
        for cfg in (0, 1):
            os.environ["RP_PAIR_CFG"] = str(cfg)
            with simulator.Scene(s["params"], s["facets"], s["targets"]) as sc:
                outs.append(sc.simulate(form="fast"))
    finally:
        os.environ.pop("RP_PAIR_CFG", None)
        simulator.autotune(True)
    assert np.array_equal(_bits(outs[0]), _bits(outs[1]))


def test_fast_specular_batched_with_default_mode(built_lib):
    # a specular scene between default-mode scenes in one batched call: each
    # scene's radargram is bitwise its own single-scene result
    from europaraypaths_gb300 import simulator, traces as tr_mod
    specs = [tiny_scene(nside=24, ntside=3, ns=3), _spec(tiny_scene(nside=30, ntside=4, ns=2)),
             tiny_scene(nside=20, ntside=2, ns=2)]
    scenes = [simulator.Scene(s["params"], s["facets"], s["targets"]) for s in specs]
    try:
        trs = [tr_mod.linear_track(sc.params) for sc in scenes]
        single = [sc.simulate(tr, form="fast") for sc, tr in zip(scenes, trs)]
        batched = simulator.simulate_batch(list(zip(scenes, trs)))
        for a, b in zip(single, batched):
            assert np.array_equal(_bits(a), _bits(b))
    finally:
        for sc in scenes:
            sc.close()


@pytest.mark.parametrize("case", ["targets", "surface_only", "prisms_rerad4", "non_pow2"])
def test_fast_specular_without_convolution(built_lib, oracle, case):
    # no convolution: reflRadarSignal and refrRadarSignal, direct sums of
    # sinc((r - R)/res) phasors over every (source, bin), ttype-0 targets
    from europaraypaths_gb300 import scenes
    over = {"convolution": False}
    if case == "non_pow2":
        over.update(rx_window_m=scenes.rx_window_for_bins(250, 4e6), rx_window_offset_m=24000.0)
    sc = _spec(tiny_scene(), **over)
    sc["targets"][6, :] = 0.0
    prisms = None
    if case == "prisms_rerad4":
        sc["params"]["rerad_funct"] = 4
        prisms = np.array([[2e-3], [-500.0], [-500.0], [-1200.0], [300.0], [400.0], [-100.0]])
    tg = np.zeros((7, 0)) if case == "surface_only" else None
    got, ref, cnt, rcnt = _run(sc, oracle, prisms=prisms, targets=tg, complex128=True)
    assert np.array_equal(cnt, rcnt)
    check(got, ref)
    if tg is None:      # the targets' part alone (complex128 difference)
        got0, ref0, _, _ = _run(sc, oracle, prisms=prisms, targets=np.zeros((7, 0)), complex128=True)
        dg, dr = got - got0, ref - ref0
        assert np.abs(dr).max() > 0
        assert rel_l2(dg, dr) <= REL_L2, rel_l2(dg, dr)


@pytest.mark.parametrize("nr", [None, 250])
def test_fast_specular_circular_convolution(built_lib, oracle, nr):
    # circular convolution (ttype-0 targets only): the surface is zero (the
    # reference's convolution call is commented out) and the targets' summed
    # phasor trace is convolved with genChirp's wrapped chirp; nr = 250: the
    # nr-point Bluestein transform
    from europaraypaths_gb300 import scenes
    over = {} if nr is None else {"rx_window_m": scenes.rx_window_for_bins(nr, 4e6), "rx_window_offset_m": 24000.0}
    sc = _spec(tiny_scene(**over), convolution_linear=False)
    sc["targets"][6, :] = 0.0
    got, ref, cnt, rcnt = _run(sc, oracle, complex128=True)
    assert np.array_equal(cnt, rcnt)
    check(got, ref)


def test_fast_specular_autotuner_records_choice(built_lib):
    from europaraypaths_gb300 import simulator
    simulator.autotune(True)
    s = _spec(tiny_scene(nside=30, ntside=3, ns=2))
    with simulator.Scene(s["params"], s["facets"], s["targets"]) as sc:
        sc.simulate(form="fast")
    tuned = [simulator.autotune_query(False, d, specular=True) for d in (0, 3, 4, 5, 6)]
    assert any(c in (0, 1) for c in tuned) and all(c in (-1, 0, 1) for c in tuned)
