"""Many scenes in one call (rp_simulate_batch): the pair stage of every scene
in one persistent launch.  Each job's radargram is bitwise the one the scene
gives alone (split facet parts off, so that no lone call regroups its part
sums), and within the fast form's tolerance of the FP64 oracle; the
pair-kernel configurations the autotuner chooses between give bitwise equal
results; a scene with more traces than one segment (multi-job kernel) equals
its traces run one at a time."""
import os

import numpy as np
import pytest

from helpers import peak_bins, phase_err_max, rel_l2, tiny_scene

pytestmark = pytest.mark.gpu

REL_L2 = 1e-3
PHASE = 0.01


def _scenes():
    from europaraypaths_gb300 import scenes
    return [
        tiny_scene(nside=40, ntside=4, ns=5),                                        # 9 MHz, 2048 bins
        tiny_scene(nside=30, ntside=3, ns=3, eps_2=4.0,
                   rx_window_m=scenes.rx_window_for_bins(1024, 4e6)),                # 1024 bins
        tiny_scene(nside=148, ntside=3, ns=2),                                       # fs 13.5 m: degree-6 sinc
        tiny_scene(nside=30, ntside=4, ns=4, rx_window_m=scenes.rx_window_for_bins(512, 4e6),
                   rx_window_offset_m=24200.0),                                      # 512 bins
        tiny_scene(nside=30, ntside=3, ns=2,
                   rx_window_m=scenes.rx_window_for_bins(8192, 4e6)),                # 8192 bins (mode 1)
    ]


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def test_batch_equals_single_and_oracle(built_lib, oracle, no_split_parts):
    from europaraypaths_gb300 import simulator, traces as tr_mod
    scs = _scenes()
    scenes = [simulator.Scene(s["params"], s["facets"], s["targets"]) for s in scs]
    try:
        trs = [tr_mod.linear_track(sc.params) for sc in scenes]
        outs, counts = simulator.simulate_batch(list(zip(scenes, trs)), return_counts=True)
        for sc, s, tr, got, cnt in zip(scenes, scs, trs, outs, counts):
            alone, acnt = sc.simulate(tr, return_counts=True)
            assert np.array_equal(_bits(alone), _bits(got))
            assert np.array_equal(acnt, cnt)
            ref, rcnt = oracle.simulate(sc.params, s["facets"], s["targets"], tr)
            assert np.array_equal(cnt, rcnt)
            assert rel_l2(got, ref) <= REL_L2
            assert phase_err_max(got, ref) <= PHASE
            assert np.array_equal(peak_bins(got), peak_bins(ref))
    finally:
        for sc in scenes:
            sc.close()


def test_batch_per_segment_launches_bitwise(built_lib):
    # multi-segment waves in configurations 4-7 (one single-batch kernel per
    # segment, on the workspace's auxiliary streams) and 8-9 (one multi-job
    # kernel per sinc-degree and frame-kind group): bitwise the same
    # radargrams as the multi-job kernel
    from europaraypaths_gb300 import simulator, traces as tr_mod
    scs = _scenes()
    res = {}
    simulator.autotune(False)
    try:
        for cfg in (1, 5, 7, 8, 9):
            os.environ["RP_PAIR_CFG"] = str(cfg)
            scenes = [simulator.Scene(s["params"], s["facets"], s["targets"]) for s in scs]
            try:
                trs = [tr_mod.linear_track(sc.params) for sc in scenes]
                res[cfg] = simulator.simulate_batch(list(zip(scenes, trs)))
            finally:
                for sc in scenes:
                    sc.close()
    finally:
        os.environ.pop("RP_PAIR_CFG", None)
        simulator.autotune(True)
    for cfg in (5, 7, 8, 9):
        for a, b in zip(res[1], res[cfg]):
            assert np.array_equal(_bits(a), _bits(b))


def test_many_segments_multi_kernel(built_lib, no_split_parts):
    # 70 traces = two segments of one scene in one wave: the multi-job kernel
    from europaraypaths_gb300 import simulator, traces as tr_mod
    s = tiny_scene(nside=24, ntside=3, ns=70)
    with simulator.Scene(s["params"], s["facets"], s["targets"]) as sc:
        tr = tr_mod.linear_track(sc.params)
        assert tr.shape[0] == 70
        full = sc.simulate(tr)
        for k in (0, 33, 64, 69):
            one = sc.simulate(tr[k:k + 1])
            assert np.array_equal(_bits(one[0]), _bits(full[k]))


def test_pair_configurations_bitwise_equal(built_lib):
    from europaraypaths_gb300 import simulator, traces as tr_mod
    s = tiny_scene(nside=40, ntside=4, ns=3)
    outs = []
    simulator.autotune(False)
    try:
        for cfg in range(4):
            os.environ["RP_PAIR_CFG"] = str(cfg)
            with simulator.Scene(s["params"], s["facets"], s["targets"]) as sc:
                tr = tr_mod.linear_track(sc.params)
                outs.append(sc.simulate(tr))
    finally:
        os.environ.pop("RP_PAIR_CFG", None)
        simulator.autotune(True)
    for o in outs[1:]:
        assert np.array_equal(_bits(o), _bits(outs[0]))


def test_autotuner_records_choice(built_lib):
    from europaraypaths_gb300 import simulator, traces as tr_mod
    simulator.autotune(True)
    s = tiny_scene(nside=30, ntside=3, ns=2)
    with simulator.Scene(s["params"], s["facets"], s["targets"]) as sc:
        sc.simulate(tr_mod.linear_track(sc.params))
    tuned = [simulator.autotune_query(False, d) for d in (0, 3, 4, 5, 6)]
    assert any(0 <= c <= 3 for c in tuned)
