"""Fused FP32 split-precision form vs the FP64 CPU oracle (through the C ABI).

Tolerances (the accuracy bar of the fast form): relative L2 <= 1e-3 of the
complex radargram, max phase error <= 0.01 rad at bins above -40 dB of the
peak, and an exact match of every trace's peak range bin.
"""
import numpy as np
import pytest

from helpers import peak_bins, phase_err_max, rel_l2, tiny_scene, vhf_scene

pytestmark = pytest.mark.gpu

REL_L2 = 1e-3
PHASE = 0.01


def fast_vs_oracle(sc, oracle, traces=None, prisms=None):
    from europaraypaths_gb300 import simulator, traces as tr_mod
    scene = simulator.Scene(sc["params"], sc["facets"], sc["targets"], prisms=prisms)
    tr = tr_mod.linear_track(scene.params) if traces is None else traces
    got, cnt = scene.simulate(tr, form="fast", return_counts=True)
    ref, rcnt = oracle.simulate(scene.params, sc["facets"], sc["targets"], tr, prisms_soa=prisms)
    scene.close()
    return got, ref, cnt, rcnt


def check(got, ref):
    assert rel_l2(got, ref) <= REL_L2, rel_l2(got, ref)
    assert phase_err_max(got, ref) <= PHASE, phase_err_max(got, ref)
    assert np.array_equal(peak_bins(got), peak_bins(ref))


def test_fast_matches_oracle_tiny(built_lib, oracle):
    sc = tiny_scene()
    got, ref, cnt, rcnt = fast_vs_oracle(sc, oracle)
    assert np.array_equal(cnt, rcnt)
    check(got, ref)


def test_fast_small_plain_scene_subset(built_lib, oracle):
    # the full small plain-form scene (40k facets, 1600 targets), 3 traces
    from europaraypaths_gb300 import scenes, traces as tr_mod, param_gen
    sc = scenes.small_plain()
    p = param_gen.to_rp_params(sc["params"])
    tr = tr_mod.linear_track(p)[[0, 50, 99]]
    got, ref, cnt, rcnt = fast_vs_oracle(sc, oracle, traces=tr)
    assert np.array_equal(cnt, rcnt)
    check(got, ref)


def test_fast_non_pow2_bins_and_lossless(built_lib, oracle):
    from europaraypaths_gb300 import scenes
    sc = tiny_scene(rx_window_m=scenes.rx_window_for_bins(250, 4e6), rx_window_offset_m=24000.0,
                    lossless=True)
    got, ref, cnt, rcnt = fast_vs_oracle(sc, oracle)
    assert got.shape[1] == 250
    check(got, ref)


def test_fast_prisms(built_lib, oracle):
    sc = tiny_scene()
    prisms = np.array([[2e-3], [-500.0], [-500.0], [-1200.0], [300.0], [400.0], [-100.0]])
    got, ref, cnt, rcnt = fast_vs_oracle(sc, oracle, prisms=prisms)
    check(got, ref)


def test_fast_deterministic(built_lib):
    from europaraypaths_gb300 import simulator
    sc = tiny_scene(nside=60, ntside=8, ns=4)
    scene = simulator.Scene(sc["params"], sc["facets"], sc["targets"])
    a = scene.simulate(form="fast")
    b = scene.simulate(form="fast")
    scene.close()
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("nside", [400, 285, 200, 148, 30])
def test_fast_polynomial_sinc_regimes(built_lib, oracle, nside):
    # at 9 MHz the largest sinc argument pik = pi^2 fs / lam picks the sinc
    # evaluation: fs 5 m (1.48 rad, degree 3), 7 m (2.08, degree 4), 10 m
    # (2.96, degree 5), 13.5 m (4.0, degree 6), 67 m (special-function path)
    from europaraypaths_gb300 import traces as tr_mod, param_gen
    sc = tiny_scene(nside=nside, ntside=3, ns=2)
    p = param_gen.to_rp_params(sc["params"])
    tr = tr_mod.linear_track(p)
    got, ref, cnt, rcnt = fast_vs_oracle(sc, oracle, traces=tr)
    assert np.array_equal(cnt, rcnt)
    check(got, ref)


@pytest.mark.parametrize("nr", [4096, 8192, 16384, 32768, 6000])
def test_fast_vhf_band(built_lib, oracle, nr):
    # compression storage modes: 4096 bins all in shared memory, 8192 one
    # transform buffer in shared memory with X parked in global scratch,
    # 16384 and 32768 the transforms in global scratch with their inner
    # stages (sub-blocks of 2048 and 4096 values) in shared memory, 6000 (not
    # a power of two) the Bluestein kernel
    sc = vhf_scene(nr)
    got, ref, cnt, rcnt = fast_vs_oracle(sc, oracle)
    assert got.shape[1] == nr
    assert np.array_equal(cnt, rcnt)
    check(got, ref)


def _slope_frames(facets):
    # tangents along the grid axes normalised independently, u ~ (1, 0,
    # dz/dx) and v ~ (0, 1, dz/dy): not orthogonal on sloped facets
    f = facets.copy()
    dzdx, dzdy = -f[3] / f[5], -f[4] / f[5]
    u = np.stack([np.ones_like(dzdx), np.zeros_like(dzdx), dzdx])
    v = np.stack([np.zeros_like(dzdy), np.ones_like(dzdy), dzdy])
    f[6:9] = u / np.linalg.norm(u, axis=0)
    f[9:12] = v / np.linalg.norm(v, axis=0)
    return f


def test_fast_non_orthonormal_frames(built_lib, oracle):
    # a rough surface whose facet frames are not orthonormal takes the
    # general directivity (the facet normal from the record)
    sc = vhf_scene(2048, n_side=80)
    sc["facets"] = _slope_frames(sc["facets"])
    uv = np.abs(np.einsum("ij,ij->j", sc["facets"][6:9], sc["facets"][9:12]))
    assert uv.max() > 1e-3
    got, ref, cnt, rcnt = fast_vs_oracle(sc, oracle)
    assert np.array_equal(cnt, rcnt)
    check(got, ref)


def test_fast_orthonormal_and_general_frames_agree(built_lib, oracle, monkeypatch):
    # the same orthonormal scene through both directivity forms: the
    # orthonormal-frame shortcut is an identity, so they differ by rounding
    sc = vhf_scene(2048, n_side=80)
    got_o, ref, _, _ = fast_vs_oracle(sc, oracle)
    monkeypatch.setenv("RP_PAIR_ORTHO", "0")
    got_g, _, _, _ = fast_vs_oracle(sc, oracle)
    check(got_o, ref)
    check(got_g, ref)
    assert rel_l2(got_o, got_g) <= 1e-4, rel_l2(got_o, got_g)


def test_fast_incoherent_matches_oracle(built_lib, oracle):
    # incoherent mode (seeded surface phases) in the fast form
    sc = tiny_scene(incoherent=True, incoherent_seed=5)
    got, ref, cnt, rcnt = fast_vs_oracle(sc, oracle)
    assert np.array_equal(cnt, rcnt)
    check(got, ref)


def test_fast_narrow_aperture_tile_culling(built_lib, oracle):
    # a 1-degree aperture over a 40k-facet store: most 1024-facet culling
    # tiles lie outside the cone and are skipped; the illuminated counts and
    # the radargram still match the oracle exactly / within tolerance
    sc = tiny_scene(nside=200, ntside=4, ns=3, aperture=1.0)
    got, ref, cnt, rcnt = fast_vs_oracle(sc, oracle)
    assert np.array_equal(cnt, rcnt) and 0 < cnt[:, 0].max() < 40000 // 4
    check(got, ref)


def test_fast_split_parts_small_call(built_lib, oracle):
    # one trace of the small plain scene fills a few target blocks, so its
    # facet parts are split further (k_pairs32's split instance) and folded
    # back before the compression: one launch more than the same trace
    # inside a 40-trace call, the same result to FP32 summation order, and
    # within the bar against the oracle
    from europaraypaths_gb300 import scenes, simulator, traces as tr_mod, param_gen
    sc = scenes.small_plain()
    p = param_gen.to_rp_params(sc["params"])
    tr = tr_mod.linear_track(p)
    scene = simulator.Scene(sc["params"], sc["facets"], sc["targets"])
    try:
        scene.simulate(tr[30:70], form="fast")      # warm-up: the first call may tune
        many = scene.simulate(tr[30:70], form="fast")
        n_many = simulator.last_launch_count()
        one = scene.simulate(tr[50:51], form="fast")
        n_one = simulator.last_launch_count()
    finally:
        scene.close()
    assert n_one == n_many + 1, (n_one, n_many)
    assert rel_l2(one[0], many[20]) <= 1e-6, rel_l2(one[0], many[20])
    assert np.array_equal(peak_bins(one), peak_bins(many[20:21]))
    ref, _ = oracle.simulate(scene.params, sc["facets"], sc["targets"], tr[50:51])
    check(one, ref)
