"""Plain FP64 form vs the FP64 CPU oracle (through the C ABI)."""
import numpy as np
import pytest

from helpers import rel_l2, tiny_scene

pytestmark = pytest.mark.gpu


def run_both(sc, oracle, prisms=None, traces=None):
    from europaraypaths_gb300 import simulator, traces as tr_mod
    scene = simulator.Scene(sc["params"], sc["facets"], sc["targets"], prisms=prisms)
    tr = tr_mod.linear_track(scene.params) if traces is None else traces
    got, cnt = scene.simulate(tr, form="plain", complex128=True, return_counts=True)
    ref, rcnt = oracle.simulate(scene.params, sc["facets"], sc["targets"], tr, prisms_soa=prisms)
    scene.close()
    return got, ref, cnt, rcnt


def test_plain_matches_oracle(built_lib, oracle):
    sc = tiny_scene()
    got, ref, cnt, rcnt = run_both(sc, oracle)
    assert np.array_equal(cnt, rcnt)
    assert rel_l2(got, ref) < 1e-10


def test_plain_non_pow2_bins(built_lib, oracle):
    # nr = 250: 2 nr is not a power of two (Bluestein for both lengths)
    from europaraypaths_gb300 import scenes
    sc = tiny_scene(rx_window_m=scenes.rx_window_for_bins(250, 4e6) * 1.0, rx_window_offset_m=24000.0)
    got, ref, cnt, rcnt = run_both(sc, oracle)
    assert got.shape[1] == 250
    assert rel_l2(got, ref) < 1e-10


def test_plain_ttype0_prisms_lossless(built_lib, oracle):
    sc = tiny_scene(lossless=True, rerad_funct=0)
    sc["targets"][6, ::2] = 0.0           # every other target is a ttype-0 target
    prisms = np.array([[2e-3], [-500.0], [-500.0], [-1200.0], [300.0], [400.0], [-100.0]])
    got, ref, cnt, rcnt = run_both(sc, oracle, prisms=prisms)
    assert rel_l2(got, ref) < 1e-10
    sc2 = tiny_scene(lossless=False)
    got, ref, cnt, rcnt = run_both(sc2, oracle, prisms=prisms)
    assert rel_l2(got, ref) < 1e-10


def test_plain_disable_surface_and_empty_trace(built_lib, oracle):
    from europaraypaths_gb300 import traces as tr_mod, param_gen
    sc = tiny_scene(disable_surface=True)
    p = param_gen.to_rp_params(sc["params"])
    tr = tr_mod.linear_track(p)
    tr[1, 0] += 1e6          # a trace far away: no facet illuminated -> zero column
    got, ref, cnt, rcnt = run_both(sc, oracle, traces=tr)
    assert cnt[1, 0] == 0 and np.all(got[1] == 0)
    assert rel_l2(got, ref) < 1e-10


@pytest.mark.parametrize("mode", ["specular_linear", "specular_none", "specular_circular"])
def test_plain_specular_modes(built_lib, oracle, mode):
    # the specular variants of the reference trace loop (sim.cu:733-986):
    # genReflPhasor/genRefrPhasor + linear convolution with every target type;
    # reflRadarSignal/refrRadarSignal direct sums; circular convolution
    over = {"specular": True, "rerad_funct": 0}
    if mode == "specular_none":
        over["convolution"] = False
    if mode == "specular_circular":
        over["convolution_linear"] = False
    sc = tiny_scene(nside=24, ntside=3, ns=2, **over)
    if mode == "specular_linear":
        sc["targets"][6, ::2] = 0.0
    else:
        sc["targets"][6, :] = 0.0
    got, ref, cnt, rcnt = run_both(sc, oracle)
    assert np.array_equal(cnt, rcnt)
    assert np.abs(ref).max() > 0
    assert rel_l2(got, ref) < 1e-10


def test_plain_incoherent_matches_oracle(built_lib, oracle):
    # incoherent mode: the seeded surface phases, FP64 like the oracle
    sc = tiny_scene(incoherent=True, incoherent_seed=5)
    got, ref, cnt, rcnt = run_both(sc, oracle)
    assert np.array_equal(cnt, rcnt)
    assert rel_l2(got, ref) < 1e-10


def test_plain_narrow_aperture_tile_culling(built_lib, oracle):
    # the input-order store's culling tiles (rows of the facet grid)
    sc = tiny_scene(nside=200, ntside=4, ns=3, aperture=1.0)
    got, ref, cnt, rcnt = run_both(sc, oracle)
    assert np.array_equal(cnt, rcnt) and 0 < cnt[:, 0].max() < 40000 // 4
    assert rel_l2(got, ref) < 1e-10
