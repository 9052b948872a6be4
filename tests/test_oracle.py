"""The C++ FP64 oracle vs the NumPy restatement, and its own invariants."""
import numpy as np
import pytest

from europaraypaths_gb300 import param_gen, scenes, traces as tr_mod
from helpers import rel_l2, tiny_scene
from oracle import np_oracle


def prep(sc, oracle):
    p = param_gen.to_rp_params(sc["params"], derive=False)
    oracle.derive(p)
    pd = np_oracle.derive(sc["params"])
    pd["P"] = p.power
    pd["B"] = p.bandwidth
    return p, pd


def both(sc, oracle, prisms=None, traces=None):
    p, pd = prep(sc, oracle)
    tr = tr_mod.linear_track(p) if traces is None else traces
    got, cnt = oracle.simulate(p, sc["facets"], sc["targets"], tr, prisms_soa=prisms)
    npr = None
    if prisms is not None:
        npr = np.array(prisms).T
    ref, rcnt = np_oracle.simulate(pd, sc["facets"].T, sc["targets"].T, tr, prisms=npr)
    return got, ref, cnt, rcnt


def test_derive_matches_numpy(oracle):
    sc = tiny_scene()
    p, pd = prep(sc, oracle)
    for k in ("lam", "k", "rng_res", "alpha1", "alpha2", "nr", "dr", "c_1", "c_2", "nu_1", "nu_2", "ks"):
        assert abs(getattr(p, k) - pd[k]) <= 1e-12 * abs(pd[k]) + 1e-300, k


def test_oracle_matches_numpy_default(oracle):
    got, ref, cnt, rcnt = both(tiny_scene(), oracle)
    assert np.array_equal(cnt, rcnt)
    assert rel_l2(got, ref) < 1e-12


def test_oracle_matches_numpy_non_pow2_lossless(oracle):
    sc = tiny_scene(rx_window_m=scenes.rx_window_for_bins(250, 4e6), rx_window_offset_m=24000.0,
                    lossless=True)
    got, ref, cnt, rcnt = both(sc, oracle)
    assert got.shape[1] == 250
    assert rel_l2(got, ref) < 1e-12


def test_oracle_matches_numpy_ttype0_prisms(oracle):
    sc = tiny_scene(rerad_funct=0)
    sc["targets"][6, ::2] = 0.0
    prisms = np.array([[2e-3], [-500.0], [-500.0], [-1200.0], [300.0], [400.0], [-100.0]])
    got, ref, cnt, rcnt = both(sc, oracle, prisms=prisms)
    assert rel_l2(got, ref) < 1e-12


@pytest.mark.parametrize("rf", [1, 2, 3, 4])
def test_oracle_rerad_functions(oracle, rf):
    sc = tiny_scene(rerad_funct=rf)
    sc["targets"][6, :] = 0.0
    got, ref, cnt, rcnt = both(sc, oracle)
    if np.linalg.norm(ref) > 0:
        assert rel_l2(got, ref) < 1e-12


def test_oracle_empty_and_far_traces(oracle):
    sc = tiny_scene(disable_surface=True)
    p, _ = prep(sc, oracle)
    tr = tr_mod.linear_track(p)
    tr[0, 0] += 1e6
    got, cnt = oracle.simulate(p, sc["facets"], sc["targets"], tr)
    assert cnt[0, 0] == 0 and np.all(got[0] == 0)
    # no targets at all: surface only
    got2, cnt2 = oracle.simulate(p, sc["facets"], np.zeros((7, 0)), tr)
    assert np.all(cnt2[:, 1] == 0)


def test_oracle_thread_count_independent(oracle):
    sc = tiny_scene(nside=30, ntside=5, ns=2)
    p, _ = prep(sc, oracle)
    tr = tr_mod.linear_track(p)
    a, _ = oracle.simulate(p, sc["facets"], sc["targets"], tr, nthreads=1)
    b, _ = oracle.simulate(p, sc["facets"], sc["targets"], tr, nthreads=4)
    assert np.array_equal(a, b)


def test_oracle_target_cap(oracle):
    sc = tiny_scene(nside=30, ntside=5, ns=1)
    p, _ = prep(sc, oracle)
    tr = tr_mod.linear_track(p)
    _, cnt = oracle.simulate(p, sc["facets"], sc["targets"], tr, max_targets=3)
    assert cnt[0, 1] == 3


def _ttype0(sc):
    sc["targets"][6, :] = 0.0
    return sc


@pytest.mark.parametrize("mode", ["specular_linear", "specular_none", "specular_circular"])
def test_oracle_matches_numpy_specular_modes(oracle, mode):
    # the specular variants the reference defines (sim.cu:733-986): linear
    # convolution with every target type; no convolution and circular
    # convolution with ttype 0 targets
    over = {"specular": True, "rerad_funct": 0}
    if mode == "specular_none":
        over["convolution"] = False
    if mode == "specular_circular":
        over["convolution_linear"] = False
    sc = tiny_scene(nside=24, ntside=3, ns=2, **over)
    if mode == "specular_linear":
        sc["targets"][6, ::2] = 0.0
    else:
        _ttype0(sc)
    got, ref, cnt, rcnt = both(sc, oracle)
    assert np.array_equal(cnt, rcnt)
    assert np.abs(ref).max() > 0
    assert rel_l2(got, ref) < 1e-11


@pytest.mark.parametrize("over", [{"convolution": False}, {"convolution_linear": False},
                                  {"specular": True, "convolution": False},
                                  {"specular": True, "convolution_linear": False}])
def test_oracle_rejects_undefined_modes(oracle, over):
    # non-specular without linear convolution, and specular without linear
    # convolution for ttype-1 targets, use buffers the reference never sized
    # or allocated: the oracle refuses them (RP_ERR_UNSUPPORTED)
    sc = tiny_scene(nside=12, ntside=2, ns=1, **over)
    p, _ = prep(sc, oracle)
    with pytest.raises(RuntimeError, match="-6"):
        oracle.simulate(p, sc["facets"], sc["targets"], tr_mod.linear_track(p))


def test_oracle_incoherent_seeded(oracle):
    # incoherent mode's surface phases come from a seeded hash of (seed,
    # source position, facet index): the C++ and NumPy oracles agree, a run
    # repeats exactly, another seed (or coherent mode) differs
    got, ref, cnt, rcnt = both(tiny_scene(incoherent=True, incoherent_seed=7), oracle)
    assert np.array_equal(cnt, rcnt) and rel_l2(got, ref) < 1e-12
    assert np.array_equal(both(tiny_scene(incoherent=True, incoherent_seed=7), oracle)[0], got)
    assert rel_l2(both(tiny_scene(incoherent=True, incoherent_seed=8), oracle)[0], got) > 1e-2
    assert rel_l2(both(tiny_scene(), oracle)[0], got) > 1e-2
    # a trace's result does not depend on the other traces of the call
    sc = tiny_scene(incoherent=True, incoherent_seed=7)
    p, _ = prep(sc, oracle)
    tr = tr_mod.linear_track(p)
    one, _ = oracle.simulate(p, sc["facets"], sc["targets"], tr[1:2])
    assert np.array_equal(one[0], got[1])


def test_incoherent_turns_distribution():
    # the 24-bit phases are uniform on [0, 1): mean and variance of 1e5 draws
    t = np_oracle.incoherent_turns(3, np.array([0.0, 1.0, 2.5e4]), np.arange(100000))
    assert t.min() >= 0.0 and t.max() < 1.0
    assert abs(t.mean() - 0.5) < 5e-3 and abs(t.var() - 1 / 12) < 2e-3
