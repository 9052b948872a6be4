"""The C ABI library loads on a machine without a GPU, exports every function
include/raypath.h declares, and its host-only entry points behave (no GPU
work is issued here)."""
import ctypes
import os
import re

import numpy as np
import pytest

from europaraypaths_gb300 import _abi, param_gen
from helpers import tiny_scene

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "raypath.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(rp_[a-z_0-9]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(built_lib):
    names = declared_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(built_lib, n), f"libraypath.so does not export {n}"
        assert n in _abi._SIGS, f"_abi has no signature for {n}"


def test_version_and_error_text(built_lib):
    assert b"raypath" in built_lib.rp_version()
    p = _abi.RpParams()
    rc = built_lib.rp_params_derive(ctypes.byref(p))
    assert rc == -1
    assert "must be positive" in _abi.last_error()
    assert built_lib.rp_params_derive(None) == -1


def test_params_derive_matches_oracle(built_lib, oracle):
    sc = tiny_scene()
    a = param_gen.to_rp_params(sc["params"])                 # library derivation
    b = param_gen.to_rp_params(sc["params"], derive=False)
    oracle.derive(b)                                        # oracle's own restatement
    for name, _ in _abi.RpParams._fields_:
        assert getattr(a, name) == getattr(b, name), name


def test_nr_follows_reference_float_expression(built_lib):
    # nr = (int)((float(rx_window_m) / 299792480.0f) * smpl) (file_io.cu:212)
    sc = tiny_scene()
    for win, smpl in ((1.25e3, 60e6), (0.75e3, 120e6), (10e3, 18e6), (153534.0, 4e6)):
        j = dict(sc["params"], rx_window_m=win, rx_sample_rate=smpl)
        p = param_gen.to_rp_params(j)
        f32 = np.float32
        assert p.nr == int(f32(f32(win) / f32(299792480.0)) * f32(smpl))
        assert abs(p.dr - win / p.nr) < 1e-12


def test_missing_required_key_raises():
    sc = tiny_scene()
    j = dict(sc["params"])
    del j["frequency"]
    with pytest.raises(KeyError):
        param_gen.to_rp_params(j, derive=False)
    j = dict(sc["params"])
    del j["rx_window_offset_m"]          # needed when there is no rx window file
    with pytest.raises(KeyError):
        param_gen.to_rp_params(j, derive=False)
    j["rx_window_position_file"] = "rx.txt"
    param_gen.to_rp_params(j, derive=False)


def test_prism_alpha(built_lib, oracle):
    from oracle import np_oracle
    sc = tiny_scene()
    p = param_gen.to_rp_params(sc["params"])
    a = ctypes.c_double()
    assert built_lib.rp_prism_alpha(ctypes.byref(p), 2e-5, ctypes.byref(a)) == 0
    pd = np_oracle.derive(sc["params"])
    assert abs(a.value - np_oracle.prism_alpha(2e-5, pd)) < 1e-15


def test_scene_create_rejects_bad_arguments(built_lib):
    sc = tiny_scene()
    p = param_gen.to_rp_params(sc["params"])
    h = ctypes.c_void_p()
    assert built_lib.rp_scene_create(ctypes.byref(p), None, 10, None, 0, None, 0, 0, ctypes.byref(h)) == -1
    assert built_lib.rp_scene_create(None, None, 0, None, 0, None, 0, 0, ctypes.byref(h)) == -1
    q = param_gen.to_rp_params(dict(sc["params"], convolution=False))
    f = np.ascontiguousarray(sc["facets"])
    assert built_lib.rp_scene_create(ctypes.byref(q), f.ctypes.data, f.shape[1], None, 0, None, 0, 0,
                                     ctypes.byref(h)) == -6
    assert built_lib.rp_simulate(None, None, 1, 1, None, 0, None, None) == -1


def test_graph_calls_reject_bad_arguments(built_lib):
    # argument checks come before any device work, so they run without a GPU
    g = ctypes.c_void_p()
    assert built_lib.rp_graph_create(None, None, None, 1, None, ctypes.byref(g)) == -1
    assert "rp_graph_create" in _abi.last_error()
    assert built_lib.rp_graph_launch(None, None) == -1
    assert built_lib.rp_graph_check(None, None) == -1
    assert built_lib.rp_graph_destroy(None) == 0
    assert built_lib.rp_graph_create_batch(None, 1, None, ctypes.byref(g)) == -1
    assert "rp_graph_create_batch" in _abi.last_error()
    jobs = (_abi.RpJob * 1)()
    ptrs = (ctypes.c_void_p * 1)()
    assert built_lib.rp_graph_create_batch(jobs, 0, ptrs, ctypes.byref(g)) == -1
    assert built_lib.rp_graph_create_batch(jobs, 1, ptrs, ctypes.byref(g)) == -1     # no scene
    assert "job 0" in _abi.last_error()
    assert built_lib.rp_split_parts(0) == 0 and built_lib.rp_split_parts(1) == 0


@pytest.mark.parametrize("over,ttype", [({"convolution": False}, 1), ({"convolution_linear": False}, 1),
                                        ({"specular": True, "convolution": False}, 1),
                                        ({"specular": True, "convolution_linear": False}, 1)])
def test_scene_create_refuses_undefined_modes(built_lib, over, ttype):
    # checked before any CUDA call: runs without a GPU
    import ctypes
    from europaraypaths_gb300 import _abi, param_gen, scenes
    sc = scenes.small_plain(n_facets_side=8, n_targets_side=2, ns=1)
    sc["params"].update(over)
    p = param_gen.to_rp_params(sc["params"])
    t = np.ascontiguousarray(sc["targets"])
    t[6, :] = ttype
    f = np.ascontiguousarray(sc["facets"])
    h = ctypes.c_void_p()
    rc = built_lib.rp_scene_create(ctypes.byref(p), f.ctypes.data, f.shape[1], t.ctypes.data, t.shape[1],
                                   None, 0, 0, ctypes.byref(h))
    assert rc == -6, _abi.last_error()


def test_autotune_query_kinds_without_a_gpu(built_lib):
    # the tuned-configuration table is host state: every kind (single-batch,
    # multi-segment, specular) answers -1 before any launch, and an unknown
    # degree too
    from europaraypaths_gb300 import simulator
    assert simulator.autotune_query(False, 99) == -1
    assert simulator.autotune_query(True) in range(-1, 10)
    assert simulator.autotune_query(False, 99, specular=True) == -1


def test_sim_auto_form_is_fast_for_every_mode():
    # every mode the reference defines runs in the fast form
    import numpy as np
    from europaraypaths_gb300 import param_gen, scenes, sim
    base = scenes.small_plain(n_facets_side=10, n_targets_side=2, ns=2)
    for over in ({}, {"specular": True}, {"specular": True, "convolution_linear": False},
                 {"specular": True, "convolution": False}):
        p = dict(base["params"])
        p.update(over)
        tg = np.array(base["targets"], copy=True)
        if over.get("convolution") is False or over.get("convolution_linear") is False:
            tg[6, :] = 0.0
        assert sim.pick_form(param_gen.to_rp_params(p), tg) == "fast"
