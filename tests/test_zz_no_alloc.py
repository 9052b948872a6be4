"""rp_surface_noalloc: surface-only columns with no device allocation.

Some callers cannot allocate device memory once they are running -- their
device memory is fixed at start-up (owned by a host application's allocator,
or a service that must not grow after initialisation).  For them the library
offers one entry point whose scratch is a fixed array inside the library.
This test calls it through the C ABI twice in a row and checks both results
against the resident fast form (rp_simulate_device) on a scene without
targets within 1e-6 relative L2, and against the FP64 CPU oracle within
1e-5; it also checks that oversized requests are refused with RP_ERR_BUDGET
and specular scenes (whose surface leg it does not compute) with
RP_ERR_UNSUPPORTED.

Every call is issued on torch's current stream, the stream whose kernels
fill the inputs and pre-fill the outputs, so the call is ordered after them.

The file name sorts last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

from helpers import rel_l2, tiny_scene

pytestmark = pytest.mark.gpu

TOL_FAST = 1e-6
TOL_ORACLE = 1e-5


def _noalloc(lib, scene, d_tr, ns, out):
    from europaraypaths_gb300 import simulator
    return lib.rp_surface_noalloc(ctypes.c_void_p(scene.handle), ctypes.c_void_p(d_tr.data_ptr()), ns,
                                  ctypes.c_void_p(out.data_ptr()), simulator.stream_handle(None, scene.device))


def test_surface_noalloc_matches_fast_form_and_oracle(built_lib, oracle):
    import torch
    from europaraypaths_gb300 import _abi, simulator, traces as tr_mod

    sc = tiny_scene(nside=40, ns=5)
    scene = simulator.Scene(sc["params"], sc["facets"], targets=None)
    tr = tr_mod.linear_track(scene.params)
    tr[2, 0] += 1e6                     # one trace sees no facet: a zero column
    ns, nr = tr.shape[0], scene.nr
    d_tr = torch.from_numpy(np.ascontiguousarray(tr)).cuda()
    ref = torch.zeros((ns, nr), dtype=torch.complex64, device="cuda")
    scene.simulate_device(d_tr, ref, form="fast")
    ref_h = ref.cpu().numpy()
    assert np.abs(ref_h).max() > 0 and np.all(ref_h[2] == 0)
    orc, _ = oracle.simulate(scene.params, sc["facets"], np.zeros((7, 0)), tr)
    lib = _abi.lib()
    for call in range(2):
        out = torch.full((ns, nr), complex(float("nan"), float("nan")), dtype=torch.complex64,
                         device="cuda")
        _abi.check("rp_surface_noalloc", _noalloc(lib, scene, d_tr, ns, out))
        got = out.cpu().numpy()        # ordered after the call on the same stream
        assert np.all(np.isfinite(got)), f"call {call}: unwritten output"
        assert rel_l2(got, ref_h) <= TOL_FAST, f"call {call}: rel L2 vs fast form {rel_l2(got, ref_h)}"
        assert rel_l2(got, orc) <= TOL_ORACLE, f"call {call}: rel L2 vs oracle {rel_l2(got, orc)}"
        assert np.all(got[2] == 0)
    # a request beyond the fixed scratch is refused, without touching the GPU
    big = torch.zeros((17, 9), dtype=torch.float64, device="cuda")
    rc = _noalloc(lib, scene, big, 17, out)
    assert rc == -7 and "at most 16 traces" in _abi.last_error()
    scene.close()


def test_surface_noalloc_incoherent_matches_fast_form(built_lib):
    # incoherent mode's seeded phases key on the facet's input index, which
    # both entry points recover from the sorted store
    import torch
    from europaraypaths_gb300 import _abi, simulator, traces as tr_mod

    sc = tiny_scene(nside=30, ns=3, incoherent=True, incoherent_seed=9)
    scene = simulator.Scene(sc["params"], sc["facets"], targets=None)
    tr = tr_mod.linear_track(scene.params)
    d_tr = torch.from_numpy(np.ascontiguousarray(tr)).cuda()
    ref = torch.zeros((tr.shape[0], scene.nr), dtype=torch.complex64, device="cuda")
    scene.simulate_device(d_tr, ref, form="fast")
    out = torch.zeros_like(ref)
    _abi.check("rp_surface_noalloc", _noalloc(_abi.lib(), scene, d_tr, tr.shape[0], out))
    assert rel_l2(out.cpu().numpy(), ref.cpu().numpy()) <= TOL_FAST
    scene.close()


def test_surface_noalloc_narrow_aperture_skips_tiles(built_lib, oracle):
    # a 1-degree aperture over a 40k-facet store: most culling tiles lie
    # outside the cone and are skipped; the columns still match the oracle
    import torch
    from europaraypaths_gb300 import _abi, simulator, traces as tr_mod

    sc = tiny_scene(nside=200, ns=3, aperture=1.0)
    scene = simulator.Scene(sc["params"], sc["facets"], targets=None)
    tr = tr_mod.linear_track(scene.params)
    d_tr = torch.from_numpy(np.ascontiguousarray(tr)).cuda()
    out = torch.zeros((tr.shape[0], scene.nr), dtype=torch.complex64, device="cuda")
    _abi.check("rp_surface_noalloc", _noalloc(_abi.lib(), scene, d_tr, tr.shape[0], out))
    orc, cnt = oracle.simulate(scene.params, sc["facets"], np.zeros((7, 0)), tr)
    assert 0 < cnt[:, 0].max() < 40000 // 4
    assert rel_l2(out.cpu().numpy(), orc) <= TOL_ORACLE
    scene.close()


def test_surface_noalloc_refuses_specular(built_lib):
    # its kernel is the default mode's surface leg: a specular scene is
    # refused before any device work
    import torch
    from europaraypaths_gb300 import _abi, simulator

    sc = tiny_scene(nside=12, ns=1, specular=True, rerad_funct=0)
    scene = simulator.Scene(sc["params"], sc["facets"], targets=None)
    d_tr = torch.zeros((1, 9), dtype=torch.float64, device="cuda")
    out = torch.zeros((1, scene.nr), dtype=torch.complex64, device="cuda")
    rc = _noalloc(_abi.lib(), scene, d_tr, 1, out)
    assert rc == -6 and "non-specular" in _abi.last_error()
    scene.close()
