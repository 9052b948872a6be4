"""The pair kernels' bounded waits: a wait that runs out is an error status,
not a hang, and the context stays usable.

A scene created with RP_TEST_STALL_COPIES=1 runs the pair kernels in a test
mode that issues no bulk copy of a chunk, so the first wait on a chunk's
mbarrier has nothing to wait for.  The wait gives up after a short bounded
number of polls; the block raises the timeout flag and stops, with no copy
in flight, and the call returns RP_ERR_TIMEOUT.  The same process then runs
a normal scene on the same device and checks it against the oracle.  Covered
for the default-mode kernel (pair_item), ttype-0 targets (pair_item_t0) and
specular mode (pair_item with the outbound window).
"""
import numpy as np
import pytest

from helpers import rel_l2, tiny_scene

pytestmark = pytest.mark.gpu

RP_ERR_TIMEOUT = -8


def _scene(kind):
    if kind == "default":
        return tiny_scene(nside=40, ntside=4, ns=2)
    if kind == "ttype0":
        sc = tiny_scene(nside=40, ntside=4, ns=2)
        sc["targets"][6, :] = 0.0
        return sc
    return tiny_scene(nside=30, ntside=3, ns=2, specular=True, rerad_funct=0)


@pytest.mark.parametrize("kind", ["default", "ttype0", "specular"])
def test_stalled_copy_wait_times_out_and_context_survives(built_lib, oracle, monkeypatch, kind):
    from europaraypaths_gb300 import _abi, simulator
    sc = _scene(kind)
    monkeypatch.setenv("RP_TEST_STALL_COPIES", "1")
    stalled = simulator.Scene(sc["params"], sc["facets"], sc["targets"])
    monkeypatch.delenv("RP_TEST_STALL_COPIES")
    with pytest.raises(_abi.RaypathError) as ei:
        stalled.simulate(form="fast")
    assert ei.value.rc == RP_ERR_TIMEOUT
    assert "timed out" in str(ei.value)
    stalled.close()
    # the device still works: a normal scene, same process, matches the oracle
    with simulator.Scene(sc["params"], sc["facets"], sc["targets"]) as scene:
        tr = scene.default_traces()
        got = scene.simulate(tr, form="fast")
        ref, _ = oracle.simulate(scene.params, sc["facets"], sc["targets"], tr)
    assert rel_l2(got, ref) <= 1e-3
