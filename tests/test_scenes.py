"""Seeded scene generators (CPU): the blocked surface builder used for the
64M-facet flyby scene gives the same facets, bit for bit, as the whole-grid
``surface_arrays`` (``gen_normals`` restated from simple_surfaces.py:3-39),
and the flyby generator keeps its sizes when reduced."""
import numpy as np
import pytest


@pytest.mark.parametrize("ny,nx,rows", [(37, 41, 5), (300, 200, 64), (3, 7, 1), (5, 5, 2), (4, 9, 1),
                                        (9, 9, 4), (130, 17, 256)])
def test_blocked_surface_is_bit_identical(ny, nx, rows):
    from europaraypaths_gb300 import simple_surfaces as ss
    h = np.random.default_rng(ny * 1000 + nx).normal(0.0, 3.0, (ny, nx))
    dom = {"fs": 2.5, "nx": nx, "ny": ny, "ox": -10.0, "oy": -7.0}
    a = ss.surface_arrays(dom, "flat", heights=h)
    b = ss.surface_arrays_blocked(dom, h, rows_per_block=rows)
    assert a.shape == b.shape
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_flyby_reduced_shapes_and_bands():
    from europaraypaths_gb300 import param_gen, scenes
    sc = scenes.flyby(n_facets_side=200)             # 500 m square at 2.5 m
    p = param_gen.to_rp_params(sc["params"])
    assert sc["facets"].shape == (12, 200 * 200)
    assert sc["targets"].shape == (7, 2 * 10 * 10)
    assert p.nr == 16384 and abs(p.frequency - 60e6) < 1 and abs(p.bandwidth - 10e6) < 1
    assert p.ns == 250 and abs(p.sdx - 2.0) < 1e-12
    z = sc["targets"][2]
    assert (np.abs(z[:100] + 1000.0) < 60).all() and (np.abs(z[100:] + 3000.0) < 60).all()
    side = sc["facets"][0].max() - sc["facets"][0].min()
    assert abs(side - (500.0 - 2.5)) < 1e-6
