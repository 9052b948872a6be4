"""CUDA-graph capture of a whole fast-form call (rp_graph_*, through the C
ABI): the replay of the recorded call equals a direct rp_simulate_device call
bit for bit -- on the traces the graph was planned with, and on other traces
written into the same device buffer (the planned traces in reverse order, so
the graph's capacities and windows still hold) -- with the same counts, on a
single-segment and a multi-segment call, and replays repeat exactly; a whole
batch of scenes (rp_graph_create_batch) replays the direct batch call bit for
bit."""
import numpy as np
import pytest

from helpers import tiny_scene, vhf_scene

pytestmark = pytest.mark.gpu


def _bits(t):
    import torch
    return torch.view_as_real(t).contiguous().view(torch.int32)


def _direct(scene, d_tr):
    import torch
    out = torch.zeros((d_tr.shape[0], scene.nr), dtype=torch.complex64, device=d_tr.device)
    cnt = np.zeros((d_tr.shape[0], 2), np.int64)
    scene.simulate_device(d_tr, out, counts=cnt)
    torch.cuda.synchronize()
    return out, cnt


@pytest.mark.parametrize("kind", ["9MHz", "60MHz"])
def test_graph_replay_equals_direct_call(built_lib, kind):
    import torch
    from europaraypaths_gb300 import simulator
    sc = tiny_scene(nside=60, ntside=4, ns=6) if kind == "9MHz" else vhf_scene(4096, n_side=120, ns=5)
    with simulator.Scene(sc["params"], sc["facets"], sc["targets"]) as scene:
        tr = np.ascontiguousarray(scene.default_traces())
        d_tr = torch.from_numpy(tr).cuda()
        ref, cnt = _direct(scene, d_tr)
        assert cnt[:, 0].min() > 0 and cnt[:, 1].min() > 0
        out = torch.zeros_like(ref)
        g = scene.capture(tr, d_tr, out)
        try:
            for _ in range(2):
                out.fill_(complex(float("nan"), float("nan")))
                g.launch()
                assert np.array_equal(g.check(), cnt)
                assert torch.equal(_bits(out), _bits(ref))
            # other traces in the same buffer, within the planned bounds
            tr2 = np.ascontiguousarray(tr[::-1])
            d_tr.copy_(torch.from_numpy(tr2))
            ref2, cnt2 = _direct(scene, d_tr)
            out.zero_()
            g.launch()
            assert np.array_equal(g.check(), cnt2)
            assert torch.equal(_bits(out), _bits(ref2))
            assert torch.equal(_bits(out[0]), _bits(ref[-1]))
        finally:
            g.close()


def test_graph_multi_segment_call(built_lib):
    # 70 traces: two segments of one wave (the multi-job pair kernel, the
    # segments' setup and tail chains on the auxiliary streams), all in the
    # one graph
    import torch
    from europaraypaths_gb300 import simulator
    sc = tiny_scene(nside=24, ntside=3, ns=70)
    with simulator.Scene(sc["params"], sc["facets"], sc["targets"]) as scene:
        tr = np.ascontiguousarray(scene.default_traces())
        d_tr = torch.from_numpy(tr).cuda()
        ref, cnt = _direct(scene, d_tr)
        out = torch.zeros_like(ref)
        g = scene.capture(tr, d_tr, out)
        try:
            out.zero_()
            g.launch()
            assert np.array_equal(g.check(), cnt)
            assert torch.equal(_bits(out), _bits(ref))
        finally:
            g.close()


def test_graph_batch_equals_direct_batch(built_lib):
    # one rp_simulate_batch call over three scenes (9 MHz at 2048 and 1024
    # bins, 60 MHz at 4096 bins: a multi-segment wave, compression job tables
    # of two length classes) recorded as one graph
    import torch
    from europaraypaths_gb300 import simulator, scenes as scn
    scs = [tiny_scene(nside=40, ntside=4, ns=5),
           tiny_scene(nside=30, ntside=3, ns=3, eps_2=4.0, rx_window_m=scn.rx_window_for_bins(1024, 4e6)),
           vhf_scene(4096, n_side=120, ns=4)]
    scenes = [simulator.Scene(s["params"], s["facets"], s["targets"]) for s in scs]
    try:
        trs = [np.ascontiguousarray(sc.default_traces()) for sc in scenes]
        ref, cnt = simulator.simulate_batch(list(zip(scenes, trs)), return_counts=True)
        d_tr = [torch.from_numpy(t).cuda() for t in trs]
        d_out = [torch.zeros((t.shape[0], sc.nr), dtype=torch.complex64, device="cuda")
                 for t, sc in zip(trs, scenes)]
        g = simulator.capture_batch(list(zip(scenes, trs)), d_tr, d_out)
        try:
            for _ in range(2):
                for o in d_out:
                    o.fill_(complex(float("nan"), float("nan")))
                g.launch()
                assert np.array_equal(g.check(), np.concatenate(cnt))
                for o, r in zip(d_out, ref):
                    assert np.array_equal(o.cpu().numpy().view(np.uint32), np.ascontiguousarray(r).view(np.uint32))
        finally:
            g.close()
    finally:
        for sc in scenes:
            sc.close()
