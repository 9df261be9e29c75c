"""The device entry points inside a CUDA graph: after one warm-up call per ROI
size (which fills the launch-shape cache), a fit captured on a stream replays
with the captured inputs and gives the results of the direct call; the
batched fit too. The plain fit's work counter comes from the stream-ordered
pool, which graph capture records as memory nodes."""
import numpy as np
import pytest

from test_fit_gpu import bsfit_mod  # noqa: F401

pytestmark = pytest.mark.gpu


def test_captured_fit_replays(bsfit_mod):
    import torch
    from bsfit import workloads as W
    wl = W.workload_3d(20000, s=13, stream=1040)
    m = bsfit_mod.Model(6, wl.coeff)
    r = torch.from_numpy(wl.rois).cuda()
    out = (torch.empty((6, len(wl.rois)), device="cuda"), torch.empty((5, len(wl.rois)), device="cuda"),
           torch.empty((len(wl.rois),), device="cuda"))
    ref = [x.cpu().numpy().copy() for x in m.fit_torch(r, wl.iterations)]
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        m.fit_torch(r, wl.iterations, out=out, stream=s)  # warm-up
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    for x in out:
        x.zero_()
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=s):
        m.fit_torch(r, wl.iterations, out=out, stream=s)
    for x in out:
        x.zero_()
    g.replay()
    torch.cuda.synchronize()
    for a, b in zip(out, ref):
        assert np.array_equal(a.cpu().numpy(), b, equal_nan=True)
    # replay on new inputs written into the captured buffer
    w2 = W.workload_3d(20000, s=13, stream=1041)
    r.copy_(torch.from_numpy(w2.rois))
    g.replay()
    torch.cuda.synchronize()
    ref2 = [x.cpu().numpy() for x in m.fit_torch(torch.from_numpy(w2.rois).cuda(), wl.iterations)]
    for a, b in zip(out, ref2):
        assert np.array_equal(a.cpu().numpy(), b, equal_nan=True)


def test_captured_batch_replays(bsfit_mod):
    import torch
    from bsfit import workloads as W
    w13 = W.workload_3d(8000, s=13, stream=1042)
    w17 = W.workload_3d(4000, s=17, stream=1043)
    m = bsfit_mod.Model(6, w13.coeff)
    b = bsfit_mod.Batch([(m, torch.from_numpy(w13.rois).cuda(), 30),
                         (m, torch.from_numpy(w17.rois).cuda(), 30)])
    ref = [[x.cpu().numpy().copy() for x in o] for o in b.run()]
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        b.run(stream=s)
    for o in b.outputs:
        for x in o:
            x.zero_()
    g.replay()
    torch.cuda.synchronize()
    for o, rr in zip(b.outputs, ref):
        for x, y in zip(o, rr):
            assert np.array_equal(x.cpu().numpy(), y, equal_nan=True)


def test_captured_fp64_fit_replays(bsfit_mod):
    """The FP64 kernel too: the warm-up call builds the model's double tables and
    its launch shape, after which a capture records the launch alone."""
    import torch
    from bsfit import workloads as W
    wl = W.workload_3d(2000, s=13, stream=1044)
    m = bsfit_mod.Model(6, wl.coeff)
    r = torch.from_numpy(wl.rois).cuda()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        ref = [x.cpu().numpy().copy() for x in m.fit_f64_torch(r, wl.iterations, stream=s)]
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        out = m.fit_f64_torch(r, wl.iterations, stream=s)
    for x in out:
        x.zero_()
    g.replay()
    torch.cuda.synchronize()
    for a, b in zip(out, ref):
        assert np.array_equal(a.cpu().numpy(), b, equal_nan=True)
