"""Host threads calling the library at the same time: the drop-in call keeps
its streams and events per thread, and a model's double tables for the FP64
kernel are built once under a lock, so concurrent calls give exactly the
results of the same calls made one after another."""
import threading

import numpy as np
import pytest

from test_fit_gpu import bsfit_mod  # noqa: F401

pytestmark = pytest.mark.gpu


def _run_threads(fns):
    out = [None] * len(fns)
    errs = []

    def work(i):
        try:
            out[i] = fns[i]()
        except Exception as e:  # reported below
            errs.append(e)

    ts = [threading.Thread(target=work, args=(i,)) for i in range(len(fns))]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout=300)
    assert not errs, errs
    return out


def test_concurrent_drop_in_calls(bsfit_mod):
    from bsfit import workloads as W
    wls = [W.workload_3d(20000, s=s, stream=1000 + s) for s in (11, 13, 17)]
    wls.append(W.workload_4d(4000, sizes=(13,), stream=1020)[0])

    def call(wl):
        kw = {"initP": wl.init_p} if wl.init_p is not None else {}
        P, C, L = bsfit_mod.GPUmleFit_LM_multiD(wl.rois, wl.fittype, wl.iterations, wl.coeff, **kw)
        return P.copy(), C.copy(), L.copy()

    alone = [call(w) for w in wls]
    together = _run_threads([lambda w=w: call(w) for w in wls])
    for a, b in zip(alone, together):
        for x, y in zip(a, b):
            assert np.array_equal(x, y, equal_nan=True)


def test_concurrent_first_fp64_use_of_one_model(bsfit_mod):
    import torch
    from bsfit import workloads as W
    wl = W.workload_3d(3000, s=13, stream=1030)
    m = bsfit_mod.Model(6, wl.coeff)
    r = torch.from_numpy(wl.rois).cuda()

    def call():
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            P, C, L = m.fit_f64_torch(r, wl.iterations, stream=s)
        s.synchronize()
        return P.cpu().numpy()

    outs = _run_threads([call for _ in range(4)])
    for o in outs[1:]:
        assert np.array_equal(o, outs[0], equal_nan=True)
    m2 = bsfit_mod.Model(6, wl.coeff)
    P2 = m2.fit_f64_torch(r, wl.iterations)[0].cpu().numpy()
    assert np.array_equal(P2, outs[0], equal_nan=True)
