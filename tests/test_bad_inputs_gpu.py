"""Malformed ROIs in a batch (NaN pixels, an infinite pixel, all-zero and
negative ROIs): the fit completes without an error for every fit type, in the
FP32 and the FP64 kernels and 4Pi, and every other ROI of the batch gets
exactly the results it gets in a clean batch (each ROI's fit is independent;
knots of non-finite positions clamp to the table, and every loop is bounded by
the iteration cap)."""
import numpy as np
import pytest

from test_fit_gpu import bsfit_mod  # noqa: F401

pytestmark = pytest.mark.gpu

BAD = (3, 7, 11, 13)


def _spoil(rois):
    r = rois.copy()
    r[3] = np.nan
    r[7, 2, 2] = np.inf
    r[11] = 0.0
    r[13] = -5.0
    return r


def _wl(fittype):
    from bsfit import workloads as W
    if fittype == 6:
        return W.workload_3d(64, s=13, stream=990)
    if fittype == 7:
        return W.workload_4d(64, sizes=(13,), stream=991)[0]
    return W.workload_5d(32, stream=992)


@pytest.mark.parametrize("precision", ["f32", "f64"])
@pytest.mark.parametrize("fittype", [6, 7, 8])
def test_bad_rois_leave_the_others_unchanged(bsfit_mod, fittype, precision):
    wl = _wl(fittype)
    kw = {"precision": precision}
    if wl.init_p is not None:
        kw["initP"] = wl.init_p
    if wl.coeff3 is not None:
        kw["coeff3"] = wl.coeff3
    good = bsfit_mod.GPUmleFit_LM_multiD(wl.rois, fittype, wl.iterations, wl.coeff, **kw)
    bad = bsfit_mod.GPUmleFit_LM_multiD(_spoil(wl.rois), fittype, wl.iterations, wl.coeff, **kw)
    keep = np.ones(len(wl.rois), bool)
    keep[list(BAD)] = False
    for g, b in zip(good, bad):
        assert np.array_equal(g[keep], b[keep], equal_nan=True)
    nv = {6: 5, 7: 6, 8: 8}[fittype]
    # iteration counts stay within the cap for the malformed ROIs too
    assert np.all(bad[0][:, nv][~keep] <= wl.iterations)


def test_bad_4pi_rois_leave_the_others_unchanged(bsfit_mod):
    import torch
    from bsfit import workloads as W
    wl = W.workload_4pi(n=32, stream=993)
    ex = wl.extra
    m = bsfit_mod.Model4Pi(wl.coeff, ex["phase_shift"])
    cu = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()  # noqa: E731
    bad_rois = wl.rois.copy()
    for c in range(4):
        bad_rois[c] = _spoil(bad_rois[c])
    outs = []
    for rois in (wl.rois, bad_rois):
        r = cu(rois)
        a = m.fit_torch(r, wl.iterations, cu(ex["init_z"]), cu(ex["init_phi"]), dT=cu(ex["dT"]))
        b = m.fit_f64_torch(r, wl.iterations, cu(ex["init_z"]), cu(ex["init_phi"]), cu(ex["dT"]))
        torch.cuda.synchronize()
        outs.append([x.cpu().numpy() for x in a + b])
    keep = np.ones(32, bool)
    keep[list(BAD)] = False
    for g, b in zip(*outs):
        assert np.array_equal(g[..., keep], b[..., keep], equal_nan=True)
