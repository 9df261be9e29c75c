"""The two-ROIs-per-warp forms of the 3D kernels (fit type 6: tuner variants 3
to 5, one ROI per half-warp; 6 and 7, both ROIs on all lanes in paired
operations) give the one-ROI form's outputs bit for bit at every ROI size:
small and large ROIs (one or two pixel chains per lane, windows of one or two
rounds), ROIs with NaN, zero and negative pixels (whose windows differ from the
other slot's), iteration caps of 0 and 1, an odd ROI count (one half of a warp
without a ROI), plain and batched with several sizes."""
import numpy as np
import pytest

from test_fit_gpu import bsfit_mod  # noqa: F401

pytestmark = pytest.mark.gpu

PAIR_VARIANTS = (3, 5, 6, 7)


def _rois(s, n, stream):
    from bsfit import workloads as W
    w = W.workload_3d(n, s=s, stream=stream)
    r = w.rois.copy()
    r[1] = np.nan
    r[2] = 0.0
    r[3] = -3.0
    r[4, s // 2, s // 2] = np.inf
    r[5, 0, 0] = np.nan
    return w, r


def _same(a, b):
    return all(np.array_equal(x, y, equal_nan=True) for x, y in zip(a, b))


@pytest.mark.parametrize("s", [5, 8, 11, 16, 17, 21, 33])
def test_pair_form_matches_one_roi_per_warp(bsfit_mod, s):
    import torch
    from bsfit import tuning as T
    n = 777 if s <= 21 else 201  # odd: the last warp has one half without a ROI
    w, r = _rois(s, n, 1200 + s)
    m = bsfit_mod.Model(6, w.coeff)
    d = torch.from_numpy(r).cuda()
    try:
        for it in (w.iterations, 1, 0):
            T._set(6, s, -1, 0)
            ref = [x.cpu().numpy() for x in m.fit_torch(d, it)]
            for v in PAIR_VARIANTS:
                for wpb in (4, 1):
                    T._set(6, s, v, wpb)
                    assert T.rois_per_warp(6, v) == 2
                    out = [x.cpu().numpy() for x in m.fit_torch(d, it)]
                    assert _same(out, ref), (s, it, v, wpb)
    finally:
        T._set(6, s, -1, 0)
    m.close()


def test_pair_form_batched_mixed_sizes(bsfit_mod):
    """Batched: segments of 11, 13 and 17 px (one of a single ROI), the pair form
    in force for the batch's largest size, against the default batched launch."""
    import torch
    from bsfit import tuning as T
    segs = []
    for k, (s, n) in enumerate([(17, 301), (11, 1), (13, 650), (11, 257)]):
        w, r = _rois(s, max(n, 6), 1300 + k)
        segs.append((w, torch.from_numpy(r[:n].copy()).cuda()))
    models = [bsfit_mod.Model(6, w.coeff) for w, _ in segs]
    entries = [(m, r, w.iterations) for m, (w, r) in zip(models, segs)]
    try:
        T._set(6, 17, -1, 0)
        b = bsfit_mod.Batch(entries)
        b.run()
        ref = [[x.cpu().numpy() for x in o] for o in b.outputs]
        for v in PAIR_VARIANTS:
            T._set(6, 17, v, 4)
            b = bsfit_mod.Batch(entries)
            b.run()
            for o, rf in zip(b.outputs, ref):
                assert _same([x.cpu().numpy() for x in o], rf), v
    finally:
        T._set(6, 17, -1, 0)
    for m in models:
        m.close()
