"""Fused multi-start (bsfit_fit_multistart_device, bsfit_fit4pi_multistart_device)
against the reference callers' loop over single-start fits: fit from start 1,
refit from each further start, keep a ROI's new result when its
log-likelihood is higher by at least 1e-4 (by more than 1e-4 when strict),
MultiD_fitter/simplefitter_cspline.m:463-490, demo_orientation/store/fitb5n3.m:15-46,
demo_4pi/bspline_based_4piloc_v4.m:193-215. The fused kernel stages each ROI
once and runs all starts in one launch; its outputs must equal the loop's bit
for bit."""
import numpy as np
import pytest

from test_fit_gpu import bsfit_mod  # noqa: F401

pytestmark = pytest.mark.gpu


def compose(results, strict):
    """The callers' loop over per-start (P, CRLB, LL) numpy results."""
    P, C, L = (x.copy() for x in results[0])
    for Ph, Ch, Lh in results[1:]:
        d = (Lh - L).astype(np.float32)
        better = d > np.float32(1e-4) if strict else d >= np.float32(1e-4)
        P[:, better] = Ph[:, better]
        C[:, better] = Ch[:, better]
        L[better] = Lh[better]
    return P, C, L


def _np(t):
    return tuple(x.cpu().numpy() for x in t)


@pytest.mark.parametrize("strict", [False, True])
def test_multistart_4d_matches_loop(bsfit_mod, strict):
    import torch
    from bsfit import workloads as W
    wl = W.workload_4d(1500, sizes=(13,), stream=901)[0]
    z, w = float(wl.init_p[0]), float(wl.init_p[1])
    starts = np.array([[1.2 * z, w], [z, w], [0.8 * z, w]], np.float32)
    r = torch.from_numpy(wl.rois).cuda()
    m = bsfit_mod.Model(7, wl.coeff, init_p=wl.init_p)
    fused = _np(m.fit_multistart_torch(r, wl.iterations, starts, strict=strict))
    singles = [_np(bsfit_mod.Model(7, wl.coeff, init_p=st).fit_torch(r, wl.iterations))
               for st in starts]
    torch.cuda.synchronize()
    ref = compose(singles, strict)
    for a, b in zip(fused, ref):
        assert np.array_equal(a, b, equal_nan=True)
    # the starts matter: some ROIs take a later start's result
    assert np.any(fused[2] != singles[0][2])


def test_multistart_5d_matches_loop(bsfit_mod):
    import torch
    from bsfit import workloads as W
    wl = W.workload_5d(160, stream=902)
    s0 = wl.init_p.copy()
    s1 = wl.init_p.copy()
    s1[1] = W.phi_to_w(np.pi / 3)
    starts = np.stack([s0, s1]).astype(np.float32)
    r = torch.from_numpy(wl.rois).cuda()
    m = bsfit_mod.Model(8, wl.coeff, coeff3=wl.coeff3, init_p=wl.init_p)
    fused = _np(m.fit_multistart_torch(r, wl.iterations, starts))
    singles = [_np(bsfit_mod.Model(8, wl.coeff, coeff3=wl.coeff3, init_p=st).fit_torch(r, wl.iterations))
               for st in starts]
    torch.cuda.synchronize()
    for a, b in zip(fused, compose(singles, False)):
        assert np.array_equal(a, b, equal_nan=True)


def test_multistart_4pi_matches_loop(bsfit_mod):
    """The demo's two phase starts, 2 pi and pi (bspline_based_4piloc_v4.m:193)."""
    import torch
    from bsfit import workloads as W
    wl = W.workload_4pi(2000, stream=903)
    ex = wl.extra
    n = wl.n_fits
    phis = np.stack([np.full(n, 2 * np.pi / W.PHI_STEP), np.full(n, np.pi / W.PHI_STEP)]).astype(np.float32)
    zs = np.stack([ex["init_z"], ex["init_z"]]).astype(np.float32)
    cu = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    m = bsfit_mod.Model4Pi(wl.coeff, ex["phase_shift"])
    r = cu(wl.rois)
    fused = _np(m.fit_multistart_torch(r, wl.iterations, cu(zs), cu(phis), dT=cu(ex["dT"])))
    singles = [_np(m.fit_torch(r, wl.iterations, cu(zs[k]), cu(phis[k]), dT=cu(ex["dT"])))
               for k in range(2)]
    torch.cuda.synchronize()
    for a, b in zip(fused, compose(singles, False)):
        assert np.array_equal(a, b, equal_nan=True)
    # the second start rescues phase-ambiguous ROIs: the kept LL is never lower
    assert np.all(fused[2] >= singles[0][2] - 1e-6)


def test_multistart_rejects(bsfit_mod):
    import torch
    from bsfit import workloads as W
    wl = W.workload_3d(8, s=13, stream=904)
    m = bsfit_mod.Model(6, wl.coeff)
    r = torch.from_numpy(wl.rois).cuda()
    with pytest.raises(bsfit_mod.BsfitError) as e:
        m.fit_multistart_torch(r, 30, np.zeros((2, 2), np.float32))
    assert e.value.status == 5
    w4 = W.workload_4d(8, sizes=(13,), stream=905)[0]
    m4 = bsfit_mod.Model(7, w4.coeff, init_p=w4.init_p)
    r4 = torch.from_numpy(w4.rois).cuda()
    with pytest.raises(bsfit_mod.BsfitError) as e:
        m4.fit_multistart_torch(r4, 30, np.zeros((9, 2), np.float32))
    assert e.value.status == 11
    with pytest.raises(bsfit_mod.BsfitError) as e:
        m4.fit_multistart_torch(r4, 30, np.zeros((2, 1), np.float32))
    assert e.value.status == 10


@pytest.mark.parametrize("strict", [False, True])
def test_batched_multistart_matches_plain(bsfit_mod, strict):
    """Multi-start inside the persistent batched launch
    (bsfit_batch_fit_multistart_device): 4D segments of two ROI sizes and a 5D
    segment, each with its own starts, equal the plain fused multi-start of
    each segment bit for bit."""
    import torch
    from bsfit import workloads as W
    w13, w15 = W.workload_4d(600, sizes=(13, 15), stream=905)
    w5 = W.workload_5d(96, stream=906)
    z, w = float(w13.init_p[0]), float(w13.init_p[1])
    st4a = np.array([[1.2 * z, w], [z, w], [0.8 * z, w]], np.float32)
    st4b = np.array([[z, w], [0.9 * z, w]], np.float32)
    s1 = w5.init_p.copy()
    s1[1] = W.phi_to_w(np.pi / 3)
    st5 = np.stack([w5.init_p, s1]).astype(np.float32)
    m13 = bsfit_mod.Model(7, w13.coeff, init_p=w13.init_p)
    m15 = bsfit_mod.Model(7, w15.coeff, init_p=w15.init_p)
    m5 = bsfit_mod.Model(8, w5.coeff, coeff3=w5.coeff3, init_p=w5.init_p)
    r13, r15, r5 = (torch.from_numpy(x.rois).cuda() for x in (w13, w15, w5))
    entries = [(m13, r13, w13.iterations), (m15, r15, w15.iterations), (m5, r5, w5.iterations)]
    starts = [st4a, st4b, st5]
    b = bsfit_mod.Batch(entries, starts=starts, strict=strict)
    outs = [_np(o) for o in b.run()]
    plain = [_np(m.fit_multistart_torch(r, it, st, strict=strict))
             for (m, r, it), st in zip(entries, starts)]
    torch.cuda.synchronize()
    for o, p in zip(outs, plain):
        for a, c in zip(o, p):
            assert np.array_equal(a, c, equal_nan=True)
    claimed, done = b.counters()
    assert list(done) == [len(w13.rois), len(w15.rois), len(w5.rois)]


def test_batched_multistart_rejects(bsfit_mod):
    import torch
    from bsfit import BsfitError
    from bsfit import workloads as W
    w3 = W.workload_3d(64, s=13, stream=907)
    m = bsfit_mod.Model(6, w3.coeff)
    r = torch.from_numpy(w3.rois).cuda()
    with pytest.raises(BsfitError):  # fit type 6 has no initP: at most one start
        bsfit_mod.Batch([(m, r, 30)], starts=[[[1.0, 2.0], [3.0, 4.0]]]).run()
    # one start (or none) on a 3D segment is its plain fit
    one = [x.cpu().numpy() for x in bsfit_mod.Batch([(m, r, 30)], starts=[[]]).run()[0]]
    plain = [x.cpu().numpy() for x in m.fit_torch(r, 30)]
    for a_, b_ in zip(one, plain):
        assert np.array_equal(a_, b_, equal_nan=True)
    w4 = W.workload_4d(64, sizes=(13,), stream=908)[0]
    m4 = bsfit_mod.Model(7, w4.coeff, init_p=w4.init_p)
    with pytest.raises(ValueError):
        bsfit_mod.Batch([(m4, torch.from_numpy(w4.rois).cuda(), 60)], starts=[np.zeros((9, 2))])
