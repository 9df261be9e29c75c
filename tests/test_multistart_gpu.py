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
