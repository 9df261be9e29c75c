"""GPU frame -> ROI front end (bsfit_find_rois_device) against the restatement
of the reference's per-frame loop (oracle/frontend.py, whose non-maximum
suppression is pinned to the reference's maximumfind2.c): the filter agrees
with a float64 filter2 to FP32 rounding; given the GPU's own filtered frames,
the maxima, their order, coordinates and the cut-out ROIs are identical; and
planted emitters are all found."""
import numpy as np
import pytest

from test_fit_gpu import bsfit_mod  # noqa: F401

pytestmark = pytest.mark.gpu

OFFSET, CONV = 100.0, 0.5


def _movie(F=5, H=96, W=128, n_spots=10, seed=41):
    """ADU frames (F, W, H) with Poisson background and well-separated spots;
    returns frames and the planted (frame, x0, y0) centres (0-based pixels)."""
    from bsfit import workloads as W_
    rng = np.random.default_rng(seed)
    frames = np.empty((F, W, H), np.float32)
    spots = []
    for f in range(F):
        lam = np.full((W, H), 12.0)
        gx_c = rng.choice(np.arange(12, W - 12, 16), n_spots // 2, replace=False)
        gy_c = rng.choice(np.arange(12, H - 12, 16), n_spots // 2, replace=False)
        for x0, y0 in zip(gx_c, gy_c):
            x = x0 + rng.uniform(-0.4, 0.4)
            y = y0 + rng.uniform(-0.4, 0.4)
            z = rng.uniform(-300, 300)
            sx, sy = W_.astig_sigmas(np.array([z]), 1.3)
            gx = W_._int_gauss(np.array([x]), sx, W)[0]
            gy = W_._int_gauss(np.array([y]), sy, H)[0]
            lam += 3000.0 * gx[:, None] * gy[None, :]
            spots.append((f, int(x0), int(y0)))
        photons = rng.poisson(lam)
        frames[f] = (photons / CONV + OFFSET).astype(np.float32)
    return frames, spots


@pytest.mark.parametrize("mode,sigma,mirror", [(1, 1.0, False), (0, 1.2, False), (1, 1.5, True)])
def test_frontend_matches_restatement(bsfit_mod, mode, sigma, mirror):
    import torch
    from oracle import frontend as FE
    frames, spots = _movie()
    h = bsfit_mod.peak_kernel(mode, sigma)
    np.testing.assert_allclose(h, FE.peak_kernel(mode, sigma), rtol=1e-6, atol=1e-9)
    cutoff = 2.0 if mode == 1 else 30.0
    rois, coords, filt = bsfit_mod.find_rois_torch(torch.from_numpy(frames).cuda(), OFFSET, CONV, h,
                                                   dog=(mode == 1), cutoff=cutoff, roi_size=13,
                                                   mirror=mirror, filtered=True)
    torch.cuda.synchronize()
    rois, coords, filt = rois.cpu().numpy(), coords.cpu().numpy(), filt.cpu().numpy()
    # the filter: FP32 accumulation against float64
    ph = FE.imphot(frames, OFFSET, CONV)
    for f in range(frames.shape[0]):
        x = ph[f] - (ph[f][0].min() if mode == 1 else 0.0)
        ref = FE.filter2_same(FE.peak_kernel(mode, sigma), x)
        assert np.abs(filt[f] - ref).max() <= 2e-5 * np.abs(ref).max()
    # maxima, order, coordinates and ROIs from the same filtered frames
    R, C, _ = FE.find_rois(frames, OFFSET, CONV, None, mode == 1, cutoff, 13, mirror=mirror,
                           impf=filt)
    assert len(C) > 0
    assert np.array_equal(coords, C.astype(np.float32))
    assert np.array_equal(rois, R)
    # every planted spot has a ROI within one pixel
    found = {(int(f) - 1, int(x) - 1, int(y) - 1) for x, y, f in coords}
    for f, x0, y0 in spots:
        assert any(ff == f and abs(xx - x0) <= 1 and abs(yy - y0) <= 1 for ff, xx, yy in found)


def test_frontend_capacity_and_empty(bsfit_mod):
    import torch
    frames, _ = _movie(F=2)
    h = bsfit_mod.peak_kernel(1, 1.0)
    fr = torch.from_numpy(frames).cuda()
    r_all, c_all = bsfit_mod.find_rois_torch(fr, OFFSET, CONV, h, True, 2.0, 13)
    r_cap, c_cap = bsfit_mod.find_rois_torch(fr, OFFSET, CONV, h, True, 2.0, 13, capacity=3)
    torch.cuda.synchronize()
    assert len(c_cap) == 3 and torch.equal(c_cap, c_all[:3]) and torch.equal(r_cap, r_all[:3])
    r0, c0 = bsfit_mod.find_rois_torch(fr, OFFSET, CONV, h, True, 1e30, 13)
    assert len(c0) == 0


def test_frontend_rejects(bsfit_mod):
    import torch
    fr = torch.zeros((1, 32, 32), device="cuda")
    with pytest.raises(bsfit_mod.BsfitError) as e:
        bsfit_mod.find_rois_torch(fr, 0, 1, np.ones((3, 3)), False, 0.0, 12)
    assert e.value.status == 3
