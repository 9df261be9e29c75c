"""GPU 4Pi fit against the oracle's 4Pi restatement (through the C ABI).

The reference's 4Pi fitter exists only as a compiled mex, so these tests
compare with the restated method (its likelihood pinned to the reference's
4D evaluation on CPU). Tolerances are those of the other fit types: x, y
1e-4 px, z 1e-2 nm, N and bg 1e-5 relative, phase 1e-4 knots, CRLB 1e-4
relative; like them, the GPU must agree with the FP64 oracle at least as
often as the oracle's own FP32 build does.
"""
import os

import numpy as np
import pytest

from test_fit_gpu import Z_NM_PER_UNIT, bsfit_mod, tol_pass  # noqa: F401

pytestmark = pytest.mark.gpu


def _wl(n, stream):
    from bsfit import workloads as W
    return W.workload_4pi(n=n, stream=stream)


def _host_fit(bsfit_mod, wl):
    ex = wl.extra
    return bsfit_mod.GPUmleFit_LM_4Pi_bspline(wl.rois, np.ones(6, np.uint32), wl.iterations,
                                              wl.coeff, ex["dT"], ex["init_z"], ex["init_phi"],
                                              ex["phase_shift"])


def test_4pi_eval_matches_oracle(bsfit_mod, oracle):
    """One evaluation at fixed parameters (the FP64 oracle's fit), with
    per-channel lateral offsets: deviance, gradient, Hessian, Fisher."""
    import torch
    wl = _wl(256, 801)
    ex = wl.extra
    rng = np.random.default_rng(3)
    dT = (rng.normal(0, 0.3, (wl.n_fits, 4, 6)) * np.array([1, 1, 0, 0, 0, 0])).astype(np.float32)
    R, _, _ = oracle.fit4pi(wl.rois, wl.iterations, wl.coeff, dT, ex["init_z"], ex["init_phi"],
                            ex["phase_shift"], precision="f64", threads=os.cpu_count() or 1)
    theta = R[:, :6].astype(np.float32)
    m = bsfit_mod.Model4Pi(wl.coeff, ex["phase_shift"])
    r = torch.from_numpy(wl.rois).cuda()
    th = torch.from_numpy(np.ascontiguousarray(theta.T)).cuda()
    d = torch.from_numpy(dT).cuda()
    nv = 6
    idx = [(l, k) for l in range(nv) for k in range(l, nv)]
    for fisher in (False, True):
        g = m.eval_torch(r, th, dT=d, fisher=fisher).cpu().numpy().astype(np.float64)
        ref = oracle.eval4pi(wl.rois, wl.coeff, dT, ex["phase_shift"], theta.astype(np.float64),
                             fisher=fisher)
        diag = np.stack([ref[:, 1 + nv + idx.index((k, k))] for k in range(nv)], 1)
        diag = np.maximum(diag, 1e-6 * np.median(diag, 0))
        e0 = np.abs(g[:, 0] - ref[:, 0]).max() / np.abs(ref[:, 0]).max()
        eJ = (np.abs(g[:, 1:1 + nv] - ref[:, 1:1 + nv]) / np.sqrt(diag)).max()
        eH = max((np.abs(g[:, 1 + nv + i] - ref[:, 1 + nv + i]) /
                  np.sqrt(diag[:, l] * diag[:, k])).max() for i, (l, k) in enumerate(idx))
        assert e0 < 1e-5 and eJ < 1e-3 and eH < 1e-3, (fisher, e0, eJ, eH)


def test_4pi_parity_at_scale(bsfit_mod, oracle):
    wl = _wl(3000, 802)
    ex = wl.extra
    P, C, L = _host_fit(bsfit_mod, wl)
    args = (wl.rois, wl.iterations, wl.coeff, ex["dT"], ex["init_z"], ex["init_phi"],
            ex["phase_shift"])
    threads = os.cpu_count() or 1
    R, RC, RL = oracle.fit4pi(*args, precision="f64", threads=threads)
    S, SC, SL = oracle.fit4pi(*args, precision="f32", threads=threads)
    ok = tol_pass(P, C, R, RC, 6)
    ok32 = tol_pass(S, SC, R, RC, 6)
    assert ok.mean() >= 0.5, ok.mean()
    assert ok.mean() >= ok32.mean() - 0.02, (ok.mean(), ok32.mean())
    assert np.median(np.abs(P[:, 0] - R[:, 0])) < 1e-5
    assert np.median(np.abs(P[:, 5] - R[:, 5])) < 1e-4
    assert np.median(np.abs(P[:, 4] - R[:, 4])) * Z_NM_PER_UNIT < 1e-3
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = np.abs(C / RC - 1)
    assert np.median(rel[np.isfinite(rel)]) < 1e-4
    assert np.median(np.abs(L - RL)) < 1e-3
    assert np.all(P[:, 5] >= 1.0) and np.all(P[:, 5] <= wl.coeff.shape[0] - 3)


def test_4pi_device_matches_host_call(bsfit_mod):
    import torch
    wl = _wl(500, 803)
    ex = wl.extra
    P, C, L = _host_fit(bsfit_mod, wl)
    m = bsfit_mod.Model4Pi(wl.coeff, ex["phase_shift"])
    cu = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    Pd, Cd, Ld = m.fit_torch(cu(wl.rois), wl.iterations, cu(ex["init_z"]), cu(ex["init_phi"]),
                             dT=cu(ex["dT"]))
    torch.cuda.synchronize()
    assert np.array_equal(Pd.cpu().numpy().T, P, equal_nan=True)
    assert np.array_equal(Cd.cpu().numpy().T, C, equal_nan=True)
    assert np.array_equal(Ld.cpu().numpy(), L, equal_nan=True)
    # no dT pointer means zero offsets
    Pz, _, _ = m.fit_torch(cu(wl.rois), wl.iterations, cu(ex["init_z"]), cu(ex["init_phi"]))
    torch.cuda.synchronize()
    assert np.array_equal(Pz.cpu().numpy().T, P, equal_nan=True)


def test_4pi_model_rejected_by_other_entry_points(bsfit_mod):
    import torch
    from bsfit import _native
    wl = _wl(8, 804)
    m = bsfit_mod.Model4Pi(wl.coeff, wl.extra["phase_shift"])
    r = torch.zeros((8, 13, 13), device="cuda")
    out = torch.zeros((8, 8), device="cuda")
    lib = _native.lib()
    st = lib.bsfit_fit_device(m._h, r.data_ptr(), 13, 8, 10, out.data_ptr(), out.data_ptr(),
                              out.data_ptr(), None)
    assert st == 5


def test_4pi_stated_configuration_parity(bsfit_mod, oracle):
    """The benchmark's stated 4Pi configuration (4 x 16 x 16 px ROIs, a 33 x 33
    x 61 x 16 sample grid periodic in phase, per-channel lateral offsets within
    +-0.5 px passed as dT, photons split over the channels): the GPU agrees with
    the FP64 restatement at least as often as the restatement's FP32 build, and
    the fits recover the simulated emitters to within their CRLB."""
    from bsfit import workloads as W
    wl = W.workload_4pi_c4(2000, stream=805)
    ex = wl.extra
    P, C, L = _host_fit(bsfit_mod, wl)
    args = (wl.rois, wl.iterations, wl.coeff, ex["dT"], ex["init_z"], ex["init_phi"],
            ex["phase_shift"])
    threads = os.cpu_count() or 1
    R, RC, RL = oracle.fit4pi(*args, precision="f64", threads=threads)
    S, SC, SL = oracle.fit4pi(*args, precision="f32", threads=threads)
    ok = tol_pass(P, C, R, RC, 6)
    ok32 = tol_pass(S, SC, R, RC, 6)
    assert ok.mean() >= 0.9, ok.mean()
    assert ok.mean() >= ok32.mean() - 0.02, (ok.mean(), ok32.mean())
    # the phase is periodic with 16 knots: compare it on the circle
    tr = wl.truth
    dw = (P[:, 5] - tr["w"] + 8.0) % 16.0 - 8.0
    for err, var in ((P[:, 0] - tr["x"], C[:, 0]), ((P[:, 4] - tr["z"]), C[:, 4]), (dw, C[:, 5])):
        z = err / np.sqrt(var)
        assert 0.55 < np.median(np.abs(z)) < 0.8, np.median(np.abs(z))
