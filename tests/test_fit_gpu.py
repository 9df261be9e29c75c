"""GPU parity of the CUDA fitter against the reference method.

Checks, through the C ABI on cuda:0:
  * the golden fixtures (outputs of the reference's own CPU fitter, FP32 and
    FP64 builds) and the oracle on the GPU machine;
  * seeded workloads at scale against the FP64 oracle, per ROI, with the
    tolerances of the reference method's precision budget:
        x, y within 1e-4 px; z within 1e-2 nm (5e-4 knot units on the 20 nm
        grid); photons and background within 1e-5 relative; extra dimensions
        within 1e-4; CRLB within 1e-4 relative (both "unidentifiable", i.e.
        > 1e25 or inf, also counts as agreement).
The LM trajectory of the reference method has discrete decisions (convergence
threshold, update-sign clamp halving, accept/reject, the 4D "let it go"
switch); rounding differences flip some of them, after which a ROI can end
elsewhere. The reference's own FP32 build differs from its FP64 build on such
ROIs too. The tests therefore bound the per-ROI pass fraction and require the
GPU to be at least as close to the FP64 oracle as the reference's FP32 build.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, Z_NM_PER_UNIT, golden_cases, tol_pass

pytestmark = pytest.mark.gpu



@pytest.fixture(scope="module")
def bsfit_mod():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()
    import bsfit
    return bsfit


def _fit(bsfit_mod, d):
    kw = {}
    if "init_p" in d:
        kw["initP"] = d["init_p"]
    if "coeff3" in d:
        kw["coeff3"] = d["coeff3"]
    return bsfit_mod.GPUmleFit_LM_multiD(d["rois"], int(d["fittype"]), int(d["iterations"]),
                                         d["coeff"], **kw)


def degenerate_rois(oracle, d):
    """ROIs whose FP64 reference trajectory passes through a (near-)singular
    Hessian: a solve step larger than 1e4 in x, y or z. There the reference's
    next move is decided by rounding noise of its double derivative sums
    (a tiny pivot, a huge step of noise-determined sign, cut to +-clamp), which
    no other arithmetic reproduces."""
    ft = int(d["fittype"])
    kw = {"init_p": d["init_p"]} if "init_p" in d else {}
    out = np.zeros(len(d["rois"]), bool)
    for r in range(len(d["rois"])):
        tr, *_ = oracle.trace(d["rois"], ft, int(d["iterations"]), d["coeff"], r, precision="f64",
                              **kw)
        steps = tr[:, [6, 7, 10]]
        out[r] = bool(np.any(np.abs(steps) > 1e4))
    return out


@pytest.mark.parametrize("case", golden_cases())
def test_golden_fixture(bsfit_mod, oracle, case):
    d = np.load(os.path.join(GOLDEN, case + ".npz"))
    ft = int(d["fittype"])
    nv = {6: 5, 7: 6, 8: 8}[ft]
    P, C, L = _fit(bsfit_mod, d)
    n = len(d["rois"])
    assert P.shape == (n, nv + 1) and C.shape == (n, nv) and L.shape == (n,)
    # the oracle on this machine still reproduces the reference's fixture
    kw = {k: d[k] for k in ("init_p", "coeff3") if k in d}
    Po, Co, Lo = oracle.fit(d["rois"], ft, int(d["iterations"]), d["coeff"], precision="f64", **kw)
    assert np.array_equal(Po, d["f64_P"], equal_nan=True)
    R, RC = d["f64_P"], d["f64_CRLB"]
    finite = np.isfinite(R).all(1)
    if int(d["iterations"]) == 0:
        # no LM step: the initial guesses and the CRLB pass only
        np.testing.assert_allclose(P[finite], R[finite].astype(np.float32), rtol=1e-5, atol=1e-5)
        return
    ok = tol_pass(P, C, R, RC, nv)
    ok32 = tol_pass(d["f32_P"], d["f32_CRLB"], R, RC, nv)
    keep = ~degenerate_rois(oracle, d) & finite
    # On ROIs with a regular reference trajectory: at least as close to the
    # FP64 reference as the reference's FP32 build, with one ROI in 8 of slack
    # for these small cases (one in 4 for fit type 7, whose "let it go" switch
    # and 1e-5 initial w clamp make its trajectory far more rounding-sensitive:
    # the reference's own FP32 and FP64 builds agree on only a third of 4D ROIs).
    slack = max(1, keep.sum() // (4 if ft in (7, 8) else 8))
    assert ok[keep].sum() >= ok32[keep].sum() - slack, (
        case, ok[keep].mean(), ok32[keep].mean(), np.where(keep & ~ok)[0])
    # Iteration counts are integers in the last column.
    assert np.all(P[:, nv] == np.round(P[:, nv])) and np.all(P[:, nv] <= int(d["iterations"]))


def test_special_rois_no_crash(bsfit_mod):
    """All-zero, negative, single-pixel and constant ROIs (m6_edges tail):
    finite where the reference is finite, NaN where it is NaN."""
    d = np.load(os.path.join(GOLDEN, "m6_edges.npz"))
    P, C, L = _fit(bsfit_mod, d)
    R = d["f64_P"]
    assert np.array_equal(np.isnan(P[:, :5]), np.isnan(R[:, :5]))


# Tolerance census of the FP32 kernels at every ROI size of the workloads (3D
# 11 / 13 / 17 px of the batched headline mix, 4D 13 / 15 px, 5D 17 px): the
# absolute fraction within the tolerances, and at least the fraction of the
# reference's own FP32 build on the same ROIs.
@pytest.mark.parametrize("fittype,s,n,min_frac,stream", [
    (6, 13, 20000, 0.955, 501), (6, 11, 5000, 0.94, 511), (6, 17, 5000, 0.94, 517),
    (7, 13, 3000, 0.33, 502), (7, 15, 3000, 0.30, 515), (8, 17, 2000, 0.30, 503)])
def test_parity_at_scale(bsfit_mod, oracle, fittype, s, n, min_frac, stream):
    from bsfit import workloads as W
    if fittype == 6:
        wl = W.workload_3d(n, s=s, stream=stream)
    elif fittype == 7:
        wl = W.workload_4d(n, sizes=(s,), stream=stream)[0]
    else:
        wl = W.workload_5d(n, s=s, stream=stream)
    nv = {6: 5, 7: 6, 8: 8}[fittype]
    kw = {"initP": wl.init_p} if wl.init_p is not None else {}
    if wl.coeff3 is not None:
        kw["coeff3"] = wl.coeff3
    P, C, L = bsfit_mod.GPUmleFit_LM_multiD(wl.rois, fittype, wl.iterations, wl.coeff, **kw)
    threads = os.cpu_count() or 1
    okw = dict(init_p=wl.init_p, coeff3=wl.coeff3, threads=threads)
    R, RC, RL = oracle.fit(wl.rois, fittype, wl.iterations, wl.coeff, precision="f64", **okw)
    S, SC, SL = oracle.fit(wl.rois, fittype, wl.iterations, wl.coeff, precision="f32", **okw)
    ok = tol_pass(P, C, R, RC, nv)
    ok32 = tol_pass(S, SC, R, RC, nv)
    assert ok.mean() >= min_frac, ok.mean()
    assert ok.mean() >= ok32.mean() - 0.02, (ok.mean(), ok32.mean())
    # Typical accuracy: 3D far inside the tolerances; 4D at the level of the
    # reference's own FP32 build (median |dz| 1.6e-3 nm against FP64).
    assert np.median(np.abs(P[:, 0] - R[:, 0])) < 1e-5
    zmed = np.median(np.abs(P[:, 4] - R[:, 4])) * Z_NM_PER_UNIT
    zmed32 = np.median(np.abs(S[:, 4] - R[:, 4])) * Z_NM_PER_UNIT
    assert zmed < (1e-3 if fittype == 6 else 2 * zmed32 + 1e-3), (zmed, zmed32)
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = np.abs(C / RC - 1)
    assert np.median(rel[np.isfinite(rel)]) < (1e-4 if fittype == 6 else 1e-3)
    assert np.median(np.abs(L - RL)) < 1e-3


def test_fit_device_matches_host_call(bsfit_mod):
    """The device-pointer entry point gives the same results as the host call."""
    import torch
    d = np.load(os.path.join(GOLDEN, "m6_basic.npz"))
    P, C, L = _fit(bsfit_mod, d)
    m = bsfit_mod.Model(6, d["coeff"])
    r = torch.from_numpy(d["rois"]).cuda()
    Pd, Cd, Ld = m.fit_torch(r, int(d["iterations"]))
    torch.cuda.synchronize()
    assert np.array_equal(Pd.cpu().numpy().T, P)
    assert np.array_equal(Cd.cpu().numpy().T, C)
    assert np.array_equal(Ld.cpu().numpy(), L)


def test_eval_matches_oracle_at_fixed_parameters(bsfit_mod, oracle):
    """One evaluation at the reference's final parameters: deviance, gradient,
    Hessian and Fisher information, trajectory-free. Gradient entry k is
    compared in units of sqrt(H_kk), Hessian entry (k, l) in units of
    sqrt(H_kk H_ll) (with a floor of 1e-6 of the column median, so an
    identically zero curvature on a boundary knot does not divide by zero)."""
    import torch
    for case in ("m6_basic", "m7_basic", "m8_basic"):
        d = np.load(os.path.join(GOLDEN, case + ".npz"))
        ft = int(d["fittype"])
        nv = {6: 5, 7: 6, 8: 8}[ft]
        theta = d["f64_P"][:, :nv].astype(np.float32)
        c3 = d["coeff3"] if "coeff3" in d else None
        m = bsfit_mod.Model(ft, d["coeff"], coeff3=c3, init_p=d["init_p"] if "init_p" in d else None)
        r = torch.from_numpy(d["rois"]).cuda()
        th = torch.from_numpy(np.ascontiguousarray(theta.T)).cuda()
        idx = [(l, k) for l in range(nv) for k in range(l, nv)]
        for fisher in (False, True):
            g = m.eval_torch(r, th, fisher=fisher).cpu().numpy().astype(np.float64)
            ref = oracle.eval(d["rois"], ft, d["coeff"], theta.astype(np.float64), fisher=fisher,
                              coeff3=c3)
            diag = np.stack([ref[:, 1 + nv + idx.index((k, k))] for k in range(nv)], 1)
            diag = np.maximum(diag, 1e-6 * np.median(diag, 0))
            e0 = np.abs(g[:, 0] - ref[:, 0]).max() / np.abs(ref[:, 0]).max()
            eJc = (np.abs(g[:, 1:1 + nv] - ref[:, 1:1 + nv]) / np.sqrt(diag)).max(0)
            eHc = [(np.abs(g[:, 1 + nv + i] - ref[:, 1 + nv + i]) /
                    np.sqrt(diag[:, l] * diag[:, k])).max() for i, (l, k) in enumerate(idx)]
            # The 5D mixture sums 64 coefficients per node and two correction
            # maps; its FP32 derivative error is a few 1e-3 of the curvature
            # scale where a curvature is small.
            tol = 1e-3 if ft != 8 else 1e-2
            assert e0 < 1e-5 and eJc.max() < tol and max(eHc) < tol, (
                case, fisher, e0, eJc.round(5).tolist(), np.round(eHc, 5).tolist())


def test_batch_matches_plain(bsfit_mod):
    """Segments of mixed ROI sizes and fit types in one batched call give the
    same results as one plain call per segment, and every ROI is claimed and
    finished exactly once."""
    import torch
    from bsfit import workloads as W
    g3 = W.workload_3d_mixed(3000, sizes=(11, 13, 17), ratio=(1, 2, 1), stream=601)
    g4 = W.workload_4d(400, sizes=(13,), stream=602)[0]
    g5 = W.workload_5d(40, stream=603)
    m3 = bsfit_mod.Model(6, g3[0].coeff)
    m4 = bsfit_mod.Model(7, g4.coeff, init_p=g4.init_p)
    m5 = bsfit_mod.Model(8, g5.coeff, coeff3=g5.coeff3, init_p=g5.init_p)
    entries = [(m3, torch.from_numpy(g.rois).cuda(), g.iterations) for g in g3]
    entries.append((m4, torch.from_numpy(g4.rois).cuda(), g4.iterations))
    entries.append((m5, torch.from_numpy(g5.rois).cuda(), g5.iterations))
    b = bsfit_mod.Batch(entries)
    outs = b.run()
    torch.cuda.synchronize()
    claimed, finished = b.counters()
    n = np.array([e[1].shape[0] for e in entries])
    assert np.all(finished == n) and np.all(claimed >= n)
    for (m, r, it), (P, C, L) in zip(entries, outs):
        Pp, Cp, Lp = m.fit_torch(r, it)
        torch.cuda.synchronize()
        assert np.array_equal(P.cpu().numpy(), Pp.cpu().numpy(), equal_nan=True)
        assert np.array_equal(C.cpu().numpy(), Cp.cpu().numpy(), equal_nan=True)
        assert np.array_equal(L.cpu().numpy(), Lp.cpu().numpy(), equal_nan=True)


def test_batch_rejects_bad_arguments(bsfit_mod):
    from bsfit import _native
    lib = _native.lib()
    assert lib.bsfit_batch_fit_device(None, 49, None, 0, None) == 11
    assert lib.bsfit_batch_scratch_bytes(3) == 256
