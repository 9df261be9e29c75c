"""FP64 reference-precision fitter (bsfit_fit_f64_device) against the FP64
oracle and the reference's own FP64 outputs (golden fixtures).

The kernel evaluates the reference method in double in the reference's order
of operations, so its LM takes the double build's decisions: the per-ROI
agreement with the FP64 oracle (tolerances of tests/test_fit_gpu.py) is far
above the FP32 paths' (which match the reference's float build: a third of 4D
ROIs), and most ROIs agree bit for bit. The remaining differences come from
the last bit of log() (CUDA's against the C library's)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_cases
from test_fit_gpu import bsfit_mod, tol_pass  # noqa: F401

pytestmark = pytest.mark.gpu

NV = {6: 5, 7: 6, 8: 8}


def _fit64(bsfit_mod, fittype, rois, iterations, coeff, init_p=None, coeff3=None, var=None):
    import torch
    m = bsfit_mod.Model(fittype, coeff, coeff3=coeff3, init_p=init_p)
    r = torch.from_numpy(np.ascontiguousarray(rois, dtype=np.float32)).cuda()
    v = None if var is None else torch.from_numpy(np.ascontiguousarray(var, np.float32)).cuda()
    P, C, L = m.fit_f64_torch(r, iterations, var=v)
    torch.cuda.synchronize()
    return P.cpu().numpy().T, C.cpu().numpy().T, L.cpu().numpy()


@pytest.mark.parametrize("case", golden_cases())
def test_golden_fixture_f64(bsfit_mod, case):
    """Against the reference's own FP64 build (fixture outputs): every ROI of
    every case within the tolerances, iteration counts equal."""
    d = np.load(os.path.join(GOLDEN, case + ".npz"))
    ft = int(d["fittype"])
    nv = NV[ft]
    P, C, L = _fit64(bsfit_mod, ft, d["rois"], int(d["iterations"]), d["coeff"],
                     init_p=d["init_p"] if "init_p" in d else None,
                     coeff3=d["coeff3"] if "coeff3" in d else None)
    R, RC = d["f64_P"], d["f64_CRLB"]
    finite = np.isfinite(R).all(1)
    assert np.array_equal(np.isnan(P[:, :nv]), np.isnan(R[:, :nv])), case
    ok = tol_pass(P[finite], C[finite], R[finite], RC[finite], nv)
    frac = ok.mean() if ok.size else 1.0
    # one ROI of slack per case for a log() rounding flip
    assert ok.sum() >= ok.size - 1, (case, frac, np.where(~ok)[0])
    same_kk = (P[finite, nv] == R[finite, nv]).mean() if finite.any() else 1.0
    assert same_kk >= 0.95, (case, same_kk)


@pytest.mark.parametrize("fittype,n,min_frac", [(6, 20000, 0.995), (7, 3000, 0.97),
                                                (8, 320, 0.95)])
def test_f64_parity_at_scale(bsfit_mod, oracle, fittype, n, min_frac):
    from bsfit import workloads as W
    if fittype == 6:
        wl = W.workload_3d(n, s=13, stream=501)
    elif fittype == 7:
        wl = W.workload_4d(n, sizes=(13,), stream=502)[0]
    else:
        wl = W.workload_5d(n, stream=503)
    nv = NV[fittype]
    P, C, L = _fit64(bsfit_mod, fittype, wl.rois, wl.iterations, wl.coeff, init_p=wl.init_p,
                     coeff3=wl.coeff3)
    R, RC, RL = oracle.fit(wl.rois, fittype, wl.iterations, wl.coeff, precision="f64",
                           init_p=wl.init_p, coeff3=wl.coeff3, threads=os.cpu_count() or 1)
    ok = tol_pass(P, C, R, RC, nv)
    exact = np.all(P == R, axis=1)
    print(f"fit type {fittype}: {ok.mean():.4f} within tolerance, {exact.mean():.4f} bit-identical "
          f"parameters, iterations equal {np.mean(P[:, nv] == R[:, nv]):.4f}")
    assert ok.mean() >= min_frac, (ok.mean(), exact.mean())
    assert np.median(np.abs(L - RL)) <= 1e-9 * np.median(np.abs(RL))


def test_f64_scmos_parity(bsfit_mod, oracle):
    from bsfit import workloads as W
    from test_scmos import scmos_rois
    wl = W.workload_4d(1000, sizes=(13,), stream=963)[0]
    noisy, var = scmos_rois(wl)
    P, C, L = _fit64(bsfit_mod, 7, noisy, wl.iterations, wl.coeff, init_p=wl.init_p, var=var)
    R, RC, RL = oracle.fit(noisy, 7, wl.iterations, wl.coeff, init_p=wl.init_p, precision="f64",
                           threads=os.cpu_count() or 1, var=var)
    ok = tol_pass(P, C, R, RC, 6)
    same = np.all(P == R, axis=1)
    print(f"sCMOS fit type 7: {ok.mean():.4f} within tolerance, {same.mean():.4f} bit-identical")
    assert ok.mean() >= 0.99, ok.mean()
    assert same.mean() >= 0.99, same.mean()


def test_f64_rejects(bsfit_mod):
    import torch
    from bsfit import _native
    from bsfit import workloads as W
    lib = _native.lib()
    wl = W.workload_4pi(4, stream=964)
    m4 = bsfit_mod.Model4Pi(wl.coeff, wl.extra["phase_shift"])
    r = torch.zeros((4, 13, 13), device="cuda")
    out = torch.zeros((8, 4), device="cuda", dtype=torch.float64)
    p = out.data_ptr()
    assert lib.bsfit_fit_f64_device(m4._h, r.data_ptr(), None, 13, 4, 10, p, p, p, None) == 5
    w3 = W.workload_3d(4, s=13, stream=965)
    m = bsfit_mod.Model(6, w3.coeff)
    assert lib.bsfit_fit_f64_device(m._h, r.data_ptr(), None, 52, 4, 10, p, p, p, None) == 3
    assert lib.bsfit_fit_f64_device(m._h, None, None, 13, 4, 10, p, p, p, None) == 11
    assert lib.bsfit_fit_f64_device(m._h, r.data_ptr(), None, 13, 0, 10, p, p, p, None) == 0


@pytest.mark.parametrize("case", golden_cases())
def test_f64_dropin_host_call(bsfit_mod, case):
    """The host drop-in with precision="f64" (bsfit_GPUmleFit_LM_multiD_f64)
    returns the device entry point's results bit for bit; against the
    reference's own FP64 build (fixture) the parameters of every finite ROI are
    bit-identical up to log()-rounding flips (at most one ROI per case)."""
    d = np.load(os.path.join(GOLDEN, case + ".npz"))
    ft = int(d["fittype"])
    nv = NV[ft]
    kw = {}
    if "init_p" in d:
        kw["initP"] = d["init_p"]
    if "coeff3" in d:
        kw["coeff3"] = d["coeff3"]
    P, C, L = bsfit_mod.GPUmleFit_LM_multiD(d["rois"], ft, int(d["iterations"]), d["coeff"],
                                            precision="f64", **kw)
    assert P.dtype == np.float64 and C.dtype == np.float64 and L.dtype == np.float64
    Pd, Cd, Ld = _fit64(bsfit_mod, ft, d["rois"], int(d["iterations"]), d["coeff"],
                        init_p=d["init_p"] if "init_p" in d else None,
                        coeff3=d["coeff3"] if "coeff3" in d else None)
    assert np.array_equal(P, Pd, equal_nan=True)
    assert np.array_equal(C, Cd, equal_nan=True)
    assert np.array_equal(L, Ld, equal_nan=True)
    R = d["f64_P"]
    same = np.all((P == R) | (np.isnan(P) & np.isnan(R)), axis=1)
    print(f"{case}: {same.mean():.4f} of ROIs bit-identical to the reference's FP64 build")
    assert (~same).sum() <= 1, (case, np.where(~same)[0])


def test_f64_dropin_rejects(bsfit_mod):
    from bsfit import BsfitError
    from bsfit import workloads as W
    w3 = W.workload_3d(4, s=13, stream=966)
    with pytest.raises(BsfitError):
        bsfit_mod.GPUmleFit_LM_multiD(np.zeros((2, 52, 52), np.float32), 6, 10, w3.coeff,
                                      precision="f64")
    with pytest.raises(BsfitError):
        bsfit_mod.GPUmleFit_LM_multiD(w3.rois, 3, 10, w3.coeff, precision="f64")
    with pytest.raises(ValueError):
        bsfit_mod.GPUmleFit_LM_multiD(w3.rois, 6, 10, w3.coeff, precision="f16")


def test_f64_4pi_bit_identical_to_restatement(bsfit_mod, oracle):
    """The 4Pi fit in double (bsfit_fit4pi_f64_device) against the oracle's
    FP64 4Pi restatement: the same parameters bit for bit on the 4Pi parity
    workload (the reference's 4Pi fit exists only as a compiled mex, so the
    restatement is the method; its likelihood is pinned to the reference's
    fit type 7 in tests/test_4pi_oracle.py)."""
    import torch
    from bsfit import workloads as W
    wl = W.workload_4pi(n=3000, stream=802)
    ex = wl.extra
    m = bsfit_mod.Model4Pi(wl.coeff, ex["phase_shift"])
    cu = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()  # noqa: E731
    P, C, L = m.fit_f64_torch(cu(wl.rois), wl.iterations, cu(ex["init_z"]), cu(ex["init_phi"]),
                              cu(ex["dT"]))
    torch.cuda.synchronize()
    P, C, L = P.cpu().numpy().T, C.cpu().numpy().T, L.cpu().numpy()
    R, RC, RL = oracle.fit4pi(wl.rois, wl.iterations, wl.coeff, ex["dT"], ex["init_z"],
                              ex["init_phi"], ex["phase_shift"], precision="f64",
                              threads=os.cpu_count() or 1)
    same = np.all(P == R, axis=1)
    ok = tol_pass(P, C, R, RC, 6)
    print(f"4Pi: {same.mean():.4f} bit-identical, {ok.mean():.4f} within tolerance")
    assert same.mean() >= 0.99, same.mean()
    assert np.median(np.abs(L - RL)) <= 1e-9 * np.median(np.abs(RL))
