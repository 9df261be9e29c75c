"""sCMOS likelihood in the oracle (CPU): with a zero variance map it is the
EMCCD fit bit for bit, and with read noise the variance-aware fit is closer to
the truth than the plain one on data that carry that noise."""
import numpy as np

from bsfit import workloads as W


def test_zero_variance_is_emccd(oracle):
    wl = W.workload_3d(200, s=13, stream=951)
    P, C, L = oracle.fit(wl.rois, 6, 30, wl.coeff, precision="f64")
    Pv, Cv, Lv = oracle.fit(wl.rois, 6, 30, wl.coeff, precision="f64",
                            var=np.zeros_like(wl.rois))
    assert np.array_equal(P, Pv) and np.array_equal(C, Cv) and np.array_equal(L, Lv)
    w4 = W.workload_4d(60, sizes=(13,), stream=952)[0]
    P, _, _ = oracle.fit(w4.rois, 7, w4.iterations, w4.coeff, init_p=w4.init_p, precision="f64")
    Pv, _, _ = oracle.fit(w4.rois, 7, w4.iterations, w4.coeff, init_p=w4.init_p, precision="f64",
                          var=np.zeros_like(w4.rois))
    assert np.array_equal(P, Pv)


def scmos_rois(wl, seed=7):
    rng = np.random.default_rng(seed)
    var = rng.uniform(1.0, 40.0, wl.rois.shape).astype(np.float32)
    noisy = (wl.rois + rng.normal(0.0, np.sqrt(var))).astype(np.float32)
    return noisy, var


def test_variance_aware_fit_is_closer(oracle):
    wl = W.workload_3d(400, s=13, stream=953)
    noisy, var = scmos_rois(wl)
    P0, _, _ = oracle.fit(noisy, 6, 30, wl.coeff, precision="f64", threads=8)
    Pv, _, _ = oracle.fit(noisy, 6, 30, wl.coeff, precision="f64", threads=8, var=var)
    e0 = np.median(np.abs(P0[:, 4] - wl.truth["z"]))
    ev = np.median(np.abs(Pv[:, 4] - wl.truth["z"]))
    assert ev <= e0 * 1.02, (ev, e0)
