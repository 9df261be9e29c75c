"""The oracle (CPU restatement of the reference method) against the golden
fixtures produced by the reference's own CPU fitter, and - where the reference
sources are present - against that fitter live on fresh seeded inputs.

Bit-exact: the restatement reproduces the reference's FP32 build and its
float-promoted FP64 build exactly."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_cases


def _load(case):
    d = np.load(os.path.join(GOLDEN, case + ".npz"))
    kw = {}
    if "init_p" in d:
        kw["init_p"] = d["init_p"]
    if "coeff3" in d:
        kw["coeff3"] = d["coeff3"]
    return d, kw


def _same(a, b):
    return np.array_equal(a, b, equal_nan=True)


@pytest.mark.parametrize("case", golden_cases())
@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_oracle_matches_golden(oracle, case, precision):
    d, kw = _load(case)
    P, C, L = oracle.fit(d["rois"], int(d["fittype"]), int(d["iterations"]), d["coeff"],
                         precision=precision, **kw)
    assert _same(P, d[f"{precision}_P"]), case
    assert _same(C, d[f"{precision}_CRLB"]), case
    assert _same(L, d[f"{precision}_LL"]), case


def _reference():
    from oracle.oracle import ReferenceOracle, reference_available
    from oracle import build
    if not reference_available() and build.build_reference() is None:
        pytest.skip("reference sources not present")
    return ReferenceOracle()


@pytest.mark.parametrize("fittype", [6, 7, 8])
def test_oracle_matches_reference_live(oracle, fittype):
    """Fresh seeded workloads at the benchmark grids, both precisions."""
    ref = _reference()
    from bsfit import workloads as W
    if fittype == 6:
        wl = W.workload_3d(300, s=13, stream=101)
    elif fittype == 7:
        wl = W.workload_4d(120, sizes=(15,), stream=102)[0]
    else:
        wl = W.workload_5d(6, stream=103)
    for prec in ("f32", "f64"):
        kw = dict(init_p=wl.init_p, coeff3=wl.coeff3, precision=prec)
        Pr, Cr, Lr = ref.fit(wl.rois, fittype, wl.iterations, wl.coeff, **kw)
        Po, Co, Lo = oracle.fit(wl.rois, fittype, wl.iterations, wl.coeff, threads=4, **kw)
        assert _same(Pr, Po) and _same(Cr, Co) and _same(Lr, Lo), (fittype, prec)


def test_basis_matches_reference(oracle):
    ref = _reference()
    xs = np.concatenate([np.linspace(-2.5, 2.5, 2001),
                         [-2, -1.5, -1, -0.5, 0, 0.5, 1, 1.5, 2],
                         np.nextafter(np.float32([-2, -1.5, -1, -0.5, 0, 0.5, 1, 1.5, 2]), -3),
                         ]).astype(np.float32)
    for deg in (2, 3):
        a = np.array([oracle.eval_bspline(float(x), deg) for x in xs], np.float32)
        b = np.array([ref.eval_bspline(float(x), deg) for x in xs], np.float32)
        assert np.array_equal(a, b)
