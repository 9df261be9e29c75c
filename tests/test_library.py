"""The C-ABI library: it loads, exports every symbol include/bsfit.h declares,
and rejects malformed calls with the reference's error classes before touching
a GPU (so these run on CPU-only machines too)."""
import os
import re

import numpy as np
import pytest

from conftest import PKG, ROOT


def _declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "bsfit.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    return sorted(set(re.findall(r"\b(bsfit_\w+)\s*\(", hdr)))


@pytest.fixture(scope="module")
def lib():
    from bsfit import build, _native
    build.build()
    return _native.lib()


def test_exports_every_declared_symbol(lib):
    names = _declared_symbols()
    assert "bsfit_GPUmleFit_LM_multiD" in names and "bsfit_fit_device" in names
    for n in names:
        assert hasattr(lib, n), n


def test_binding_matches_header():
    from bsfit import _native
    assert sorted(_native.SIGNATURES) == _declared_symbols()


def test_status_strings(lib):
    for st in range(0, 15):
        assert lib.bsfit_status_str(st) != b"unknown status"
    assert b"square" in lib.bsfit_status_str(4)


def _call(rois, fittype=6, coeff=None, **kw):
    import bsfit
    if coeff is None:
        coeff = np.zeros((10, 9, 9), np.float32)
    return bsfit.GPUmleFit_LM_multiD(rois, fittype, 30, coeff, **kw)


def test_rejects_large_roi():
    import bsfit
    with pytest.raises(bsfit.BsfitError) as e:
        _call(np.zeros((2, 52, 52), np.float32))
    assert e.value.status == 3


def test_rejects_nonsquare_roi():
    import bsfit
    with pytest.raises(bsfit.BsfitError) as e:
        _call(np.zeros((2, 13, 12), np.float32))
    assert e.value.status == 4


@pytest.mark.parametrize("fittype", [1, 2, 3, 4, 5, 9])
def test_rejects_other_fittypes(fittype):
    import bsfit
    with pytest.raises(bsfit.BsfitError) as e:
        _call(np.zeros((2, 13, 13), np.float32), fittype=fittype)
    assert e.value.status == 5


def test_num_params(lib):
    assert [lib.bsfit_num_params(t) for t in (5, 6, 7, 8)] == [0, 5, 6, 8]


def _call4pi(shared=(1, 1, 1, 1, 1, 1), channels=4, n=2, s=13, **kw):
    import bsfit
    im = np.zeros((channels, n, s, s), np.float32)
    args = dict(shared=np.asarray(shared, np.uint32), iterations=100,
                coeff=np.zeros((12, 10, 9, 9), np.float32), dT=np.zeros((n, 4, 6), np.float32),
                initZ=np.zeros(n, np.float32), initPhi=np.ones(n, np.float32),
                phase_shift=np.zeros(4, np.float32))
    args.update(kw)
    return bsfit.GPUmleFit_LM_4Pi_bspline(im, **args)


@pytest.mark.parametrize("shared", [(1, 1, 1, 1, 1, 0), (0, 1, 1, 1, 1, 1), (1, 1, 1)])
def test_4pi_rejects_unshared(shared):
    import bsfit
    with pytest.raises(bsfit.BsfitError) as e:
        _call4pi(shared=shared)
    assert e.value.status == 14


def test_4pi_rejects_channel_count():
    import bsfit
    with pytest.raises(bsfit.BsfitError) as e:
        _call4pi(channels=3)
    assert e.value.status == 14


def test_4pi_rejects_short_inputs():
    import bsfit
    with pytest.raises(bsfit.BsfitError) as e:
        _call4pi(dT=np.zeros((1, 4, 6), np.float32))
    assert e.value.status == 1
    with pytest.raises(bsfit.BsfitError) as e:
        _call4pi(s=52)
    assert e.value.status == 3


def test_batch_entry_points_reject_before_any_device_work(lib):
    """Argument checks of the batched entries that need no GPU: an empty batch
    is a no-op, too many segments and a missing starts array are refused."""
    from bsfit import _native
    segs = (_native.Segment * 1)()
    st = (_native.Starts * 1)()
    assert lib.bsfit_batch_fit_device(None, 0, None, 0, None) == 0
    assert lib.bsfit_batch_fit_device(segs, 49, None, 0, None) == 11
    assert lib.bsfit_batch_fit_multistart_device(segs, None, 1, None, 0, None) == 10
    assert lib.bsfit_batch_fit_multistart_device(segs, st, 0, None, 0, None) == 0
    assert lib.bsfit_batch_fit_multistart_device(segs, st, 49, None, 0, None) == 11
    assert lib.bsfit_batch_scratch_bytes(3) >= 3 * 16


def test_fp64_entry_points_reject_before_any_device_work(lib):
    """The FP64 entries refuse a missing model or arguments the reference's
    mex refuses (ROI larger than 51, non-square, unsupported fit type) before
    any CUDA call."""
    d = np.zeros(3 * 52 * 52, np.float32)
    out = np.zeros(100, np.float64)
    p = out.ctypes.data
    assert lib.bsfit_fit_f64_device(None, None, None, 13, 4, 10, p, p, p, None) == 11
    dims = (np.ctypeslib.ctypes.c_int64 * 3)(29, 29, 64)
    c = np.zeros(29 * 29 * 64, np.float32)
    fp = np.ctypeslib.ctypes.POINTER(np.ctypeslib.ctypes.c_float)
    args = lambda s1, s2, ft: (d.ctypes.data_as(fp), s1, s2, 3, ft, 10, c.ctypes.data_as(fp), 3,  # noqa: E731
                               dims, None, 0, 1, None, 0, None, 0, None, p, p, p)
    assert lib.bsfit_GPUmleFit_LM_multiD_f64(*args(52, 52, 6)) == 3   # SubregionSize
    assert lib.bsfit_GPUmleFit_LM_multiD_f64(*args(13, 12, 6)) == 4   # SubregionShape
    assert lib.bsfit_GPUmleFit_LM_multiD_f64(*args(13, 13, 3)) == 5   # unsupported fit type
    assert lib.bsfit_GPUmleFit_LM_multiD_f64(None, 13, 13, 3, 6, 10, c.ctypes.data_as(fp), 3, dims,
                                             None, 0, 1, None, 0, None, 0, None, p, p, p) == 2


def test_cpu_call_name_is_the_drop_in():
    import inspect
    import bsfit
    a = inspect.signature(bsfit.CPUmleFit_LM).parameters
    b = inspect.signature(bsfit.GPUmleFit_LM_multiD).parameters
    assert list(a) == list(b)


def test_double_float_log_table():
    """The double-float kernels' logarithm table (bsfit_fitdd.cu, kLogTab):
    entry j holds log(1 + j/128) as the nearest float and the nearest float to
    the remainder, so hi + lo is within 2^-48 of the value. Recomputed here
    with 50-digit decimal arithmetic."""
    import re
    from decimal import Decimal, getcontext
    getcontext().prec = 50
    src = open(os.path.join(PKG, "csrc", "bsfit_fitdd.cu")).read()
    body = src[src.index("kLogTab[129] = {"):]
    body = body[:body.index("};")]
    pairs = re.findall(r"\{([-+0-9.e]+)f, ([-+0-9.e]+)f\}", body)
    assert len(pairs) == 129
    for j, (hi, lo) in enumerate(pairs):
        exact = (Decimal(1) + Decimal(j) / Decimal(128)).ln()
        h, l_ = np.float32(hi), np.float32(lo)
        assert h == np.float32(float(exact)), j
        assert l_ == np.float32(float(exact - Decimal(float(h)))), j
        assert abs(Decimal(float(h)) + Decimal(float(l_)) - exact) < Decimal(2) ** -48, j
