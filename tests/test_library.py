"""The C-ABI library: it loads, exports every symbol include/bsfit.h declares,
and rejects malformed calls with the reference's error classes before touching
a GPU (so these run on CPU-only machines too)."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT


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
    for st in range(0, 14):
        assert lib.bsfit_status_str(st)
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
