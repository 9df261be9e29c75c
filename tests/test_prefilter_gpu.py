"""GPU coefficient builder (bsfit_bsarray_coeffs*) against the numpy
restatement of the reference's bsarray (bsfit/prefilter.py,
MultiD_bspline/bsarray/directFilter.m:200-298): the double coefficients agree
to rounding (different summation order of the causal initial value), the
float coefficients to one unit in the last place, the interpolation property
holds (the spline through the coefficients reproduces the samples), and the
fitter gives the same results with either set of coefficients."""
import numpy as np
import pytest

from test_fit_gpu import bsfit_mod  # noqa: F401

pytestmark = pytest.mark.gpu


def _cases():
    from bsfit import workloads as W
    rng = np.random.default_rng(5)
    yield "psf3d", W.psf3d_samples()[0]
    yield "psf4d", W.psf4d_samples()[0]
    yield "rand_odd", rng.random((7, 5, 9, 3))
    yield "rand_2", rng.random((2, 11, 6))
    yield "rand_1", rng.random((1, 4, 13))
    yield "line", rng.random(50)


@pytest.mark.parametrize("name,samples", list(_cases()))
def test_gpu_coefficients_match_restatement(bsfit_mod, name, samples):
    import torch
    from bsfit import prefilter
    ref = prefilter.bsarray_coeffs(samples)
    c32, c64 = bsfit_mod.bsarray_coeffs_torch(torch.from_numpy(np.ascontiguousarray(samples)).cuda(),
                                              out64=True)
    torch.cuda.synchronize()
    c64 = c64.cpu().numpy()
    c32 = c32.cpu().numpy()
    assert c64.shape == ref.shape
    scale = np.abs(ref).max()
    assert np.abs(c64 - ref).max() <= 1e-13 * scale, (name, np.abs(c64 - ref).max() / scale)
    # float copies: one unit in the last place, or the double bound near zero
    r32 = ref.astype(np.float32)
    ulp = np.maximum(np.spacing(np.abs(r32)), np.float32(1e-13 * scale))
    assert np.all(np.abs(c32 - r32) <= ulp), name
    # host entry point gives the same float coefficients
    h32 = bsfit_mod.bsarray_coeffs(samples)
    assert np.array_equal(h32, c32)


def test_interpolation_property(bsfit_mod):
    from bsfit import prefilter
    rng = np.random.default_rng(6)
    x = rng.random(40)
    c = bsfit_mod.bsarray_coeffs(x).astype(np.float64)
    # position m of the padded vector holds the knot at sample m - 1
    v = prefilter.eval_spline_1d(c, np.arange(40) + 1.0)
    assert np.abs(v - x).max() < 1e-5  # float32 coefficients


def test_fit_with_gpu_coefficients(bsfit_mod):
    """The 3D fit with coefficients built on the GPU equals the fit with the
    numpy-built ones where the float coefficients agree bit for bit."""
    from bsfit import workloads as W
    samples, _ = W.psf3d_samples()
    c_gpu = bsfit_mod.bsarray_coeffs(samples)
    c_np = W.coeff3d()
    wl = W.workload_3d(2000, s=13, stream=907)
    P1, C1, L1 = bsfit_mod.GPUmleFit_LM_multiD(wl.rois, 6, 30, c_np)
    P2, C2, L2 = bsfit_mod.GPUmleFit_LM_multiD(wl.rois, 6, 30, c_gpu)
    if np.array_equal(c_gpu, c_np):
        assert np.array_equal(P1, P2)
    else:
        assert np.median(np.abs(P1[:, 0] - P2[:, 0])) < 1e-4


def test_rejects(bsfit_mod):
    from bsfit import _native
    lib = _native.lib()
    assert lib.bsfit_bsarray_coeffs(None, 3, None, None) == 11
