"""The coefficient builder pinned to the reference's bsarray recursion.

Expected coefficients come from a literal restatement, written out here with
1-based loops, of the reference's MATLAB code for the cubic, lambda = 0 case:

- MultiD_bspline/bsarray/getBSplineFiltCoeffs.m:219-224: one pole
  z = sqrt(3) - 2 and the gain C0 = 6;
- MultiD_bspline/bsarray/directFilter.m:44, :255-273: per MATLAB dimension
  d = 1 .. ndims in order (MATLAB dimension 1 is the fastest axis, the last of
  a C-order array), K0 = ceil(log(eps) / log|z|), the index vector
  KVec = [1:N, N-1:-1:2] repeated and cut to K0, the scale
  c0 = -z / (1 - z^2), the filter applied to every line along d, then the
  whole array multiplied by the gain;
- MultiD_bspline/bsarray/symExpFilt.m:27-44: Y(1) = sum_k z^(k-1) X(KVec(k)),
  Y(k) = X(k) + z Y(k-1), Y(N) = (2 Y(N) - X(N)) c0, Y(k) = (Y(k+1) - Y(k)) z;
- directFilter.m:286-298: the pad by floor(3/2) = 1 along every dimension,
  index dimNums(mod(-1:N, 2N-2) + 1) with dimNums = [1:N, N-1:-1:2].

It is independent of bsfit/prefilter.py (the numpy restatement the other
builder tests use). The CPU test checks that restatement against it; the GPU
test checks the GPU builder's float coefficients to one unit in the last place
on every element, edge planes included. A constant stack, whose interpolating
spline is that constant, is the hand-checked case: every coefficient equals it.
"""
import math

import numpy as np
import pytest

from conftest import PKG  # noqa: F401


def _sym_exp_filt(X, z, c0, K0, KVec):
    N = len(X) - 1  # X and Y are 1-based (element 0 unused)
    Y = [0.0] * (N + 1)
    for k in range(1, K0 + 1):
        Y[1] = Y[1] + (z ** (k - 1)) * X[KVec[k - 1]]
    for k in range(2, N + 1):
        Y[k] = X[k] + z * Y[k - 1]
    Y[N] = (2 * Y[N] - X[N]) * c0
    for k in range(N - 1, 0, -1):
        Y[k] = (Y[k + 1] - Y[k]) * z
    return Y


def matlab_bsarray_cubic(samples):
    """bsarray(samples) coefficients, degree 3, lambda 0, as the reference's
    MATLAB computes them (see the module docstring). samples: C order, the
    reference's fastest axis last; every axis of length >= 2."""
    C = np.array(samples, dtype=np.float64)
    nd = C.ndim
    z = math.sqrt(3.0) - 2.0
    gain = 6.0
    K0 = math.ceil(math.log(np.finfo(np.float64).eps) / math.log(abs(z)))
    c0 = -z / (1.0 - z * z)
    for d in range(1, nd + 1):           # MATLAB dimension d
        axis = nd - d                    # the C-order axis it is
        N = C.shape[axis]
        ind_reflect = list(range(1, N + 1)) + list(range(N - 1, 1, -1))
        reps = math.ceil(K0 / (2 * N - 2))
        KVec = (ind_reflect * reps)[:K0]
        moved = np.moveaxis(C, axis, -1)
        flat = moved.reshape(-1, N)
        for row in range(flat.shape[0]):
            X = [0.0] + list(flat[row])   # 1-based
            Y = _sym_exp_filt(X, z, c0, K0, KVec)
            flat[row] = Y[1:]
        C = np.moveaxis(flat.reshape(moved.shape), -1, axis).copy()
        C = C * gain
    for axis in range(nd):
        M = C.shape[axis]
        dim_nums = list(range(1, M + 1)) + list(range(M - 1, 1, -1))
        idx = [dim_nums[(p % (2 * M - 2))] - 1 for p in range(-1, M + 1)]
        C = np.take(C, idx, axis=axis)
    return C


def _cases():
    rng = np.random.default_rng(17)
    yield "rand3", rng.random((5, 4, 6))
    yield "rand4", rng.random((3, 4, 2, 5)) * 100.0
    yield "line", rng.random(7)
    yield "two", rng.random((2, 3))


def test_numpy_restatement_matches_matlab_recursion():
    from bsfit import prefilter
    for name, x in _cases():
        exp = matlab_bsarray_cubic(x)
        got = prefilter.bsarray_coeffs(x)
        assert got.shape == exp.shape == tuple(n + 2 for n in x.shape)
        assert np.abs(got - exp).max() <= 1e-14 * np.abs(exp).max(), name


def test_constant_stack_gives_constant_coefficients():
    exp = matlab_bsarray_cubic(np.full((4, 5, 6), 3.25))
    assert exp.shape == (6, 7, 8)
    assert np.abs(exp - 3.25).max() < 1e-13


@pytest.mark.gpu
def test_gpu_builder_matches_matlab_recursion():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()
    import bsfit
    cases = list(_cases()) + [("const", np.full((4, 5, 6), 3.25))]
    for name, x in cases:
        exp = matlab_bsarray_cubic(x)
        c32, c64 = bsfit.bsarray_coeffs_torch(torch.from_numpy(np.ascontiguousarray(x)).cuda(),
                                              out64=True)
        torch.cuda.synchronize()
        c32, c64 = c32.cpu().numpy(), c64.cpu().numpy()
        assert np.abs(c64 - exp).max() <= 1e-13 * np.abs(exp).max(), name
        e32 = exp.astype(np.float32)
        ulp = np.spacing(np.abs(e32))
        assert np.all(np.abs(c32.astype(np.float64) - e32.astype(np.float64)) <= ulp), name
        # the edge planes (the mirror pad) along every axis
        for ax in range(x.ndim):
            for plane in (0, c32.shape[ax] - 1):
                a = np.take(c32, plane, axis=ax).astype(np.float64)
                b = np.take(e32, plane, axis=ax).astype(np.float64)
                u = np.spacing(np.abs(np.take(e32, plane, axis=ax)))
                assert np.all(np.abs(a - b) <= u), (name, ax, plane)
