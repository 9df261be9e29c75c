"""Cubic B-spline coefficient builder (CPU, numpy, float64).

Restates the reference's coefficient producer ``bsarray`` for the case the
fitter consumes: degree 3 along every axis, no smoothing (lambda = 0).

- ``MultiD_bspline/bsarray/directFilter.m:200-282``: per axis, the direct
  B-spline filter is a symmetric exponential filter with pole
  z = sqrt(3) - 2 (``getBSplineFiltCoeffs.m:45-50``), followed by the gain
  6 = (1 - z)(1 - 1/z).
- ``MultiD_bspline/bsarray/symExpFilt.m:27-44``: causal pass initialised with a
  truncated mirror sum of K0 = ceil(log(eps) / log|z|) terms
  (``directFilter.m:255``); anticausal pass initialised with
  (2 y[N-1] - x[N-1]) * (-z / (1 - z^2)).
- ``directFilter.m:286-298``: the result is padded by floor(3 / 2) = 1 sample
  on each side by whole-sample mirroring (c[-1] = c[1], c[N] = c[N-2]), so the
  coefficient array is two larger than the sample array along every axis.

The GPU fitter reads exactly this layout: coefficient index m along an axis
holds the knot at sample position m - 1.
"""
import math

import numpy as np

POLE = math.sqrt(3.0) - 2.0
GAIN = 6.0
K0 = int(math.ceil(math.log(np.finfo(np.float64).eps) / math.log(abs(POLE))))


def _mirror_indices(n, k0):
    # [0..n-1, n-2..1] repeated, as KVec in directFilter.m:261-263.
    if n == 1:
        return np.zeros(k0, dtype=np.int64)
    period = np.concatenate([np.arange(n), np.arange(n - 2, 0, -1)])
    reps = int(math.ceil(k0 / len(period)))
    return np.tile(period, reps)[:k0]


def filter_axis(a, axis):
    """Mirror-boundary cubic prefilter of ``a`` along ``axis`` (float64)."""
    x = np.moveaxis(np.asarray(a, dtype=np.float64), axis, 0)
    n = x.shape[0]
    if n == 1:
        return np.moveaxis(x.copy(), 0, axis)
    z = POLE
    y = np.empty_like(x)
    kvec = _mirror_indices(n, K0)
    powers = z ** np.arange(K0)
    y[0] = np.tensordot(powers, x[kvec], axes=(0, 0))
    for k in range(1, n):
        y[k] = x[k] + z * y[k - 1]
    c0 = -z / (1.0 - z * z)
    y[n - 1] = (2.0 * y[n - 1] - x[n - 1]) * c0
    for k in range(n - 2, -1, -1):
        y[k] = (y[k + 1] - y[k]) * z
    y *= GAIN
    return np.moveaxis(y, 0, axis)


def filter_axis_periodic(a, axis):
    """Periodic cubic prefilter along ``axis`` (exact, via the DFT).

    Used for an axis that the fitter wraps (the azimuth axis of the 5D model):
    the coefficients interpolate the samples on a circle.
    """
    x = np.moveaxis(np.asarray(a, dtype=np.float64), axis, 0)
    n = x.shape[0]
    # B3 at integer shifts: 1/6, 4/6, 1/6.
    h = np.zeros(n)
    h[0] = 4.0 / 6.0
    h[1 % n] += 1.0 / 6.0
    h[-1 % n] += 1.0 / 6.0
    hf = np.fft.fft(h)
    c = np.fft.ifft(np.fft.fft(x, axis=0) / hf.reshape((n,) + (1,) * (x.ndim - 1)), axis=0).real
    return np.moveaxis(c, 0, axis)


def mirror_pad(c, axes=None):
    """Whole-sample mirror pad by one along each axis (directFilter.m:286-298)."""
    axes = range(c.ndim) if axes is None else axes
    out = c
    for ax in axes:
        n = out.shape[ax]
        if n == 1:
            idx = np.array([0, 0, 0])
        else:
            idx = np.concatenate([[1], np.arange(n), [n - 2]])
        out = np.take(out, idx, axis=ax)
    return out


def bsarray_coeffs(samples):
    """Coefficients of the interpolating cubic spline of ``samples``.

    ``samples`` is indexed with the reference's fastest axis LAST (C order of
    a MATLAB column-major array reversed), i.e. shape (..., Z, X, Y). Returns a
    float64 array two larger along every axis.
    """
    c = np.asarray(samples, dtype=np.float64)
    for ax in range(c.ndim):
        c = filter_axis(c, ax)
    return mirror_pad(c)


def eval_spline_1d(c, pos):
    """Evaluate a padded 1D coefficient vector at padded positions (float64)."""
    pos = np.asarray(pos, dtype=np.float64)
    k = np.floor(pos).astype(np.int64)
    t = pos - k
    out = np.zeros_like(pos)
    for off in (-1, 0, 1, 2):
        out += c[np.clip(k + off, 0, len(c) - 1)] * _b3(t - off)
    return out


def _b3(x):
    ax = np.abs(x)
    return np.where(ax < 1, 2.0 / 3.0 - ax ** 2 + 0.5 * ax ** 3,
                    np.where(ax < 2, (2.0 - ax) ** 3 / 6.0, 0.0))
