"""Frame -> ROI front end restated in numpy (test infrastructure only).

The reference's per-frame loop, MultiD_fitter/simplefitter_cspline.m:197-319:
  imphot = (single(image) - offset) * conversion                      (:226)
  impf   = filter2(h, imphot)                          Gaussian mode   (:244-246)
  impf   = filter2(h, imphot - min(imphot(:, 1)))      DoG mode        (:240-243)
  maxima = maximumfindcall(impf)      3x3 strict non-maximum suppression,
           MultiD_fitter/shared/maximumfind2.c:18-66 (raster order, columns
           outer, 1-based (x, y, value))
  keep value > cutoff, dx < x <= W - dx, dx < y <= H - dx              (:249-251)
  ROI k  = imphot(y-dx:y+dx, x-dx:x+dx) (x reversed when mirrored)     (:295-301)
with dx = floor(roifit / 2) (:136) and the kernels of :197-211:
  hgauss = fspecial('gaussian', max(3, ceil(3 sigma + 1)), sigma)
  hdog   = fspecial('gaussian', r, sigma) - fspecial('gaussian', r, max(1, 2.5 sigma)),
           r = max(ceil(6 sigma + 1), 3).
fspecial and filter2 are MATLAB built-ins; they are restated from their
documented definitions (a normalised Gaussian with values below eps * max set
to zero; 'same'-size correlation with zero padding). Arrays follow the
reference's layout: a frame stack is the C-order view (F, W, H) of MATLAB's
[H, W, F], i.e. pixel (y, x) of frame f at frames[f, x, y].
"""
import ctypes
import math
import os

import numpy as np

from . import build as _build


def fspecial_gaussian(hsize, sigma):
    """MATLAB fspecial('gaussian', hsize, sigma), float64, indexed [row][col]."""
    half = (hsize - 1) / 2.0
    ax = np.arange(hsize) - half
    x, y = np.meshgrid(ax, ax)
    h = np.exp(-(x * x + y * y) / (2.0 * sigma * sigma))
    h[h < np.finfo(np.float64).eps * h.max()] = 0.0
    s = h.sum()
    return h / s if s != 0 else h


def peak_kernel(mode, sigma):
    """The front end's filter kernel: mode 0 Gaussian, 1 difference of Gaussians."""
    if mode == 0:
        return fspecial_gaussian(max(3, int(math.ceil(3 * sigma + 1))), sigma)
    r = max(int(math.ceil(6 * sigma + 1)), 3)
    return fspecial_gaussian(r, sigma) - fspecial_gaussian(r, max(1.0, 2.5 * sigma))


def imphot(frames, offset, conversion):
    f = np.asarray(frames, dtype=np.float32)
    return (f - np.float32(offset)) * np.float32(conversion)


def filter2_same(h, img_xy):
    """filter2(h, X, 'same') for one frame given as (W, H) = [x][y], float64.

    Y(i, j) = sum_{u,v} h(u, v) X(i + u - o, j + v - o), o = (k - 1) div 2, i
    the row (y) and j the column (x); zero outside the image."""
    X = np.asarray(img_xy, dtype=np.float64).T  # [y][x]
    k = h.shape[0]
    o = (k - 1) // 2
    Hh, Ww = X.shape
    P = np.zeros((Hh + k - 1, Ww + k - 1))
    P[o:o + Hh, o:o + Ww] = X
    Y = np.zeros_like(X)
    for u in range(k):
        for v in range(k):
            if h[u, v] != 0.0:
                Y += h[u, v] * P[u:u + Hh, v:v + Ww]
    return Y.T  # back to [x][y]


def nms(impf_xy):
    """Strict 3x3 local maxima of one frame ([x][y]), in the reference's scan
    order (x outer, y inner, interior only): list of (x1, y1, value) 1-based.
    maximumfind2.c skips the pixel after a maximum, which can never be a
    strict maximum itself, so the mask below gives the same list."""
    a = np.asarray(impf_xy, dtype=np.float32)
    c = a[1:-1, 1:-1]
    m = np.ones_like(c, dtype=bool)
    for dxo in (-1, 0, 1):
        for dyo in (-1, 0, 1):
            if dxo == 0 and dyo == 0:
                continue
            m &= c > a[1 + dxo:a.shape[0] - 1 + dxo, 1 + dyo:a.shape[1] - 1 + dyo]
    xs, ys = np.nonzero(m)
    return [(int(x) + 2, int(y) + 2, float(c[x, y])) for x, y in zip(xs, ys)]


def find_rois(frames, offset, conversion, kernel, subtract_first_column_min, cutoff, roi_size,
              mirror=False, impf=None):
    """The whole front end for a (F, W, H) stack. Returns (rois (N, s, s) float32
    in the fitter's layout, coords (N, 3) = (x, y, frame) 1-based, impf).
    With impf given (a (F, W, H) filtered stack), the filter step is skipped and
    those values are used, so the maxima and cut-outs can be checked exactly
    against another implementation's filtered image."""
    ph = imphot(frames, offset, conversion)
    F, W, Hh = ph.shape
    dx = roi_size // 2
    if impf is None:
        impf = np.empty(ph.shape, np.float64)
        for f in range(F):
            x = ph[f]
            if subtract_first_column_min:
                x = x - x[0].min()
            impf[f] = filter2_same(kernel, x)
    rois, coords = [], []
    for f in range(F):
        for x1, y1, v in nms(impf[f]):
            if not (float(v) > cutoff):
                continue
            if not (x1 > dx and x1 <= W - dx and y1 > dx and y1 <= Hh - dx):
                continue
            x0, y0 = x1 - 1, y1 - 1
            cols = np.arange(x0 + dx, x0 - dx - 1, -1) if mirror else np.arange(x0 - dx, x0 + dx + 1)
            rois.append(ph[f][cols][:, y0 - dx:y0 + dx + 1])
            coords.append((x1, y1, f + 1))
    s = 2 * dx + 1
    R = np.array(rois, np.float32).reshape(-1, s, s)
    return R, np.array(coords, np.float64).reshape(-1, 3), impf


def reference_nms_available():
    return os.path.exists(os.path.join(_build.REF_DIR, "libref_maxfind.so"))


def reference_nms(impf_xy):
    """The reference's own NMS (maximumfind2.c, compiled by build_ref.sh) on one
    frame ([x][y] float32): list of (x1, y1, value)."""
    lib = ctypes.CDLL(os.path.join(_build.REF_DIR, "libref_maxfind.so"))
    fn = lib.NMS
    fn.restype = None
    fn.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_float),
                   ctypes.c_short, ctypes.c_short, ctypes.c_long]
    img = np.ascontiguousarray(impf_xy, dtype=np.float32)
    W, Hh = img.shape
    cap = W * Hh  # no maximum count can exceed it (the function does not check)
    out = np.zeros((3, cap), np.float64)
    fn(out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
       img.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), Hh, W, cap)
    n = int(np.argmax(out[0] == 0)) if np.any(out[0] == 0) else cap
    return [(int(out[0, k]), int(out[1, k]), float(out[2, k])) for k in range(n)]
