"""ctypes bindings for the oracle libraries (test infrastructure only).

``Oracle`` wraps ``liboracle.so`` (the restatement in ``bsfit_oracle.cpp``);
``ReferenceOracle`` wraps ``_ref/libref_{f32,f64}.so`` (the reference's CPU
fitter built by ``build_ref.sh``). Both expose the same ``fit`` call, shaped
like the reference mex: ``fit(rois, fittype, iterations, coeff, init_p,
coeff3, precision)`` -> (P, CRLB, LL) with P of shape (N, NV + 1) (last column
= iterations), CRLB (N, NV), LL (N,).
"""
import ctypes
import os

import numpy as np

from . import build as _build

NV = {6: 5, 7: 6, 8: 8}

_fp = ctypes.POINTER(ctypes.c_float)
_dp = ctypes.POINTER(ctypes.c_double)
_i = ctypes.c_int


def _ptr(a, dt):
    return a.ctypes.data_as(_fp if dt == np.float32 else _dp)


class _Base:
    def _call(self, fn_name, dt, rois, fittype, iterations, coeff, init_p, coeff3, threads,
              var=None):
        rois = np.ascontiguousarray(rois, dtype=dt)
        if rois.ndim == 2:
            rois = rois[None]
        n, s = rois.shape[0], rois.shape[-1]
        coeff = np.ascontiguousarray(coeff, dtype=dt)
        dims = list(reversed(coeff.shape))
        nv = NV[fittype]
        P = np.zeros((nv + 1, n), dtype=dt)
        C = np.zeros((nv, n), dtype=dt)
        L = np.zeros(n, dtype=dt)
        fn = getattr(self.lib(dt), fn_name)
        args = [_ptr(rois, dt)]
        if var is not None:
            v = np.ascontiguousarray(var, dtype=dt)
            assert v.shape == rois.shape
            args.append(_ptr(v, dt))
        args.append(_ptr(coeff, dt))
        if fittype == 8:
            c3 = np.ascontiguousarray(coeff3, dtype=dt)
            args.append(_ptr(c3, dt))
        args += [_i(d) for d in dims]
        args += [_i(s), _i(iterations)]
        keep = []
        if fittype in (7, 8):
            ip = np.ascontiguousarray(init_p, dtype=dt)
            keep.append(ip)
            args.append(_ptr(ip, dt))
        args += [_i(n), _ptr(P, dt), _ptr(C, dt), _ptr(L, dt)]
        if threads is not None:
            args.append(_i(threads))
        fn(*args)
        return P.T.copy(), C.T.copy(), L


class Oracle(_Base):
    """The CPU restatement (``liboracle.so``), FP32 or FP64. ``fma=True`` loads
    the build with FMA contraction (``liboracle_fma.so``; raises where the CPU
    has no FMA)."""

    def __init__(self, path=None, fma=False):
        if path is None and fma:
            path = _build.build_oracle_fma()
            if path is None:
                raise RuntimeError("no FMA on this CPU: the contracted oracle is not built")
        path = path or _build.build_oracle()
        self._lib = ctypes.CDLL(path)
        for fn in ("oracle_fit6_f32", "oracle_fit6_f64", "oracle_fit7_f32", "oracle_fit7_f64",
                   "oracle_fit8_f32", "oracle_fit8_f64"):
            getattr(self._lib, fn).restype = None
        self._lib.oracle_eval_bspline_f32.restype = ctypes.c_float
        self._lib.oracle_eval_bspline_f32.argtypes = [ctypes.c_float, ctypes.c_int]
        self._lib.oracle_eval_bspline_f64.restype = ctypes.c_double
        self._lib.oracle_eval_bspline_f64.argtypes = [ctypes.c_double, ctypes.c_int]

    def lib(self, dt):
        return self._lib

    def fit(self, rois, fittype, iterations, coeff, init_p=None, coeff3=None, precision="f32",
            threads=1, var=None):
        """var: sCMOS per-pixel variance / gain^2 (same shape as rois), or None."""
        dt = np.float32 if precision == "f32" else np.float64
        if var is not None:
            return self._call(f"oracle_fit{fittype}_scmos_{precision}", dt, rois, fittype,
                              iterations, coeff, init_p, coeff3, threads, var=var)
        return self._call(f"oracle_fit{fittype}_{precision}", dt, rois, fittype, iterations, coeff,
                          init_p, coeff3, threads)

    def eval_bspline(self, x, deg, precision="f32"):
        fn = self._lib.oracle_eval_bspline_f32 if precision == "f32" else self._lib.oracle_eval_bspline_f64
        return fn(x, deg)


def reference_available():
    return all(os.path.exists(os.path.join(_build.REF_DIR, f"libref_{p}.so")) for p in ("f32", "f64"))


class ReferenceOracle(_Base):
    """The reference CPU fitter compiled from its own sources (FP32 and the
    float-promoted FP64 build). Present only where the reference sources are."""

    def __init__(self):
        if not reference_available():
            _build.build_reference()
        self._libs = {np.float32: ctypes.CDLL(os.path.join(_build.REF_DIR, "libref_f32.so")),
                      np.float64: ctypes.CDLL(os.path.join(_build.REF_DIR, "libref_f64.so"))}
        self._libs[np.float32].ref_eval_bspline_f32.restype = ctypes.c_float
        self._libs[np.float32].ref_eval_bspline_f32.argtypes = [ctypes.c_float, ctypes.c_int]

    def lib(self, dt):
        return self._libs[dt]

    def fit(self, rois, fittype, iterations, coeff, init_p=None, coeff3=None, precision="f32"):
        dt = np.float32 if precision == "f32" else np.float64
        return self._call(f"ref_fit{fittype}_{precision}", dt, rois, fittype, iterations, coeff,
                          init_p, coeff3, None)

    def eval_bspline(self, x, deg):
        return self._libs[np.float32].ref_eval_bspline_f32(x, deg)


def _eval_entry(self, rois, fittype, coeff, theta, fisher=False, coeff3=None):
    """One evaluation per ROI at theta ((N, NV) array): returns (N, 1+NV+NH)
    float64 rows [value, gradient, packed upper-triangle Hessian/Fisher]."""
    rois = np.ascontiguousarray(rois, dtype=np.float64)
    n, s = rois.shape[0], rois.shape[-1]
    coeff = np.ascontiguousarray(coeff, dtype=np.float64)
    dims = list(reversed(coeff.shape))
    nv = NV[fittype]
    th = np.ascontiguousarray(np.asarray(theta, np.float64)[:, :nv].T)
    out = np.zeros((n, 1 + nv + nv * (nv + 1) // 2), np.float64)
    fn = getattr(self._lib, f"oracle_eval{fittype}_f64")
    args = [_ptr(rois, np.float64), _ptr(coeff, np.float64)]
    if fittype == 8:
        c3 = np.ascontiguousarray(coeff3, dtype=np.float64)
        args.append(_ptr(c3, np.float64))
    fn(*args, *[_i(d) for d in dims], _i(s), _i(n), _ptr(th, np.float64), _i(int(fisher)),
       _ptr(out, np.float64))
    return out


Oracle.eval = _eval_entry


def _trace(self, rois, fittype, iterations, coeff, roi, init_p=None, precision="f64"):
    """Per-iteration decision records of one ROI (see oracle_trace_f32)."""
    dt = np.float32 if precision == "f32" else np.float64
    rois = np.ascontiguousarray(rois, dtype=dt)
    n, s = rois.shape[0], rois.shape[-1]
    coeff = np.ascontiguousarray(coeff, dtype=dt)
    dims = (ctypes.c_int * 5)(*(list(reversed(coeff.shape)) + [1] * (5 - coeff.ndim)))
    nv = NV[fittype]
    P = np.zeros((nv + 1, n), dt); C = np.zeros((nv, n), dt); L = np.zeros(n, dt)
    tr = np.zeros((iterations + 1, 32), np.float64)
    ip = np.ascontiguousarray(init_p if init_p is not None else np.zeros(4), dtype=dt)
    fn = getattr(self._lib, f"oracle_trace_{precision}")
    fn(_i(fittype), _ptr(rois, dt), _ptr(coeff, dt), None, dims, _i(s), _i(iterations),
       _ptr(ip, dt), _i(roi), _i(n), _ptr(P, dt), _ptr(C, dt), _ptr(L, dt),
       tr.ctypes.data_as(_dp), _i(iterations + 1))
    return tr, P[:, roi], C[:, roi], L[roi]


Oracle.trace = _trace


def _fit4pi(self, rois, iterations, coeff, dT, init_z, init_phi, phase_shift, precision="f64",
            threads=1):
    """4Pi fit (oracle_fit4pi_*): rois (4, N, s, s); dT (N, 4, 6); init_z,
    init_phi (N,); phase_shift (4,). Returns P (N, 7), CRLB (N, 6), LL (N,)."""
    dt = np.float32 if precision == "f32" else np.float64
    rois = np.ascontiguousarray(rois, dtype=dt)
    n, s = rois.shape[1], rois.shape[-1]
    coeff = np.ascontiguousarray(coeff, dtype=dt)
    dims = (ctypes.c_int * 4)(*reversed(coeff.shape))
    arrs = [np.ascontiguousarray(a, dtype=dt) for a in (dT, init_z, init_phi, phase_shift)]
    P = np.zeros((7, n), dt)
    C = np.zeros((6, n), dt)
    L = np.zeros(n, dt)
    fn = getattr(self._lib, f"oracle_fit4pi_{precision}")
    fn(_ptr(rois, dt), _ptr(coeff, dt), dims, _i(s), _i(n), _i(iterations),
       *[_ptr(a, dt) for a in arrs], _ptr(P, dt), _ptr(C, dt), _ptr(L, dt), _i(threads))
    return P.T.copy(), C.T.copy(), L


def _eval4pi(self, rois, coeff, dT, phase_shift, theta, fisher=False):
    """One 4Pi evaluation per ROI at theta ((N, 6)): (N, 28) float64 rows."""
    rois = np.ascontiguousarray(rois, dtype=np.float64)
    n, s = rois.shape[1], rois.shape[-1]
    coeff = np.ascontiguousarray(coeff, dtype=np.float64)
    dims = (ctypes.c_int * 4)(*reversed(coeff.shape))
    d = np.ascontiguousarray(dT, dtype=np.float64)
    ps = np.ascontiguousarray(phase_shift, dtype=np.float64)
    th = np.ascontiguousarray(np.asarray(theta, np.float64)[:, :6].T)
    out = np.zeros((n, 28), np.float64)
    self._lib.oracle_eval4pi_f64(_ptr(rois, np.float64), _ptr(coeff, np.float64), dims, _i(s),
                                 _i(n), _ptr(d, np.float64), _ptr(ps, np.float64),
                                 _ptr(th, np.float64), _i(int(fisher)), _ptr(out, np.float64))
    return out


Oracle.fit4pi = _fit4pi
Oracle.eval4pi = _eval4pi
