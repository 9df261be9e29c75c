"""bsfit: GB300-native B-spline PSF MLE fitter (fit types 6, 7, 8 and the 4Pi fit).

Python mirror of the reference's MATLAB call surface over the C ABI of
libbsfit.so:

    P, CRLB, LL = GPUmleFit_LM_multiD(imstack, fittype, iterations, coeff,
                                      varmap, silent, initP, coeff3)

``imstack`` is a float32 array of shape (N, s, s) (the C-order view of the
MATLAB [s, s, N] stack) or (s, s); ``coeff`` is the C-order view of the MATLAB
coefficient array (shape (..., Z, X, Y)). Outputs: P (N, NV + 1) with the
iteration count last, CRLB (N, NV), LL (N,), all float32.
"""
import numpy as np

from . import _native
from ._native import BsfitError, check

NUM_PARAMS = {6: 5, 7: 6, 8: 8}
FIT_4PI = 9  # model tag of 4Pi models (BSFIT_FITTYPE_4PI)

_fp = _native._fp


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _dims(a):
    return (np.ctypeslib.ctypes.c_int64 * a.ndim)(*reversed(a.shape))


def GPUmleFit_LM_multiD(imstack, fittype, iterations=50, coeff=None, varmap=0, silent=1,
                        initP=None, coeff3=None, out=None, precision="f32"):
    """Drop-in for the reference mex (fit types 6, 7, 8); raises BsfitError.

    Returns (P, CRLB, LL) shaped (N, NV + 1), (N, NV), (N,): views of the C
    ABI's column-major outputs (no copy). precision="parity" runs the
    double-float kernels (bsfit_GPUmleFit_LM_multiD_parity): float32 outputs
    that follow the reference's FP64 trajectory as closely as a second FP64
    build of it. out=(P, CRLB, LL) passes caller-owned
    buffers in the C ABI's layout ((NV + 1, N), (NV, N), (N,)), which are
    filled and returned as the same views, as a host application calling the C
    ABI directly would reuse its buffers. precision="f64" runs the FP64
    reference-precision kernel (bsfit_GPUmleFit_LM_multiD_f64) and returns
    float64 results, those of the reference method computed in double."""
    lib = _native.lib()
    im = _f32(imstack)
    if im.ndim == 2:
        im = im[None]
    if im.ndim != 3:
        raise ValueError("imstack must be (N, s, s) or (s, s)")
    n, s2, s1 = im.shape
    fittype = int(fittype)
    nv = NUM_PARAMS.get(fittype, 0)
    c = _f32(coeff) if coeff is not None else None
    c3 = _f32(coeff3) if coeff3 is not None else None
    ip = _f32(np.atleast_1d(initP)) if initP is not None else None
    vm = _f32(np.atleast_1d(varmap)) if varmap is not None else None
    if precision not in ("f32", "f64", "parity"):
        raise ValueError("precision must be 'f32', 'parity' or 'f64'")
    dt = np.float64 if precision == "f64" else np.float32
    if out is None:
        P = np.empty((max(nv, 1) + 1, n), dt)
        C = np.empty((max(nv, 1), n), dt)
        L = np.empty(n, dt)
    else:
        P, C, L = out
        assert P.shape == (nv + 1, n) and C.shape == (nv, n) and L.shape == (n,)
        assert all(x.dtype == dt and x.flags.c_contiguous for x in (P, C, L))
    ptr = lambda a: a.ctypes.data_as(_fp) if a is not None else None  # noqa: E731
    optr = (lambda a: a.ctypes.data) if precision == "f64" else (lambda a: a.ctypes.data_as(_fp))
    fn = {"f32": lib.bsfit_GPUmleFit_LM_multiD, "parity": lib.bsfit_GPUmleFit_LM_multiD_parity,
          "f64": lib.bsfit_GPUmleFit_LM_multiD_f64}[precision]
    st = fn(
        ptr(im), s1, s2, n, fittype, int(iterations),
        ptr(c), c.ndim if c is not None else 0, _dims(c) if c is not None else None,
        ptr(vm), vm.size if vm is not None else 0, int(silent),
        ptr(ip), ip.size if ip is not None else 0,
        ptr(c3), c3.ndim if c3 is not None else 0, _dims(c3) if c3 is not None else None,
        optr(P), optr(C), optr(L))
    check(st, "GPUmleFit_LM_multiD")
    return P.T, C.T, L


def CPUmleFit_LM(imstack, fittype, iterations=50, coeff=None, varmap=0, silent=1, initP=None,
                 coeff3=None, out=None, precision="f32"):
    """The reference's CPU mex has the same call as GPUmleFit_LM_multiD
    (VC/CPUmleFit_LM/mexFunction.cpp:130-263), and the CUDA kernels here follow
    the CPU method (its initial guesses, clamps, bounds and consistent x/y use),
    so a CPUmleFit_LM caller switches by name: this is GPUmleFit_LM_multiD.
    precision="f64" returns the CPU method's double-precision results bit for
    bit."""
    return GPUmleFit_LM_multiD(imstack, fittype, iterations, coeff, varmap, silent, initP, coeff3,
                               out=out, precision=precision)


class Model:
    """A PSF model whose coefficient tables stay resident on the device."""

    def __init__(self, fittype, coeff, coeff3=None, init_p=None, tune_cache=None):
        """tune_cache: a tuning cache file (bsfit.tuning); its choices for this
        device are put in force for the fits of every model."""
        lib = _native.lib()
        self.fittype = int(fittype)
        self.nv = NUM_PARAMS[self.fittype]
        c = _f32(coeff)
        c3 = _f32(coeff3) if coeff3 is not None else None
        ip = _f32(np.atleast_1d(init_p)) if init_p is not None else None
        h = np.ctypeslib.ctypes.c_void_p()
        st = lib.bsfit_model_create(
            self.fittype, c.ctypes.data_as(_fp), c.ndim, _dims(c),
            c3.ctypes.data_as(_fp) if c3 is not None else None, c3.ndim if c3 is not None else 0,
            _dims(c3) if c3 is not None else None,
            ip.ctypes.data_as(_fp) if ip is not None else None, ip.size if ip is not None else 0,
            np.ctypeslib.ctypes.byref(h))
        check(st, "bsfit_model_create")
        self._h = h
        if tune_cache is not None:
            from . import tuning
            tuning.apply_cache(tune_cache, tuning.device_name())

    def fit_device(self, d_rois, roi_size, nfits, iterations, d_P, d_CRLB, d_LL, stream=0,
                   precision="f32", exact_steps=-1):
        """Asynchronous fit with raw device pointers (ints) on a CUDA stream;
        precision="parity" runs the double-float kernels (exact_steps: leading
        LM steps in the FP64 reference order, -1 the default per fit type)."""
        lib = _native.lib()
        if precision == "parity":
            st = lib.bsfit_fit_parity_steps_device(self._h, d_rois, roi_size, nfits, iterations,
                                                   int(exact_steps), d_P, d_CRLB, d_LL, stream)
            check(st, "bsfit_fit_parity_steps_device")
            return
        st = lib.bsfit_fit_device(self._h, d_rois, roi_size, nfits, iterations, d_P, d_CRLB,
                                  d_LL, stream)
        check(st, "bsfit_fit_device")

    def fit_torch(self, rois, iterations, out=None, stream=None, precision="f32", exact_steps=-1):
        """Fit a CUDA float32 tensor (N, s, s); returns (P, CRLB, LL) tensors in
        the reference's column-major layout: P (NV+1, N), CRLB (NV, N), LL (N).
        precision="parity" runs the double-float kernels."""
        import torch
        assert rois.is_cuda and rois.dtype == torch.float32 and rois.is_contiguous()
        n, s = rois.shape[0], rois.shape[-1]
        if out is None:
            P = torch.empty((self.nv + 1, n), device=rois.device, dtype=torch.float32)
            C = torch.empty((self.nv, n), device=rois.device, dtype=torch.float32)
            L = torch.empty((n,), device=rois.device, dtype=torch.float32)
        else:
            P, C, L = out
        st = stream if stream is not None else torch.cuda.current_stream(rois.device)
        self.fit_device(rois.data_ptr(), s, n, int(iterations), P.data_ptr(), C.data_ptr(),
                        L.data_ptr(), st.cuda_stream, precision=precision, exact_steps=exact_steps)
        return P, C, L

    def fit_scmos_torch(self, rois, var, iterations, stream=None):
        """sCMOS fit: var (same shape as rois) holds the per-pixel variance /
        gain^2, added to model and data in the likelihood. Returns (P, CRLB,
        LL) device tensors as fit_torch."""
        import torch
        assert rois.is_cuda and var.is_cuda and rois.shape == var.shape
        r, v = rois.contiguous(), var.contiguous()
        n, s = r.shape[0], r.shape[-1]
        P = torch.empty((self.nv + 1, n), device=r.device, dtype=torch.float32)
        C = torch.empty((self.nv, n), device=r.device, dtype=torch.float32)
        L = torch.empty((n,), device=r.device, dtype=torch.float32)
        cs = stream if stream is not None else torch.cuda.current_stream(r.device)
        check(_native.lib().bsfit_fit_scmos_device(self._h, r.data_ptr(), v.data_ptr(), s, n,
                                                   int(iterations), P.data_ptr(), C.data_ptr(),
                                                   L.data_ptr(), cs.cuda_stream),
              "bsfit_fit_scmos_device")
        return P, C, L

    def fit_f64_torch(self, rois, iterations, var=None, stream=None):
        """FP64 reference-precision fit (fit types 6, 7, 8): the reference's
        method in double with its order of operations. rois: float32 device
        tensor (N, s, s); var: optional sCMOS variance of the same shape.
        Returns (P (NV+1, N), CRLB (NV, N), LL (N,)) float64 device tensors."""
        import torch
        assert rois.is_cuda and rois.dtype == torch.float32
        r = rois.contiguous()
        v = None
        if var is not None:
            assert var.is_cuda and var.dtype == torch.float32 and var.shape == rois.shape
            v = var.contiguous()
        n, s = r.shape[0], r.shape[-1]
        P = torch.empty((self.nv + 1, n), device=r.device, dtype=torch.float64)
        C = torch.empty((self.nv, n), device=r.device, dtype=torch.float64)
        L = torch.empty((n,), device=r.device, dtype=torch.float64)
        cs = stream if stream is not None else torch.cuda.current_stream(r.device)
        check(_native.lib().bsfit_fit_f64_device(
            self._h, r.data_ptr(), v.data_ptr() if v is not None else None, s, n,
            int(iterations), P.data_ptr(), C.data_ptr(), L.data_ptr(), cs.cuda_stream),
            "bsfit_fit_f64_device")
        return P, C, L

    def fit_multistart_torch(self, rois, iterations, starts, strict=False, stream=None):
        """Fused multi-start fit (fit types 7, 8): starts is a sequence of initP
        vectors; every ROI is fitted from each and the best log-likelihood kept
        (a later start wins when its LL is higher by >= 1e-4, > 1e-4 if strict).
        Returns (P (NV+1, N), CRLB (NV, N), LL (N,)) device tensors."""
        import torch
        assert rois.is_cuda and rois.dtype == torch.float32 and rois.is_contiguous()
        st_ = _f32(np.atleast_2d(starts))
        n, s = rois.shape[0], rois.shape[-1]
        P = torch.empty((self.nv + 1, n), device=rois.device, dtype=torch.float32)
        C = torch.empty((self.nv, n), device=rois.device, dtype=torch.float32)
        L = torch.empty((n,), device=rois.device, dtype=torch.float32)
        cs = stream if stream is not None else torch.cuda.current_stream(rois.device)
        check(_native.lib().bsfit_fit_multistart_device(
            self._h, rois.data_ptr(), s, n, int(iterations), st_.ctypes.data_as(_fp),
            st_.shape[1], st_.shape[0], int(bool(strict)), P.data_ptr(), C.data_ptr(),
            L.data_ptr(), cs.cuda_stream), "bsfit_fit_multistart_device")
        return P, C, L

    def trace_torch(self, rois, iterations, flags=0, trace_max=None):
        """Fit with per-iteration decision records; returns (P, CRLB, LL, trace)
        with trace of shape (N, trace_max, 32)."""
        import torch
        n, s = rois.shape[0], rois.shape[-1]
        tm = int(iterations) + 1 if trace_max is None else int(trace_max)
        P = torch.empty((self.nv + 1, n), device=rois.device)
        C = torch.empty((self.nv, n), device=rois.device)
        L = torch.empty((n,), device=rois.device)
        T = torch.zeros((n, tm, 32), device=rois.device)
        st = torch.cuda.current_stream(rois.device)
        check(_native.lib().bsfit_trace_device(self._h, rois.data_ptr(), s, n, int(iterations),
                                               int(flags), P.data_ptr(), C.data_ptr(), L.data_ptr(),
                                               T.data_ptr(), tm, st.cuda_stream), "bsfit_trace_device")
        return P, C, L, T

    def eval_torch(self, rois, theta, fisher=False, stream=None, precision="f32"):
        """One evaluation per ROI at theta (tensor (NV, N)); returns (N, 1+NV+NH),
        float32, or float64 from the double-float evaluation (precision="parity")."""
        import torch
        n, s = rois.shape[0], rois.shape[-1]
        nh = self.nv * (self.nv + 1) // 2
        dt = torch.float64 if precision == "parity" else torch.float32
        out = torch.empty((n, 1 + self.nv + nh), device=rois.device, dtype=dt)
        theta = theta.contiguous()
        st = stream if stream is not None else torch.cuda.current_stream(rois.device)
        name = "bsfit_eval_parity_device" if precision == "parity" else "bsfit_eval_device"
        check(getattr(_native.lib(), name)(self._h, rois.data_ptr(), s, n, theta.data_ptr(),
                                           int(bool(fisher)), out.data_ptr(), st.cuda_stream),
              name)
        return out

    def close(self):
        if getattr(self, "_h", None):
            _native.lib().bsfit_model_release(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def GPUmleFit_LM_4Pi_bspline(imstack, shared, iterations, coeff, dT, initZ, initPhi,
                             phase_shift, silent=1):
    """Drop-in for the reference's 4Pi mex (demo_4pi/bspline_based_4piloc_v4.m:196).

    imstack: (4, N, s, s) float32 (the C-order view of MATLAB [s, s, N, 4]);
    shared: 6 flags (all 1); coeff: (W, Z, X, Y) 4D coefficients; dT: (N, 4, 6)
    (MATLAB [6, 4, N]); initZ, initPhi: (N,); phase_shift: (4,). Returns P
    (N, 7), CRLB (N, 6), LL (N,)."""
    lib = _native.lib()
    im = _f32(imstack)
    if im.ndim == 3:
        im = im[:, None]
    if im.ndim != 4:
        raise ValueError("imstack must be (4, N, s, s)")
    ch, n, s2, s1 = im.shape
    sh = np.ascontiguousarray(np.atleast_1d(shared), dtype=np.uint32)
    c = _f32(coeff)
    dt = _f32(dT)
    z0 = _f32(np.atleast_1d(initZ))
    w0 = _f32(np.atleast_1d(initPhi))
    ps = _f32(np.atleast_1d(phase_shift))
    P = np.empty((7, n), np.float32)
    C = np.empty((6, n), np.float32)
    L = np.empty(n, np.float32)
    ptr = lambda a: a.ctypes.data_as(_fp)  # noqa: E731
    st = lib.bsfit_GPUmleFit_LM_4Pi_bspline(
        ptr(im), s1, s2, n, ch, sh.ctypes.data_as(np.ctypeslib.ctypes.POINTER(
            np.ctypeslib.ctypes.c_uint32)), sh.size, int(iterations), ptr(c), c.ndim, _dims(c),
        ptr(dt), dt.size, ptr(z0), z0.size, ptr(w0), w0.size, ptr(ps), ps.size, int(silent),
        ptr(P), ptr(C), ptr(L))
    check(st, "GPUmleFit_LM_4Pi_bspline")
    return P.T, C.T, L


class Model4Pi:
    """A 4Pi model (4D phase-resolved coefficients and the four channels'
    phase shifts in knot units) resident on the device."""

    nv = 6
    channels = 4

    def __init__(self, coeff, phase_shift):
        lib = _native.lib()
        c = _f32(coeff)
        ps = _f32(np.atleast_1d(phase_shift))
        if ps.size != self.channels:
            raise ValueError("phase_shift must hold 4 values")
        h = np.ctypeslib.ctypes.c_void_p()
        check(lib.bsfit_model_create_4pi(c.ctypes.data_as(_fp), c.ndim, _dims(c),
                                         ps.ctypes.data_as(_fp), ps.size,
                                         np.ctypeslib.ctypes.byref(h)), "bsfit_model_create_4pi")
        self._h = h

    def fit_torch(self, rois, iterations, initZ, initPhi, dT=None, stream=None):
        """rois: CUDA float32 (4, N, s, s); initZ, initPhi: (N,); dT: (N, 4, 6)
        or None. Returns (P (7, N), CRLB (6, N), LL (N,)) device tensors."""
        import torch
        assert rois.is_cuda and rois.dtype == torch.float32 and rois.is_contiguous()
        n, s = rois.shape[1], rois.shape[-1]
        z0 = initZ.contiguous()
        w0 = initPhi.contiguous()
        dt = dT.contiguous() if dT is not None else None
        P = torch.empty((7, n), device=rois.device, dtype=torch.float32)
        C = torch.empty((6, n), device=rois.device, dtype=torch.float32)
        L = torch.empty((n,), device=rois.device, dtype=torch.float32)
        st = stream if stream is not None else torch.cuda.current_stream(rois.device)
        check(_native.lib().bsfit_fit4pi_device(
            self._h, rois.data_ptr(), s, n, int(iterations),
            dt.data_ptr() if dt is not None else None, z0.data_ptr(), w0.data_ptr(),
            P.data_ptr(), C.data_ptr(), L.data_ptr(), st.cuda_stream), "bsfit_fit4pi_device")
        return P, C, L

    def fit_f64_torch(self, rois, iterations, initZ, initPhi, dT, stream=None):
        """The 4Pi fit in double (bsfit_fit4pi_f64_device): arguments as
        fit_torch (dT required); float64 (P (7, N), CRLB (6, N), LL (N,))."""
        import torch
        assert rois.is_cuda and rois.dtype == torch.float32 and rois.is_contiguous()
        n, s = rois.shape[1], rois.shape[-1]
        z0, w0, dt = initZ.contiguous(), initPhi.contiguous(), dT.contiguous()
        P = torch.empty((7, n), device=rois.device, dtype=torch.float64)
        C = torch.empty((6, n), device=rois.device, dtype=torch.float64)
        L = torch.empty((n,), device=rois.device, dtype=torch.float64)
        st = stream if stream is not None else torch.cuda.current_stream(rois.device)
        check(_native.lib().bsfit_fit4pi_f64_device(
            self._h, rois.data_ptr(), s, n, int(iterations), dt.data_ptr(), z0.data_ptr(),
            w0.data_ptr(), P.data_ptr(), C.data_ptr(), L.data_ptr(), st.cuda_stream),
            "bsfit_fit4pi_f64_device")
        return P, C, L

    def fit_multistart_torch(self, rois, iterations, initZ, initPhi, dT=None, strict=False,
                             stream=None):
        """Fused multi-start 4Pi fit: initZ, initPhi of shape (starts, N); the
        best log-likelihood over the starts is kept per ROI (the demo's rule)."""
        import torch
        n, s = rois.shape[1], rois.shape[-1]
        z0 = initZ.contiguous()
        w0 = initPhi.contiguous()
        k = z0.shape[0] if z0.dim() == 2 else 1
        dt = dT.contiguous() if dT is not None else None
        P = torch.empty((7, n), device=rois.device, dtype=torch.float32)
        C = torch.empty((6, n), device=rois.device, dtype=torch.float32)
        L = torch.empty((n,), device=rois.device, dtype=torch.float32)
        cs = stream if stream is not None else torch.cuda.current_stream(rois.device)
        check(_native.lib().bsfit_fit4pi_multistart_device(
            self._h, rois.data_ptr(), s, n, int(iterations),
            dt.data_ptr() if dt is not None else None, z0.data_ptr(), w0.data_ptr(), k,
            int(bool(strict)), P.data_ptr(), C.data_ptr(), L.data_ptr(), cs.cuda_stream),
            "bsfit_fit4pi_multistart_device")
        return P, C, L

    def eval_torch(self, rois, theta, dT=None, fisher=False, stream=None):
        """One 4Pi evaluation per ROI at theta (6, N); returns (N, 1 + 6 + 21)."""
        import torch
        n, s = rois.shape[1], rois.shape[-1]
        out = torch.empty((n, 28), device=rois.device, dtype=torch.float32)
        theta = theta.contiguous()
        dt = dT.contiguous() if dT is not None else None
        st = stream if stream is not None else torch.cuda.current_stream(rois.device)
        check(_native.lib().bsfit_eval4pi_device(
            self._h, rois.data_ptr(), s, n, dt.data_ptr() if dt is not None else None,
            theta.data_ptr(), int(bool(fisher)), out.data_ptr(), st.cuda_stream),
            "bsfit_eval4pi_device")
        return out

    def close(self):
        if getattr(self, "_h", None):
            _native.lib().bsfit_model_release(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _starts_array(starts, n_entries, strict):
    """bsfit_starts per entry from sequences of initP vectors (None or an
    empty sequence: one start from the model's initP)."""
    if len(starts) != n_entries:
        raise ValueError("one starts sequence per entry")
    st = (_native.Starts * n_entries)()
    for k, sv in enumerate(starts):
        st[k].strict = int(bool(strict))
        if sv is None or len(sv) == 0:
            st[k].n_starts = 0
            continue
        a = np.atleast_2d(np.asarray(sv, np.float32))
        if not 1 <= a.shape[0] <= 8 or a.shape[1] > 4:
            raise ValueError("1 to 8 starts of at most 4 values per entry")
        st[k].n_starts = a.shape[0]
        for i in range(a.shape[0]):
            for j in range(a.shape[1]):
                st[k].initp[i][j] = float(a[i, j])
    return st


class Batch:
    """Batched fit of ROI segments (mixed ROI sizes and models) with one
    persistent launch per fit type. Each entry: (model, rois_cuda_tensor,
    iterations). Outputs are allocated once and reused across calls; the work
    queue lives in a small device scratch buffer owned by the batch.
    starts (fit types 7, 8): one sequence of initP vectors per entry, fitted
    from each inside the launch with the best log-likelihood kept (strict: the
    4D GUI's "> 1e-4" rule instead of ">= 1e-4")."""

    def __init__(self, entries, device=None, starts=None, strict=False):
        import torch
        if not 0 < len(entries) <= 48:
            raise ValueError("a batch holds 1 to 48 segments")
        self.entries = list(entries)
        dev = device or self.entries[0][1].device
        self.outputs = []
        segs = (_native.Segment * len(self.entries))()
        for k, (m, r, it) in enumerate(self.entries):
            n, s = r.shape[0], r.shape[-1]
            P = torch.empty((m.nv + 1, n), device=dev)
            C = torch.empty((m.nv, n), device=dev)
            L = torch.empty((n,), device=dev)
            self.outputs.append((P, C, L))
            segs[k].model = m._h.value
            segs[k].d_rois = r.data_ptr()
            segs[k].roi_size = s
            segs[k].nfits = n
            segs[k].iterations = int(it)
            segs[k].d_P, segs[k].d_CRLB, segs[k].d_LL = P.data_ptr(), C.data_ptr(), L.data_ptr()
        self._segs = segs
        self._starts = None
        if starts is not None:
            self._starts = _starts_array(starts, len(self.entries), strict)
        nb = _native.lib().bsfit_batch_scratch_bytes(len(self.entries))
        self.scratch = torch.zeros((max(nb, 256) // 8,), dtype=torch.int64, device=dev)

    def run(self, stream=None):
        import torch
        st = stream if stream is not None else torch.cuda.current_stream(self.scratch.device)
        ct = np.ctypeslib.ctypes
        if self._starts is None:
            check(_native.lib().bsfit_batch_fit_device(
                ct.cast(self._segs, ct.c_void_p), len(self.entries), self.scratch.data_ptr(),
                self.scratch.numel() * 8, st.cuda_stream), "bsfit_batch_fit_device")
        else:
            check(_native.lib().bsfit_batch_fit_multistart_device(
                ct.cast(self._segs, ct.c_void_p), ct.cast(self._starts, ct.c_void_p),
                len(self.entries), self.scratch.data_ptr(), self.scratch.numel() * 8,
                st.cuda_stream), "bsfit_batch_fit_multistart_device")
        return self.outputs

    def counters(self):
        """(claimed, finished) ROI counts per segment after completion."""
        c = self.scratch.cpu().numpy()
        k = len(self.entries)
        return c[:k].copy(), c[k:2 * k].copy()


class Server:
    """Continuous-batching request loop (bsfit_server_*).

    submit([(model, rois, iterations), ...]) stages the ROIs in page-locked
    host memory, returns a request id and queues or starts the request;
    poll() returns {id: [(P, CRLB, LL), ...]} for every request finished since
    the last call (P (N, NV+1), CRLB (N, NV), LL (N,) per segment, as
    GPUmleFit_LM_multiD); wait(id) blocks until one request is done."""

    def __init__(self, max_inflight=4, arena_bytes=2 << 30, merge=1, priority=False):
        """merge: most queued requests fitted by one launch (bsfit_server_set_merge);
        priority: launches on streams of three priorities by their estimated
        device time, with blocks that retire while they run
        (bsfit_server_set_priority)."""
        h = np.ctypeslib.ctypes.c_void_p()
        check(_native.lib().bsfit_server_create(int(max_inflight), int(arena_bytes),
                                                np.ctypeslib.ctypes.byref(h)), "bsfit_server_create")
        self._h = h
        for on, fn, arg in ((merge != 1, "bsfit_server_set_merge", int(merge)),
                            (bool(priority), "bsfit_server_set_priority", 1)):
            if on:
                st = getattr(_native.lib(), fn)(h, arg)
                if st != 0:
                    self.close()
                    check(st, fn)
        self._live = {}
        self._done = {}  # results collected by poll() and not yet taken by wait()

    def submit(self, entries, starts=None, strict=False):
        """Submit one request: entries (model, host ROIs, iterations); starts:
        optional per-entry initP sequences (None or [] for one start), fitted
        with the multi-start rule inside the batched launch."""
        import torch
        segs = (_native.HostSegment * len(entries))()
        keep = []
        for k, (m, rois, it) in enumerate(entries):
            r = torch.as_tensor(np.ascontiguousarray(rois, dtype=np.float32))
            if r.ndim == 2:
                r = r[None]
            r = r.pin_memory()
            n, s = r.shape[0], r.shape[-1]
            P = torch.empty((m.nv + 1, n), dtype=torch.float32).pin_memory()
            C = torch.empty((m.nv, n), dtype=torch.float32).pin_memory()
            L = torch.empty((n,), dtype=torch.float32).pin_memory()
            keep.append((m, r, P, C, L))
            segs[k].model = m._h.value
            segs[k].rois = r.data_ptr()
            segs[k].roi_size = s
            segs[k].nfits = n
            segs[k].iterations = int(it)
            segs[k].P, segs[k].CRLB, segs[k].LL = P.data_ptr(), C.data_ptr(), L.data_ptr()
        ct = np.ctypeslib.ctypes
        rid = ct.c_int64()
        if starts is None:
            check(_native.lib().bsfit_server_submit(self._h, ct.cast(segs, ct.c_void_p),
                                                    len(entries), ct.byref(rid)),
                  "bsfit_server_submit")
        else:
            st = _starts_array(starts, len(entries), strict)
            keep.append(st)
            check(_native.lib().bsfit_server_submit_multistart(
                self._h, ct.cast(segs, ct.c_void_p), ct.cast(st, ct.c_void_p), len(entries),
                ct.byref(rid)), "bsfit_server_submit_multistart")
        self._live[rid.value] = (segs, keep)
        return rid.value

    def _results(self, rid):
        segs, keep = self._live.pop(rid)
        return [(P.numpy().T.copy(), C.numpy().T.copy(), L.numpy().copy())
                for m, r, P, C, L in (k for k in keep if isinstance(k, tuple))]

    def poll(self):
        ct = np.ctypeslib.ctypes
        ids = (ct.c_int64 * 256)()
        n = ct.c_int32()
        out = {}
        while True:
            check(_native.lib().bsfit_server_poll(self._h, ids, 256, ct.byref(n)), "bsfit_server_poll")
            for i in range(n.value):
                out[ids[i]] = self._results(ids[i])
                self._done[ids[i]] = out[ids[i]]
            if n.value < 256:
                return out

    def wait(self, rid, timeout=60.0):
        if rid in self._done:
            return self._done.pop(rid)
        check(_native.lib().bsfit_server_wait(self._h, int(rid), float(timeout)), "bsfit_server_wait")
        return self._results(rid)

    def stats(self):
        ct = np.ctypeslib.ctypes
        d = [ct.c_double() for _ in range(3)]
        i = [ct.c_int64() for _ in range(3)]
        check(_native.lib().bsfit_server_stats(self._h, *[ct.byref(x) for x in d],
                                               *[ct.byref(x) for x in i]), "bsfit_server_stats")
        return {"p50_ms": d[0].value, "p99_ms": d[1].value, "fits_per_s": d[2].value,
                "completed": i[0].value, "in_flight": i[1].value, "queued": i[2].value}

    def latencies(self, max_n=100000):
        """{request id: latency ms} of the requests completed since the last
        reset_stats."""
        ct = np.ctypeslib.ctypes
        ids = (ct.c_int64 * max_n)()
        ms = (ct.c_double * max_n)()
        n = ct.c_int32()
        check(_native.lib().bsfit_server_latencies(self._h, ids, ms, max_n, ct.byref(n)),
              "bsfit_server_latencies")
        return {ids[i]: ms[i] for i in range(n.value)}

    def reset_stats(self):
        check(_native.lib().bsfit_server_reset_stats(self._h), "bsfit_server_reset_stats")

    def close(self):
        if getattr(self, "_h", None):
            _native.lib().bsfit_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def bsarray_coeffs(samples):
    """Cubic B-spline coefficients of a sampled stack on the GPU (the
    reference's bsarray, degree 3): samples in C order with the reference's
    fastest axis last, shape (..., Z, X, Y); returns float32 coefficients two
    larger along every axis, the fitter's coefficient input."""
    x = np.ascontiguousarray(samples, dtype=np.float64)
    out = np.empty(tuple(d + 2 for d in x.shape), np.float32)
    check(_native.lib().bsfit_bsarray_coeffs(
        x.ctypes.data_as(np.ctypeslib.ctypes.POINTER(np.ctypeslib.ctypes.c_double)), x.ndim,
        _dims(x), out.ctypes.data_as(_fp)), "bsfit_bsarray_coeffs")
    return out


def bsarray_coeffs_torch(samples, out64=False, stream=None):
    """Device form: samples a CUDA float64 tensor (C order, reference's fastest
    axis last); returns the float32 coefficients (and the float64 ones with
    out64) as CUDA tensors."""
    import torch
    x = samples.contiguous()
    assert x.is_cuda and x.dtype == torch.float64
    shape = tuple(d + 2 for d in x.shape)
    work = torch.empty_like(x)
    c32 = torch.empty(shape, device=x.device, dtype=torch.float32)
    c64 = torch.empty(shape, device=x.device, dtype=torch.float64) if out64 else None
    dims = (np.ctypeslib.ctypes.c_int64 * x.dim())(*reversed(x.shape))
    cs = stream if stream is not None else torch.cuda.current_stream(x.device)
    check(_native.lib().bsfit_bsarray_coeffs_device(
        x.data_ptr(), x.dim(), dims, work.data_ptr(), c32.data_ptr(),
        c64.data_ptr() if c64 is not None else None, cs.cuda_stream), "bsfit_bsarray_coeffs_device")
    return (c32, c64) if out64 else c32


def peak_kernel(mode, sigma):
    """The reference's peak-finding filter kernel (0: Gaussian, 1: difference of
    Gaussians) as a (k, k) float32 array h[u, v] (u the row offset)."""
    buf = np.zeros(31 * 31, np.float32)
    k = np.ctypeslib.ctypes.c_int32()
    check(_native.lib().bsfit_peak_kernel(int(mode), float(sigma), buf.ctypes.data_as(_fp),
                                          np.ctypeslib.ctypes.byref(k)), "bsfit_peak_kernel")
    return buf[:k.value * k.value].reshape(k.value, k.value).T.copy()


def find_rois_torch(frames, offset, conversion, kernel, dog, cutoff, roi_size, mirror=False,
                    capacity=None, filtered=False, stream=None):
    """Frame -> ROI front end on the GPU. frames: CUDA float32 (F, W, H) (the
    C-order view of MATLAB [H, W, F]); kernel: (k, k) float array h[u, v];
    dog: subtract the first column's minimum before filtering. Returns
    (rois (N, s, s), coords (N, 3) = x, y, frame 1-based[, filtered (F, W, H)])
    as CUDA tensors, N the number found (all of them)."""
    import torch
    assert frames.is_cuda and frames.dtype == torch.float32
    fr = frames.contiguous()
    F, W, H = fr.shape
    h = np.ascontiguousarray(np.asarray(kernel, np.float32).T)  # [u + k v]
    fe = _native.Frontend(float(offset), float(conversion), h.ctypes.data_as(_fp), h.shape[0],
                          int(bool(dog)), float(cutoff), int(roi_size), int(bool(mirror)))
    lib = _native.lib()
    nb = lib.bsfit_find_rois_scratch_bytes(F, H, W)
    scratch = torch.empty((max(nb, 256),), dtype=torch.uint8, device=fr.device)
    filt = torch.empty_like(fr) if filtered else None
    cs = stream if stream is not None else torch.cuda.current_stream(fr.device)
    s = int(roi_size)
    cap = int(capacity) if capacity is not None else max(1, F * W * H // 100)
    for _ in range(2):
        rois = torch.empty((cap, s, s), dtype=torch.float32, device=fr.device)
        coords = torch.empty((3, cap), dtype=torch.float32, device=fr.device)
        n = np.ctypeslib.ctypes.c_int64()
        check(lib.bsfit_find_rois_device(fr.data_ptr(), F, H, W, np.ctypeslib.ctypes.byref(fe),
                                         rois.data_ptr(), coords.data_ptr(), cap,
                                         np.ctypeslib.ctypes.byref(n),
                                         filt.data_ptr() if filt is not None else None,
                                         scratch.data_ptr(), nb, cs.cuda_stream), "bsfit_find_rois_device")
        if n.value <= cap or capacity is not None:
            break
        cap = n.value
    k = min(n.value, cap)
    out = (rois[:k], coords[:, :k].T.contiguous())
    return out + (filt,) if filtered else out


def measure_fp32_peak():
    """Measured FP32 FMA throughput of the current device, TFLOP/s."""
    v = np.ctypeslib.ctypes.c_double()
    check(_native.lib().bsfit_measure_fp32_peak(np.ctypeslib.ctypes.byref(v)), "fp32 peak")
    return v.value


def measure_fp32_peaks():
    """(scalar, paired) measured FP32 FMA throughput of the current device,
    TFLOP/s: scalar FFMA chains and paired FFMA2 chains."""
    a, b = np.ctypeslib.ctypes.c_double(), np.ctypeslib.ctypes.c_double()
    check(_native.lib().bsfit_measure_fp32_peaks(np.ctypeslib.ctypes.byref(a),
                                                 np.ctypeslib.ctypes.byref(b)), "fp32 peaks")
    return a.value, b.value


def eval_flops(fittype, s, channels=1):
    """Algorithmic FLOPs of one ROI evaluation (separable minimum): contract the
    non-lateral axes over the (s+4)^2 knot window, one 4-tap pass per lateral
    axis and output map, then the Jacobian, Hessian and deviance per pixel.
    K = 4^(D-2) coefficients per lateral node. The 4Pi fit (FIT_4PI) is the
    4D evaluation once per channel."""
    if fittype == FIT_4PI:
        return 4 * eval_flops(7, s, channels)
    d = {6: 3, 7: 4, 8: 5}[fittype]
    nv = NUM_PARAMS[fittype]
    k = 4 ** (d - 2)
    f = 2 * (d - 1) * k * (s + 4) ** 2 + (d + 1) * 8 * s * (2 * s + 4) + s * s * (2 * nv + nv * (nv + 1) + 6)
    if fittype == 8:
        # the 3D part of the mixture and the per-pixel mixing of model and dudt
        f += 2 * 2 * 4 * (s + 4) ** 2 + 4 * 8 * s * (2 * s + 4) + 12 * s * s
    return channels * f


def version():
    return _native.lib().bsfit_version().decode()
