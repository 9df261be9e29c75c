"""ctypes binding of libbsfit.so (the C ABI in include/bsfit.h).

The library is required: importing this module on a machine where it has not
been built raises, so there is no silent CPU fallback anywhere."""
import ctypes
import os

from .build import LIB

_lib = None

_fp = ctypes.POINTER(ctypes.c_float)
_i64p = ctypes.POINTER(ctypes.c_int64)

# name -> (restype, argtypes); mirrors include/bsfit.h
SIGNATURES = {
    "bsfit_status_str": (ctypes.c_char_p, [ctypes.c_int]),
    "bsfit_version": (ctypes.c_char_p, []),
    "bsfit_num_params": (ctypes.c_int, [ctypes.c_int32]),
    "bsfit_measure_fp32_peak": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double)]),
    "bsfit_measure_fp32_peaks": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double),
                                                ctypes.POINTER(ctypes.c_double)]),
    "bsfit_GPUmleFit_LM_multiD": (ctypes.c_int, [
        _fp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
        _fp, ctypes.c_int32, _i64p, _fp, ctypes.c_int64, ctypes.c_int32, _fp, ctypes.c_int64,
        _fp, ctypes.c_int32, _i64p, _fp, _fp, _fp]),
    "bsfit_GPUmleFit_LM_multiD_parity": (ctypes.c_int, [
        _fp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
        _fp, ctypes.c_int32, _i64p, _fp, ctypes.c_int64, ctypes.c_int32, _fp, ctypes.c_int64,
        _fp, ctypes.c_int32, _i64p, _fp, _fp, _fp]),
    "bsfit_eval_parity_device": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
        ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]),
    "bsfit_tune_num_variants": (ctypes.c_int, [ctypes.c_int32]),
    "bsfit_tune_min_blocks": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32]),
    "bsfit_tune_rois_per_warp": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32]),
    "bsfit_tune_set": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int64, ctypes.c_int32,
                                      ctypes.c_int32]),
    "bsfit_tune_get": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int64,
                                      ctypes.POINTER(ctypes.c_int32),
                                      ctypes.POINTER(ctypes.c_int32)]),
    "bsfit_autotune_device": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
        ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
        ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]),
    "bsfit_fit_parity_steps_device": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
        ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "bsfit_fit_parity_device": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "bsfit_GPUmleFit_LM_multiD_f64": (ctypes.c_int, [
        _fp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
        _fp, ctypes.c_int32, _i64p, _fp, ctypes.c_int64, ctypes.c_int32, _fp, ctypes.c_int64,
        _fp, ctypes.c_int32, _i64p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "bsfit_model_create": (ctypes.c_int, [
        ctypes.c_int32, _fp, ctypes.c_int32, _i64p, _fp, ctypes.c_int32, _i64p, _fp,
        ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p)]),
    "bsfit_model_release": (ctypes.c_int, [ctypes.c_void_p]),
    "bsfit_eval_device": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
        ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]),
    "bsfit_trace_device": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
        ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_int32, ctypes.c_void_p]),
    "bsfit_batch_scratch_bytes": (ctypes.c_int64, [ctypes.c_int32]),
    "bsfit_batch_fit_device": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]),
    "bsfit_batch_fit_device_static": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]),
    "bsfit_batch_fit_multistart_device": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64,
        ctypes.c_void_p]),
    "bsfit_model_fittype": (ctypes.c_int32, [ctypes.c_void_p]),
    "bsfit_server_create": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int64,
                                           ctypes.POINTER(ctypes.c_void_p)]),
    "bsfit_server_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "bsfit_server_set_merge": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "bsfit_server_set_priority": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "bsfit_server_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                           ctypes.POINTER(ctypes.c_int64)]),
    "bsfit_server_submit_multistart": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
        ctypes.POINTER(ctypes.c_int64)]),
    "bsfit_server_poll": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64),
                                         ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]),
    "bsfit_server_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_double]),
    "bsfit_server_latencies": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64),
                                              ctypes.POINTER(ctypes.c_double), ctypes.c_int32,
                                              ctypes.POINTER(ctypes.c_int32)]),
    "bsfit_server_stats": (ctypes.c_int, [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_double)] * 3 +
                           [ctypes.POINTER(ctypes.c_int64)] * 3),
    "bsfit_server_reset_stats": (ctypes.c_int, [ctypes.c_void_p]),
    "bsfit_fit_device": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "bsfit_GPUmleFit_LM_4Pi_bspline": (ctypes.c_int, [
        _fp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
        ctypes.POINTER(ctypes.c_uint32), ctypes.c_int64, ctypes.c_int32, _fp, ctypes.c_int32,
        _i64p, _fp, ctypes.c_int64, _fp, ctypes.c_int64, _fp, ctypes.c_int64, _fp,
        ctypes.c_int64, ctypes.c_int32, _fp, _fp, _fp]),
    "bsfit_model_create_4pi": (ctypes.c_int, [
        _fp, ctypes.c_int32, _i64p, _fp, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]),
    "bsfit_fit4pi_device": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_void_p, ctypes.c_void_p]),
    "bsfit_fit_multistart_device": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, _fp,
        ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_void_p, ctypes.c_void_p]),
    "bsfit_fit4pi_multistart_device": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "bsfit_bsarray_coeffs_device": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int32, _i64p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_void_p]),
    "bsfit_bsarray_coeffs": (ctypes.c_int, [
        ctypes.POINTER(ctypes.c_double), ctypes.c_int32, _i64p, _fp]),
    "bsfit_peak_kernel": (ctypes.c_int, [ctypes.c_int32, ctypes.c_double, _fp,
                                         ctypes.POINTER(ctypes.c_int32)]),
    "bsfit_find_rois_scratch_bytes": (ctypes.c_int64, [ctypes.c_int64] * 3),
    "bsfit_find_rois_device": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64),
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]),
    "bsfit_fit_scmos_device": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
        ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "bsfit_eval4pi_device": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
        ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]),
    "bsfit_fit4pi_f64_device": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32,
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_void_p, ctypes.c_void_p]),
    "bsfit_fit_f64_device": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
        ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
}


def lib():
    global _lib
    if _lib is None:
        path = os.environ.get("BSFIT_LIB", LIB)  # an alternative build of the same library
        if not os.path.exists(path):
            raise ImportError(f"{path} is not built: run __graft_entry__.build() first")
        handle = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


class BsfitError(RuntimeError):
    def __init__(self, status, where=""):
        self.status = status
        msg = lib().bsfit_status_str(status).decode()
        super().__init__(f"{where}: bsfit status {status}: {msg}" if where else msg)


def check(status, where=""):
    if status != 0:
        raise BsfitError(status, where)


class Segment(ctypes.Structure):
    """bsfit_segment (include/bsfit.h)."""
    _fields_ = [("model", ctypes.c_void_p), ("d_rois", ctypes.c_void_p),
                ("roi_size", ctypes.c_int64), ("nfits", ctypes.c_int64),
                ("iterations", ctypes.c_int32), ("d_P", ctypes.c_void_p),
                ("d_CRLB", ctypes.c_void_p), ("d_LL", ctypes.c_void_p)]


class Starts(ctypes.Structure):
    """bsfit_starts (include/bsfit.h)."""
    _fields_ = [("n_starts", ctypes.c_int32), ("strict", ctypes.c_int32),
                ("initp", (ctypes.c_float * 4) * 8)]


class Frontend(ctypes.Structure):
    """bsfit_frontend (include/bsfit.h)."""
    _fields_ = [("offset", ctypes.c_float), ("conversion", ctypes.c_float),
                ("kernel", ctypes.POINTER(ctypes.c_float)), ("ksize", ctypes.c_int32),
                ("subtract_first_column_min", ctypes.c_int32), ("cutoff", ctypes.c_double),
                ("roi_size", ctypes.c_int32), ("mirror", ctypes.c_int32)]


class HostSegment(ctypes.Structure):
    """bsfit_host_segment (include/bsfit.h)."""
    _fields_ = [("model", ctypes.c_void_p), ("rois", ctypes.c_void_p),
                ("roi_size", ctypes.c_int64), ("nfits", ctypes.c_int64),
                ("iterations", ctypes.c_int32), ("P", ctypes.c_void_p),
                ("CRLB", ctypes.c_void_p), ("LL", ctypes.c_void_p)]
