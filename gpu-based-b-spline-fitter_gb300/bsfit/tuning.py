"""Autotuner of the FP32 fit kernels' launch configuration.

The reference launches every fit with one fixed shape (64-thread blocks, one
thread per ROI: VC/GPUmleFit_LM/mexFunction.cpp:407). Here a fit launch has two
free parameters per fit type, ROI size and device: the kernel variant (the
minimum resident 4-warp blocks per SM it is compiled for, which sets its
register budget) and the warps per block (4, 2 or 1). ``autotune`` times every
configuration on a sample of the caller's ROIs through the library
(``bsfit_autotune_device``), keeps the fastest in force and can record it in a
JSON cache file; ``apply_cache`` (or ``Model(..., tune_cache=path)``) puts the
cached choices of this device back in force in a later process. Every
configuration gives bit-identical results.

Cache file format (one file may hold several devices):

    {"format": "bsfit-tune-1",
     "devices": {"<device name>": {"<fit type>:<ROI size>":
                  {"variant": v, "warps_per_block": w, "min_blocks": b, "ms": t}}}}
"""
import ctypes
import json
import os

from . import _native
from ._native import check

FORMAT = "bsfit-tune-1"
WARPS_PER_BLOCK = (4, 2, 1)  # the order of bsfit_autotune_device's all_ms columns


def cache_key(fittype, roi_size):
    return f"{int(fittype)}:{int(roi_size)}"


def empty_cache():
    return {"format": FORMAT, "devices": {}}


def load_cache(path):
    """The cache at ``path``; an empty one when the file is missing, unreadable
    or of another format."""
    try:
        with open(path) as f:
            c = json.load(f)
    except (OSError, ValueError):
        return empty_cache()
    if not isinstance(c, dict) or c.get("format") != FORMAT or not isinstance(c.get("devices"), dict):
        return empty_cache()
    return c


def save_cache(path, cache):
    tmp = f"{path}.tmp{os.getpid()}"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def record(cache, device, fittype, roi_size, choice):
    cache.setdefault("devices", {}).setdefault(device, {})[cache_key(fittype, roi_size)] = {
        k: choice[k] for k in ("variant", "warps_per_block", "min_blocks", "ms")}
    return cache


def lookup(cache, device, fittype, roi_size):
    return cache.get("devices", {}).get(device, {}).get(cache_key(fittype, roi_size))


def _set(fittype, roi_size, variant, wpb):
    check(_native.lib().bsfit_tune_set(int(fittype), int(roi_size), int(variant), int(wpb)),
          "bsfit_tune_set")


def apply_cache(cache, device, setter=_set):
    """Puts the cached choices for ``device`` in force (``setter(fittype,
    roi_size, variant, warps_per_block)``, by default the library's
    bsfit_tune_set on the current device); other devices' entries are ignored.
    ``cache`` is a path or a loaded cache. Returns the number applied."""
    if isinstance(cache, (str, os.PathLike)):
        cache = load_cache(cache)
    n = 0
    for key, ch in cache.get("devices", {}).get(device, {}).items():
        try:
            ft, s = (int(x) for x in key.split(":"))
            setter(ft, s, int(ch["variant"]), int(ch["warps_per_block"]))
        except (ValueError, KeyError, TypeError):
            continue
        n += 1
    return n


def num_variants(fittype):
    return _native.lib().bsfit_tune_num_variants(int(fittype))


def min_blocks(fittype, variant):
    return _native.lib().bsfit_tune_min_blocks(int(fittype), int(variant))


def rois_per_warp(fittype, variant):
    """ROIs a warp fits at once in a variant (2: fit type 6's pair form), 0 if
    the variant does not exist."""
    return _native.lib().bsfit_tune_rois_per_warp(int(fittype), int(variant))


def current(fittype, roi_size):
    """(variant, warps_per_block) in force on the current device; variant -1
    when the default applies."""
    v, w = ctypes.c_int32(), ctypes.c_int32()
    check(_native.lib().bsfit_tune_get(int(fittype), int(roi_size), ctypes.byref(v),
                                       ctypes.byref(w)), "bsfit_tune_get")
    return v.value, w.value


def device_name():
    import torch
    return torch.cuda.get_device_name()


def autotune(model, rois, iterations, reps=3, cache=None, stream=None):
    """Times every configuration of ``model``'s fit type at the ROI size of
    ``rois`` (a CUDA float32 tensor (N, s, s), a sample of the workload), puts
    the fastest in force and returns it:
    {"variant", "warps_per_block", "min_blocks", "ms", "candidates"} with
    candidates["v<variant>w<warps>"] the mean ms per call (None where the
    configuration cannot launch). With ``cache`` (a path) the choice is recorded
    there under this device's name."""
    import torch
    n, s = rois.shape[0], rois.shape[-1]
    nv = num_variants(model.fittype)
    P = torch.empty((model.nv + 1, n), device=rois.device)
    C = torch.empty((model.nv, n), device=rois.device)
    L = torch.empty((n,), device=rois.device)
    st = stream if stream is not None else torch.cuda.current_stream(rois.device)
    bv, bw, bms = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_double()
    all_ms = (ctypes.c_double * (3 * nv))()
    check(_native.lib().bsfit_autotune_device(
        model._h, rois.data_ptr(), s, n, int(iterations), P.data_ptr(), C.data_ptr(),
        L.data_ptr(), int(reps), ctypes.byref(bv), ctypes.byref(bw), ctypes.byref(bms), all_ms,
        st.cuda_stream), "bsfit_autotune_device")
    cand = {f"v{v}w{w}": (all_ms[v * 3 + i] if all_ms[v * 3 + i] > 0 else None)
            for v in range(nv) for i, w in enumerate(WARPS_PER_BLOCK)}
    choice = {"variant": bv.value, "warps_per_block": bw.value,
              "min_blocks": min_blocks(model.fittype, bv.value),
              "rois_per_warp": rois_per_warp(model.fittype, bv.value), "ms": bms.value,
              "candidates": cand}
    if cache is not None:
        c = load_cache(cache)
        record(c, device_name(), model.fittype, s, choice)
        save_cache(cache, c)
    return choice
