"""Autotuner on the GPU: every launch configuration (kernel variant x warps
per block) of the FP32 fit kernels gives results bit-identical to the default,
plain and batched; the tuner's choice is put in force, recorded in the cache
and restored from it."""
import numpy as np
import pytest

from test_fit_gpu import bsfit_mod  # noqa: F401

pytestmark = pytest.mark.gpu


def _wl(fittype, n, stream):
    from bsfit import workloads as W
    if fittype == 6:
        return W.workload_3d(n, s=13, stream=stream)
    if fittype == 7:
        return W.workload_4d(n, sizes=(13,), stream=stream)[0]
    return W.workload_5d(n, stream=stream)


@pytest.mark.parametrize("fittype,n", [(6, 3000), (7, 800), (8, 160)])
def test_every_configuration_is_bit_identical(bsfit_mod, fittype, n):
    import torch
    from bsfit import tuning as T
    wl = _wl(fittype, n, 901 + fittype)
    m = bsfit_mod.Model(fittype, wl.coeff, coeff3=wl.coeff3, init_p=wl.init_p)
    r = torch.from_numpy(wl.rois).cuda()
    s = wl.roi_size
    T._set(fittype, s, -1, 0)
    ref = [x.cpu().numpy() for x in m.fit_torch(r, wl.iterations)]
    bref = bsfit_mod.Batch([(m, r, wl.iterations)])
    bref.run()
    bref = [x.cpu().numpy() for x in bref.outputs[0]]
    assert all(np.array_equal(a, b, equal_nan=True) for a, b in zip(ref, bref))
    tried = 0
    try:
        for v in range(T.num_variants(fittype)):
            for w in (4, 2, 1):
                T._set(fittype, s, v, w)
                assert T.current(fittype, s) == (v, w)
                try:
                    out = [x.cpu().numpy() for x in m.fit_torch(r, wl.iterations)]
                except bsfit_mod.BsfitError:
                    continue  # this configuration cannot launch (shared memory)
                tried += 1
                for a, b in zip(out, ref):
                    assert np.array_equal(a, b, equal_nan=True), (v, w)
                b = bsfit_mod.Batch([(m, r, wl.iterations)])
                b.run()
                for a, b_ in zip([x.cpu().numpy() for x in b.outputs[0]], ref):
                    assert np.array_equal(a, b_, equal_nan=True), ("batched", v, w)
    finally:
        T._set(fittype, s, -1, 0)
    assert tried >= T.num_variants(fittype)
    assert T.current(fittype, s) == (-1, 0)
    m.close()


def test_autotune_chooses_and_caches(bsfit_mod, tmp_path):
    import torch
    from bsfit import tuning as T
    wl = _wl(6, 20000, 911)
    m = bsfit_mod.Model(6, wl.coeff)
    r = torch.from_numpy(wl.rois).cuda()
    cache = tmp_path / "tune.json"
    try:
        ch = T.autotune(m, r, wl.iterations, reps=2, cache=str(cache))
        assert 0 <= ch["variant"] < T.num_variants(6) and ch["warps_per_block"] in (1, 2, 4)
        assert ch["min_blocks"] == T.min_blocks(6, ch["variant"])
        timed = [t for t in ch["candidates"].values() if t is not None]
        assert len(timed) >= 3 and abs(ch["ms"] - min(timed)) < 1e-9
        assert T.current(6, 13) == (ch["variant"], ch["warps_per_block"])
        # recorded under this device's name, and put back in force from the file
        assert T.lookup(T.load_cache(cache), T.device_name(), 6, 13)["variant"] == ch["variant"]
        T._set(6, 13, -1, 0)
        m2 = bsfit_mod.Model(6, wl.coeff, tune_cache=str(cache))
        assert T.current(6, 13) == (ch["variant"], ch["warps_per_block"])
        m2.close()
    finally:
        T._set(6, 13, -1, 0)
    m.close()
