"""Serving form (bsfit_server_*): requests of mixed models and sizes submitted
while others run give the same results as each request fitted alone through
the plain call; admission respects the device-memory budget; waits are
bounded."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bsfit_mod():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()
    import bsfit
    return bsfit


def _frames():
    from bsfit import workloads as W
    frames = []
    for k, (s, n) in enumerate([(13, 3000), (17, 1500), (11, 2500), (13, 800)]):
        w = W.workload_3d(n, s=s, stream=800 + k)
        frames.append(("3d", w))
    frames.append(("4d", W.workload_4d(500, sizes=(15,), stream=810)[0]))
    frames.append(("5d", W.workload_5d(60, stream=811)))
    return frames


def test_serving_matches_plain_in_the_mix(bsfit_mod):
    frames = _frames()
    models = {}
    for kind, w in frames:
        if kind not in models:
            models[kind] = bsfit_mod.Model(w.fittype, w.coeff, coeff3=w.coeff3, init_p=w.init_p)
    # Arena of 24 MB: the 5D model's frames and the large 3D frames cannot all be
    # resident at once, so later requests wait for memory and slots.
    srv = bsfit_mod.Server(max_inflight=3, arena_bytes=24 << 20)
    ids = [srv.submit([(models[kind], w.rois, w.iterations)]) for kind, w in frames]
    results = {}
    for rid in ids:
        results[rid] = srv.wait(rid, timeout=120.0)
    st = srv.stats()
    assert st["completed"] == len(frames) and st["in_flight"] == 0 and st["queued"] == 0
    assert st["p99_ms"] >= st["p50_ms"] > 0 and st["fits_per_s"] > 0
    # per-request latencies: one per request, the quantiles drawn from them
    lat = srv.latencies()
    assert sorted(lat) == sorted(ids) and all(v > 0 for v in lat.values())
    assert min(lat.values()) <= st["p50_ms"] <= st["p99_ms"] <= max(lat.values())
    for rid, (kind, w) in zip(ids, frames):
        kw = {}
        if w.init_p is not None:
            kw["initP"] = w.init_p
        if w.coeff3 is not None:
            kw["coeff3"] = w.coeff3
        P, C, L = bsfit_mod.GPUmleFit_LM_multiD(w.rois, w.fittype, w.iterations, w.coeff, **kw)
        Ps, Cs, Ls = results[rid][0]
        assert np.array_equal(Ps, P, equal_nan=True), kind
        assert np.array_equal(Cs, C, equal_nan=True), kind
        assert np.array_equal(Ls, L, equal_nan=True), kind
    srv.close()


def test_serving_poll_returns_each_request_once(bsfit_mod):
    from bsfit import workloads as W
    w = W.workload_3d(1000, s=13, stream=820)
    m = bsfit_mod.Model(6, w.coeff)
    srv = bsfit_mod.Server(max_inflight=2, arena_bytes=64 << 20)
    ids = {srv.submit([(m, w.rois[i * 100:(i + 1) * 100], 30)]) for i in range(10)}
    seen = {}
    import time
    t0 = time.time()
    while len(seen) < len(ids) and time.time() - t0 < 60:
        for rid, res in srv.poll().items():
            assert rid not in seen
            seen[rid] = res
            srv.wait(rid)  # taken from the poll()ed results
    assert set(seen) == ids
    srv.close()


def test_serving_budget_and_timeout(bsfit_mod):
    from bsfit import _native, workloads as W
    w = W.workload_3d(20000, s=17, stream=821)
    m = bsfit_mod.Model(6, w.coeff)
    srv = bsfit_mod.Server(max_inflight=1, arena_bytes=8 << 20)
    with pytest.raises(bsfit_mod.BsfitError) as e:
        srv.submit([(m, w.rois, 30)])  # 23 MB of ROIs > 8 MB budget
    assert e.value.status == 6
    srv.close()
    srv = bsfit_mod.Server(max_inflight=1, arena_bytes=64 << 20)
    rid = srv.submit([(m, w.rois, 30)])
    st = _native.lib().bsfit_server_wait(srv._h, rid, 0.0)
    assert st in (0, 12)  # done already, or BSFIT_E_TIMEOUT
    srv.wait(rid, timeout=120.0)
    srv.close()


def test_serving_multistart_matches_plain(bsfit_mod):
    """A request with per-segment starts (bsfit_server_submit_multistart):
    its 4D and 5D segments equal the plain fused multi-start bit for bit, a
    4D segment with no starts and a 3D segment equal the single-start fits."""
    import torch
    from bsfit import workloads as W
    w3 = W.workload_3d(800, s=13, stream=820)
    w4 = W.workload_4d(400, sizes=(13,), stream=821)[0]
    w5 = W.workload_5d(48, stream=822)
    z, w = float(w4.init_p[0]), float(w4.init_p[1])
    st4 = np.array([[1.2 * z, w], [z, w], [0.8 * z, w]], np.float32)
    s1 = w5.init_p.copy()
    s1[1] = W.phi_to_w(np.pi / 3)
    st5 = np.stack([w5.init_p, s1]).astype(np.float32)
    m3 = bsfit_mod.Model(6, w3.coeff)
    m4 = bsfit_mod.Model(7, w4.coeff, init_p=w4.init_p)
    m5 = bsfit_mod.Model(8, w5.coeff, coeff3=w5.coeff3, init_p=w5.init_p)
    srv = bsfit_mod.Server(max_inflight=2, arena_bytes=64 << 20)
    entries = [(m3, w3.rois, w3.iterations), (m4, w4.rois, w4.iterations),
               (m5, w5.rois, w5.iterations), (m4, w4.rois, w4.iterations)]
    rid = srv.submit(entries, starts=[None, st4, st5, []], strict=False)
    res = srv.wait(rid, timeout=120.0)
    np_ = lambda t: tuple(x.cpu().numpy() for x in t)  # noqa: E731
    ref = [
        np_(m3.fit_torch(torch.from_numpy(w3.rois).cuda(), w3.iterations)),
        np_(m4.fit_multistart_torch(torch.from_numpy(w4.rois).cuda(), w4.iterations, st4)),
        np_(m5.fit_multistart_torch(torch.from_numpy(w5.rois).cuda(), w5.iterations, st5)),
        np_(m4.fit_torch(torch.from_numpy(w4.rois).cuda(), w4.iterations)),
    ]
    torch.cuda.synchronize()
    for (Ps, Cs, Ls), (P, C, L) in zip(res, ref):
        assert np.array_equal(Ps, P.T, equal_nan=True)
        assert np.array_equal(Cs, C.T, equal_nan=True)
        assert np.array_equal(Ls, L, equal_nan=True)
    srv.close()


def test_serving_merged_launches_match_plain(bsfit_mod):
    """With merging on (bsfit_server_set_merge), queued single-start requests of
    mixed models fitted by shared launches give each request the plain call's
    results bit for bit; a multi-start request among them runs alone and is
    unchanged; every request is completed and collected once."""
    frames = _frames() * 2
    models = {}
    for kind, w in frames:
        if kind not in models:
            models[kind] = bsfit_mod.Model(w.fittype, w.coeff, coeff3=w.coeff3, init_p=w.init_p)
    srv = bsfit_mod.Server(max_inflight=2, arena_bytes=96 << 20, merge=4)
    ids = [srv.submit([(models[kind], w.rois, w.iterations)]) for kind, w in frames]
    w4 = frames[4][1]
    z, wv = float(w4.init_p[0]), float(w4.init_p[1])
    st4 = np.array([[1.2 * z, wv], [z, wv]], np.float32)
    ms = srv.submit([(models["4d"], w4.rois, w4.iterations)], starts=[st4])
    ids2 = [srv.submit([(models[kind], w.rois, w.iterations)]) for kind, w in frames[:3]]
    results = {rid: srv.wait(rid, timeout=120.0) for rid in ids + [ms] + ids2}
    st = srv.stats()
    assert st["completed"] == len(results) and st["in_flight"] == 0 and st["queued"] == 0
    assert sorted(srv.latencies()) == sorted(results)
    for rid, (kind, w) in list(zip(ids, frames)) + list(zip(ids2, frames[:3])):
        kw = {}
        if w.init_p is not None:
            kw["initP"] = w.init_p
        if w.coeff3 is not None:
            kw["coeff3"] = w.coeff3
        P, C, L = bsfit_mod.GPUmleFit_LM_multiD(w.rois, w.fittype, w.iterations, w.coeff, **kw)
        Ps, Cs, Ls = results[rid][0]
        assert np.array_equal(Ps, P, equal_nan=True), kind
        assert np.array_equal(Cs, C, equal_nan=True), kind
        assert np.array_equal(Ls, L, equal_nan=True), kind
    import torch
    P, C, L = (x.cpu().numpy() for x in models["4d"].fit_multistart_torch(
        torch.from_numpy(w4.rois).cuda(), w4.iterations, st4))
    Ps, Cs, Ls = results[ms][0]
    assert np.array_equal(Ps, P.T, equal_nan=True)
    assert np.array_equal(Ls, L, equal_nan=True)
    with pytest.raises(bsfit_mod.BsfitError):
        bsfit_mod.Server(max_inflight=1, arena_bytes=1 << 20, merge=0)
    srv.close()


@pytest.mark.parametrize("merge", [1, 4])
def test_serving_priority_launches_match_plain(bsfit_mod, merge):
    """With priority launches on (bsfit_server_set_priority: streams of three
    priorities by estimated device time, warps that end after a few ROIs),
    requests of mixed models, submitted together so that short ones run beside
    long ones, give each request the plain call's results bit for bit, and a
    multi-start request the fused multi-start call's. The two large frames (a
    3D frame of 20,000 ROIs, a 5D frame of 2,000) outnumber the warps that can
    be resident times their caps, so their launches retire and start blocks."""
    from bsfit import workloads as W
    frames = _frames() * 2 + [("3d", W.workload_3d(20000, s=11, stream=812)),
                              ("5d", W.workload_5d(2000, stream=813))]
    models = {}
    for kind, w in frames:
        if kind not in models:
            models[kind] = bsfit_mod.Model(w.fittype, w.coeff, coeff3=w.coeff3, init_p=w.init_p)
    srv = bsfit_mod.Server(max_inflight=3, arena_bytes=96 << 20, merge=merge, priority=True)
    ids = [srv.submit([(models[kind], w.rois, w.iterations)]) for kind, w in frames]
    w4 = frames[4][1]
    z, wv = float(w4.init_p[0]), float(w4.init_p[1])
    st4 = np.array([[1.2 * z, wv], [z, wv]], np.float32)
    ms = srv.submit([(models["4d"], w4.rois, w4.iterations)], starts=[st4])
    results = {rid: srv.wait(rid, timeout=120.0) for rid in ids + [ms]}
    st = srv.stats()
    assert st["completed"] == len(results) and st["in_flight"] == 0 and st["queued"] == 0
    for rid, (kind, w) in zip(ids, frames):
        kw = {}
        if w.init_p is not None:
            kw["initP"] = w.init_p
        if w.coeff3 is not None:
            kw["coeff3"] = w.coeff3
        P, C, L = bsfit_mod.GPUmleFit_LM_multiD(w.rois, w.fittype, w.iterations, w.coeff, **kw)
        Ps, Cs, Ls = results[rid][0]
        assert np.array_equal(Ps, P, equal_nan=True), kind
        assert np.array_equal(Cs, C, equal_nan=True), kind
        assert np.array_equal(Ls, L, equal_nan=True), kind
    import torch
    P, C, L = (x.cpu().numpy() for x in models["4d"].fit_multistart_torch(
        torch.from_numpy(w4.rois).cuda(), w4.iterations, st4))
    Ps, Cs, Ls = results[ms][0]
    assert np.array_equal(Ps, P.T, equal_nan=True)
    assert np.array_equal(Ls, L, equal_nan=True)
    srv.close()
