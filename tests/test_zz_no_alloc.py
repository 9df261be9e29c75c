"""The allocation-free batched entry point (bsfit_batch_fit_device_static).

It serves callers that must not allocate device memory when they fit (a
fixed-rate acquisition loop, an application owning the GPU's memory pool): the
work-queue counters live in a fixed array inside the library. This test calls it
through the C ABI twice in a row and checks each result against the
caller-scratch entry point, bsfit_batch_fit_device, on the same inputs; the
second call checks that the counters left behind by the first are cleared.
Around each static call it also reads the device's default stream-ordered
memory pool (used and reserved bytes) and torch's allocator: a call that
allocated device memory would move them. It also checks the segment limit of
the fixed array. It lives in a file that pytest collects last.
"""
import ctypes
import ctypes.util

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _segments(entries, outs, native):
    segs = (native.Segment * len(entries))()
    for k, ((m, r, it), (P, C, L)) in enumerate(zip(entries, outs)):
        segs[k].model = m._h.value
        segs[k].d_rois = r.data_ptr()
        segs[k].roi_size = r.shape[-1]
        segs[k].nfits = r.shape[0]
        segs[k].iterations = int(it)
        segs[k].d_P, segs[k].d_CRLB, segs[k].d_LL = P.data_ptr(), C.data_ptr(), L.data_ptr()
    return segs


def _pool_bytes(torch):
    """(used, reserved) bytes of the current device's default memory pool, read
    through the CUDA runtime's C API (attributes 7 and 5:
    cudaMemPoolAttrUsedMemCurrent, cudaMemPoolAttrReservedMemCurrent)."""
    name = ctypes.util.find_library("cudart") or "libcudart.so.13"
    rt = ctypes.CDLL(name)
    pool = ctypes.c_void_p()
    assert rt.cudaDeviceGetDefaultMemPool(ctypes.byref(pool), torch.cuda.current_device()) == 0
    out = []
    for attr in (7, 5):
        v = ctypes.c_uint64()
        assert rt.cudaMemPoolGetAttribute(pool, attr, ctypes.byref(v)) == 0
        out.append(v.value)
    return tuple(out)


def test_static_entry_matches_scratch_entry():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()
    import bsfit
    from bsfit import _native, workloads as W
    lib = _native.lib()
    groups = W.workload_3d_mixed(2400, sizes=(11, 13, 17), ratio=(1, 2, 1), stream=701)
    g4 = W.workload_4d(300, sizes=(15,), stream=702)[0]
    m3 = bsfit.Model(6, groups[0].coeff)
    m4 = bsfit.Model(7, g4.coeff, init_p=g4.init_p)
    entries = [(m3, torch.from_numpy(g.rois).cuda(), g.iterations) for g in groups]
    entries.append((m4, torch.from_numpy(g4.rois).cuda(), g4.iterations))

    def new_outs():
        return [(torch.full((m.nv + 1, r.shape[0]), float("nan"), device="cuda"),
                 torch.full((m.nv, r.shape[0]), float("nan"), device="cuda"),
                 torch.full((r.shape[0],), float("nan"), device="cuda")) for m, r, _ in entries]

    # reference: the caller-scratch entry point
    ref = new_outs()
    segs = _segments(entries, ref, _native)
    scratch = torch.zeros(lib.bsfit_batch_scratch_bytes(len(entries)) // 8, dtype=torch.int64,
                          device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    assert lib.bsfit_batch_fit_device(ctypes.cast(segs, ctypes.c_void_p), len(entries),
                                      scratch.data_ptr(), scratch.numel() * 8, stream) == 0
    torch.cuda.synchronize()

    for call in range(2):
        outs = new_outs()
        segs = _segments(entries, outs, _native)
        torch.cuda.synchronize()
        pool0, torch0 = _pool_bytes(torch), torch.cuda.memory_allocated()
        st = lib.bsfit_batch_fit_device_static(ctypes.cast(segs, ctypes.c_void_p), len(entries),
                                               stream)
        assert st == 0, lib.bsfit_status_str(st)
        torch.cuda.synchronize()
        assert _pool_bytes(torch) == pool0, f"call {call}: the memory pool changed"
        assert torch.cuda.memory_allocated() == torch0, f"call {call}: torch memory changed"
        for (P, C, L), (Pr, Cr, Lr) in zip(outs, ref):
            for a, b in ((P, Pr), (C, Cr), (L, Lr)):
                a, b = a.cpu().numpy(), b.cpu().numpy()
                assert not np.isnan(a[np.isfinite(b)]).any(), f"call {call}: ROIs left unfitted"
                np.testing.assert_allclose(a, b, rtol=1e-6, atol=0, equal_nan=True)

    too_many = (_native.Segment * 49)()
    assert lib.bsfit_batch_fit_device_static(ctypes.cast(too_many, ctypes.c_void_p), 49,
                                             stream) == 13
    assert b"48" in lib.bsfit_status_str(13)
