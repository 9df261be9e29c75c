"""Evaluations at the edges of the non-lateral knot ranges (fit types 7 and 8).

The FP32 kernels gather a lateral node's four z planes from the model's gather
table (for fit type 7 two w layers interleaved per entry, for fit type 8 the
mixture's 3D table): the entries of the first and last knots are the ones a
layout slip would read wrong. Here z, w and u sit at the ends of the range the
fit keeps them in (z in [0, nZ - 0.5], w in [0, nW - 0.5] for fit type 7,
u in [1, nU - 0.5]: VC/CPUmleFit_LM/CPUmleFit_LM.cpp:3003-3010, :3421-3447),
on and between the first and last knots, and the evaluation (deviance,
gradient, Hessian; Fisher information and log-likelihood) must agree with the
FP64 oracle's at the same parameters, with the tolerances of
test_fit_gpu.test_eval_matches_oracle_at_fixed_parameters."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from test_fit_gpu import bsfit_mod  # noqa: F401

pytestmark = pytest.mark.gpu


def _edge_thetas(theta, ft, n):
    """Copies of the fitted parameters with (z, w[, u]) moved to knot-range
    edges, one combination per ROI (cycled)."""
    nz, nw = n[2], n[3]
    zs = [0.0, 0.25, 1.0, nz - 1.0, nz - 0.75, nz - 0.5]
    if ft == 7:
        ws = [0.0, 0.3, 1.0, nw - 1.0, nw - 0.5]
        combos = [(z, w, None) for z in zs for w in ws]
    else:
        nu = n[4]
        ws = [1.0, 1.5, nw - 1.0]  # the fit keeps the periodic azimuth in (1, nW - 1]
        us = [1.0, 1.25, nu - 1.0, nu - 0.5]
        combos = [(z, w, u) for z in zs for w in ws for u in us]
    out = np.repeat(theta, (len(combos) + len(theta) - 1) // len(theta), axis=0)[:len(combos)]
    out = out.copy()
    for i, (z, w, u) in enumerate(combos):
        out[i, 4] = z
        out[i, 5] = w
        if u is not None:
            out[i, 6] = u
    return out.astype(np.float32)


@pytest.mark.parametrize("case", ["m7_basic", "m8_basic"])
def test_eval_at_knot_range_edges(bsfit_mod, oracle, case):
    import torch
    d = np.load(os.path.join(GOLDEN, case + ".npz"))
    ft = int(d["fittype"])
    nv = {7: 6, 8: 8}[ft]
    dims = list(reversed(d["coeff"].shape))  # MATLAB order (Y, X, Z, W, U)
    n = [dims[1] - 3, dims[0] - 3] + [c - 3 for c in dims[2:]]
    theta = _edge_thetas(d["f64_P"][:, :nv], ft, n)
    rois = np.resize(d["rois"], (len(theta),) + d["rois"].shape[1:]).astype(np.float32)
    c3 = d["coeff3"] if "coeff3" in d else None
    m = bsfit_mod.Model(ft, d["coeff"], coeff3=c3, init_p=d["init_p"])
    r = torch.from_numpy(np.ascontiguousarray(rois)).cuda()
    th = torch.from_numpy(np.ascontiguousarray(theta.T)).cuda()
    idx = [(l, k) for l in range(nv) for k in range(l, nv)]
    for fisher in (False, True):
        g = m.eval_torch(r, th, fisher=fisher).cpu().numpy().astype(np.float64)
        ref = oracle.eval(rois, ft, d["coeff"], theta.astype(np.float64), fisher=fisher,
                          coeff3=c3)
        assert np.isfinite(g).all() and np.isfinite(ref).all()
        diag = np.stack([ref[:, 1 + nv + idx.index((k, k))] for k in range(nv)], 1)
        # At these edges some derivatives vanish identically (the curvature of
        # z, w or u drops to 1e-13..1e-33 on the mirror-padded boundary knots),
        # where the FP32 sums keep rounding noise of the terms' usual size: the
        # curvature floor is 1e-3 of the parameter's median curvature (1e-6 at
        # the interior positions of the fixed-parameter test).
        diag = np.maximum(diag, 1e-3 * np.median(diag, 0))
        e0 = np.abs(g[:, 0] - ref[:, 0]).max() / np.abs(ref[:, 0]).max()
        eJ = (np.abs(g[:, 1:1 + nv] - ref[:, 1:1 + nv]) / np.sqrt(diag)).max()
        eH = max((np.abs(g[:, 1 + nv + i] - ref[:, 1 + nv + i]) /
                  np.sqrt(diag[:, l] * diag[:, k])).max() for i, (l, k) in enumerate(idx))
        tol = 1e-3 if ft != 8 else 1e-2
        assert e0 < 1e-5 and eJ < tol and eH < tol, (case, fisher, e0, eJ, eH)
    m.close()
