import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "gpu-based-b-spline-fitter_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")

Z_NM_PER_UNIT = 20.0


def tol_pass(P, C, R, RC, nv, z_nm=Z_NM_PER_UNIT):
    ok = np.abs(P[:, :2] - R[:, :2]).max(1) <= 1e-4
    ok &= np.abs(P[:, 4] - R[:, 4]) * z_nm <= 1e-2
    with np.errstate(divide="ignore", invalid="ignore"):
        ok &= np.abs(P[:, 2] / R[:, 2] - 1) <= 1e-5
        ok &= np.abs(P[:, 3] / R[:, 3] - 1) <= 1e-5
        for k in range(5, nv):
            ok &= np.abs(P[:, k] - R[:, k]) <= 1e-4
        big_r = (RC > 1e25) | ~np.isfinite(RC)
        big_c = (C > 1e25) | ~np.isfinite(C)
        relc = np.abs(C / RC - 1)
        relc[big_r & big_c] = 0
        ok &= (relc <= 1e-4).all(1)
    return ok


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def golden_cases():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle
    return Oracle()
