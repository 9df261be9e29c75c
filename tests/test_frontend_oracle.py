"""The front-end restatement (oracle/frontend.py) on CPU: its non-maximum
suppression equals the reference's own peak finder (maximumfind2.c, compiled
here from the reference's source) on random, plateau and tie-heavy images, and
the filter kernels are the documented fspecial Gaussian (normalised,
symmetric). Skipped for the peak finder where the reference sources are absent."""
import numpy as np
import pytest

from oracle import frontend as FE


@pytest.fixture(scope="module")
def ref_nms():
    from oracle import build
    if not FE.reference_nms_available():
        try:
            build.build_reference()
        except Exception:
            pass
    if not FE.reference_nms_available():
        pytest.skip("reference sources absent: peak finder not built")
    return FE.reference_nms


@pytest.mark.parametrize("seed,shape,levels", [(1, (40, 30), None), (2, (17, 64), 4),
                                               (3, (64, 64), 2), (4, (5, 3), None)])
def test_nms_matches_reference(ref_nms, seed, shape, levels):
    rng = np.random.default_rng(seed)
    img = rng.random(shape).astype(np.float32)
    if levels:
        img = np.floor(img * levels).astype(np.float32)  # plateaus and ties
    assert FE.nms(img) == ref_nms(img)


def test_kernels():
    for sigma in (0.8, 1.0, 1.7, 3.0):
        g = FE.peak_kernel(0, sigma)
        assert g.shape[0] == max(3, int(np.ceil(3 * sigma + 1)))
        assert abs(g.sum() - 1.0) < 1e-12 and np.allclose(g, g.T) and np.allclose(g, g[::-1, ::-1])
        d = FE.peak_kernel(1, sigma)
        assert abs(d.sum()) < 1e-12


def test_filter_is_correlation():
    rng = np.random.default_rng(5)
    x = rng.random((9, 11))
    h = np.zeros((3, 3))
    h[0, 2] = 1.0  # row -1, column +1 relative to the centre
    y = FE.filter2_same(h, x)  # [x][y]: y(i,j) = X(i-1, j+1) in (row, col)
    assert np.allclose(y[:-1, 1:], x[1:, :-1])
