"""Generate the golden fixtures in this folder from the reference itself.

Runs the reference's own CPU fitter, compiled from its sources by
``oracle/build_ref.sh`` (FP32 as shipped and the float-promoted FP64 build),
on small seeded inputs, and stores inputs and outputs as ``.npz`` files. The
GPU tests read these files; they never need the reference sources.

Usage (where the reference sources exist): python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "gpu-based-b-spline-fitter_gb300"))

from bsfit import workloads as W  # noqa: E402
from oracle.oracle import ReferenceOracle  # noqa: E402


def rng(tag):
    return np.random.default_rng([W.SEED, 900, tag])


def coeff3(n_lat, z_lo, z_hi):
    s, _ = W.psf3d_samples(n_lat, z_lo, z_hi)
    return np.ascontiguousarray(W.prefilter.bsarray_coeffs(s).astype(np.float32))


def rois3(n, s, r, spread=1.5, z_range=200.0):
    rois, truth = W.rois3d(n, s, r, xy_spread=spread, z_range=z_range)
    return rois


def save(name, ref, rois, fittype, iterations, coeff, init_p=None, coeff3=None, note=""):
    out = dict(rois=rois.astype(np.float32), fittype=np.int32(fittype),
               iterations=np.int32(iterations), coeff=coeff, note=np.array(note))
    if init_p is not None:
        out["init_p"] = np.asarray(init_p, np.float32)
    if coeff3 is not None:
        out["coeff3"] = coeff3
    for prec in ("f32", "f64"):
        P, C, L = ref.fit(rois, fittype, iterations, coeff, init_p=init_p, coeff3=coeff3,
                          precision=prec)
        out[f"{prec}_P"], out[f"{prec}_CRLB"], out[f"{prec}_LL"] = P, C, L
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, rois.shape, "->", os.path.getsize(os.path.join(HERE, name + ".npz")), "bytes")


def special_rois(s, r):
    """All-zero, negative-pixel, single-bright-pixel and constant ROIs."""
    out = np.zeros((4, s, s), np.float32)
    out[1] = r.poisson(10.0, (s, s)).astype(np.float32) - 12.0
    out[2, s // 2 + 1, s // 2 - 2] = 500.0
    out[3] = 7.0
    return out


def main():
    ref = ReferenceOracle()
    # Fit type 6 (3D). Grid of 20 lateral samples: nX - s = 6 for s = 13.
    c = coeff3(20, -200.0, 200.0)
    base = rois3(48, 13, rng(1))
    save("m6_basic", ref, base, 6, 30, c, note="3D, 20x20x21 samples, s=13, 30 iterations")
    save("m6_iters", ref, base[:8], 6, 3, c, note="iteration cap 3")
    save("m6_iters1", ref, base[:8], 6, 1, c, note="iteration cap 1")
    save("m6_iters0", ref, base[:8], 6, 0, c, note="iteration cap 0")
    edge = rois3(12, 13, rng(2), spread=4.0, z_range=200.0)
    edge = np.concatenate([edge, special_rois(13, rng(3))])
    save("m6_edges", ref, edge, 6, 30, c,
         note="emitters up to 4 px off centre; zero, negative, single-pixel, constant ROIs")
    # Odd sample count: nX - s odd, half-integer lateral offset.
    c21 = coeff3(21, -200.0, 200.0)
    save("m6_halfoffset", ref, rois3(16, 13, rng(4)), 6, 30, c21,
         note="21 lateral samples: offset (nX - s)/2 = 3.5")
    # ROI sizes: 22 lateral samples (nX = 21) keep nX - s even for odd s.
    c22 = coeff3(22, -200.0, 200.0)
    for s in (5, 7, 11, 15, 17, 20):
        save(f"m6_size{s}", ref, rois3(8, s, rng(10 + s)), 6, 30, c22, note=f"s={s}")
    # Largest ROI the reference accepts (51).
    c54 = coeff3(54, -100.0, 100.0)
    save("m6_size51", ref, rois3(3, 51, rng(5)), 6, 30, c54, note="s=51 (IMSZBIG)")
    # Fit type 7 (4D colour), small grid.
    s4, _ = W.psf4d_samples(20, -200.0, 200.0)
    c4 = np.ascontiguousarray(W.prefilter.bsarray_coeffs(s4).astype(np.float32))
    r7 = rng(7)
    wl = W.workload_4d(64, sizes=(13,), iterations=60, stream=77)[0]
    # regenerate ROIs on the small grid's z range
    rois7 = []
    for i in range(32):
        x, y = 6 + r7.uniform(-1.5, 1.5, 2)
        z = r7.uniform(-150, 150)
        lam = r7.uniform(0, 1)
        sx, sy = W.astig_sigmas(np.array([z]), 1.0)
        sc = W.color_sigma(lam)
        gx = W._int_gauss(np.array([x]), sx * sc, 13)
        gy = W._int_gauss(np.array([y]), sy * sc, 13)
        m = r7.uniform(5, 15) + r7.uniform(800, 4000) * gx[0][:, None] * gy[0][None, :]
        rois7.append(r7.poisson(m))
    rois7 = np.array(rois7, np.float32)
    del wl
    ip = np.array([W.z_to_param(0.0, -200.0), W.lam_to_w(0.5)], np.float32)
    save("m7_basic", ref, rois7, 7, 60, c4, init_p=ip, note="4D colour, initP=(z0, w0)")
    save("m7_initp0", ref, rois7[:16], 7, 60, c4, init_p=np.zeros(2, np.float32),
         note="4D colour, initP=0 selects mid-grid")
    # Fit type 8 (5D + 3D mixture), small grid: 18 lateral samples, s = 11.
    c5, c3 = W.coeff5d(18, -80.0, 80.0, n_az=5, n_pol=4)
    r8 = rng(8)
    n8 = 16
    x = 5 + r8.uniform(-1, 1, n8)
    y = 5 + r8.uniform(-1, 1, n8)
    z = r8.uniform(-60, 60, n8)
    phi = r8.uniform(0, 2 * np.pi, n8)
    th = np.deg2rad(r8.uniform(5, 25, n8))
    m = r8.uniform(5, 20, n8)[:, None, None] + r8.uniform(2000, 8000, n8)[:, None, None] * \
        W.dipole_lobes(x, y, z, phi, th, 11)
    rois8 = r8.poisson(m).astype(np.float32)
    ip8 = np.array([W.z_to_param(0.0, -80.0), 3.0, 2.0, 0.7], np.float32)
    save("m8_basic", ref, rois8, 8, 60, c5, init_p=ip8, coeff3=c3,
         note="5D+3D mixture, 18 lateral samples, 9 z, period-5 azimuth, 4 polar, s=11")


if __name__ == "__main__":
    main()
