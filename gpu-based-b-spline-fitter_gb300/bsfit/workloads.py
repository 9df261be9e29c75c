"""Seeded synthetic workloads for the B-spline fitter.

The reference publishes no dataset for this path; every input here is
synthetic, seeded with ``numpy.random.default_rng``. Each workload builds a
PSF sample stack, turns it into cubic B-spline coefficients with the
reference's prefilter (``prefilter.bsarray_coeffs``), and draws Poisson ROIs
from the analytic PSF at seeded emitter positions.

Array conventions (the reference's mex layout, MATLAB column-major):
- coefficients: numpy C-order shape (..., Z, X, Y), i.e. MATLAB [Y, X, Z, ...]
  with Y fastest; ``cdims`` lists the MATLAB sizes (Y, X, Z, W, U).
- ROIs: numpy shape (N, s, s) indexed [roi, jj, ii], i.e. MATLAB [s, s, N];
  pixel (ii, jj) is ``data[s*jj + ii]``.
- Parameter 0 (x) moves the PSF along jj (the X axis), parameter 1 (y) along
  ii (the Y axis); pixel jj of a centred emitter sits at x = jj.

Lateral grid: the reference evaluates pixel jj at knot position
(s + 1) / 2 - x + jj + (nX - s) / 2 with nX = (coefficient size - 3) and
takes the spline weights from the fractional part of (s + 1) / 2 - x only
(CPUmleFit_LM.cpp:2512-2519, CPUsplineLib.cpp:1199-1230). The model is
continuous in x only when nX - s is even, so the generators use an even
number of lateral samples (odd nX) for the odd ROI sizes 11, 13, 15 and 17, with
the PSF centred on sample (nX - 1) / 2.
"""
from dataclasses import dataclass, field
import math

import numpy as np

from . import prefilter

SEED = 1234


@dataclass
class Workload:
    name: str
    fittype: int
    iterations: int
    coeff: np.ndarray            # float32, C-order (..., Z, X, Y)
    rois: np.ndarray             # float32 (N, s, s)
    truth: dict
    init_p: np.ndarray = None    # float32 shared initP (modes 7 and 8)
    coeff3: np.ndarray = None    # float32 3D coefficients (mode 8)
    extra: dict = field(default_factory=dict)

    @property
    def cdims(self):
        """MATLAB dimension sizes of the coefficient array (Y, X, Z, ...)."""
        return tuple(reversed(self.coeff.shape))

    @property
    def roi_size(self):
        return self.rois.shape[-1]

    @property
    def n_fits(self):
        # 4Pi ROIs are (channels, N, s, s)
        return self.rois.shape[1] if self.rois.ndim == 4 else self.rois.shape[0]


def _rng(stream):
    return np.random.default_rng([SEED, stream])


def _int_gauss(center, sigma, n):
    """Pixel-integrated unit Gaussian on pixels 0..n-1; center/sigma shape (N,)."""
    edges = np.arange(n + 1, dtype=np.float64)[None, :] - 0.5
    u = (edges - center[:, None]) / (math.sqrt(2.0) * sigma[:, None])
    cdf = 0.5 * (1.0 + _erf(u))
    return np.diff(cdf, axis=1)


def _erf(x):
    try:
        from scipy.special import erf
        return erf(x)
    except ImportError:  # pragma: no cover - scipy is normally present
        return np.vectorize(math.erf)(x)


def astig_sigmas(z_nm, sigma0=1.3):
    """sigma_x, sigma_y (px) of the astigmatic PSF at z (nm)."""
    z = np.asarray(z_nm, dtype=np.float64)
    sx = sigma0 * np.sqrt(1.0 + ((z - 200.0) / 400.0) ** 2)
    sy = sigma0 * np.sqrt(1.0 + ((z + 200.0) / 400.0) ** 2)
    return sx, sy


# ---------------------------------------------------------------------------
# 3D astigmatic model (fit type 6)

Z_STEP_NM = 20.0


def psf3d_samples(n_lat=26, z_lo=-600.0, z_hi=600.0, sigma0=1.3):
    """PSF stack (Z, X, Y) at 1 px lateral pitch, centre on sample (n_lat-2)/2."""
    nz = int(round((z_hi - z_lo) / Z_STEP_NM)) + 1
    z = z_lo + Z_STEP_NM * np.arange(nz)
    c = (n_lat - 2) / 2.0
    sx, sy = astig_sigmas(z, sigma0)
    gx = _int_gauss(np.full(nz, c), sx, n_lat)  # (Z, X)
    gy = _int_gauss(np.full(nz, c), sy, n_lat)  # (Z, Y)
    return gx[:, :, None] * gy[:, None, :], z


def z_to_param(z_nm, z_lo=-600.0):
    """Fit parameter z (padded knot units) for a physical z in nm."""
    return (np.asarray(z_nm) - z_lo) / Z_STEP_NM + 1.0


def param_to_z(p, z_lo=-600.0):
    return (np.asarray(p) - 1.0) * Z_STEP_NM + z_lo


def _coeff_f32(samples):
    return np.ascontiguousarray(prefilter.bsarray_coeffs(samples).astype(np.float32))


_COEFF_CACHE = {}


def coeff3d(n_lat=26, sigma0=1.3):
    key = ("3d", n_lat, sigma0)
    if key not in _COEFF_CACHE:
        s, _ = psf3d_samples(n_lat, sigma0=sigma0)
        _COEFF_CACHE[key] = _coeff_f32(s)
    return _COEFF_CACHE[key]


def rois3d(n, s, rng, sigma0=1.3, xy_spread=1.5, z_range=600.0, n_lo=1000.0, n_hi=5000.0,
           bg_lo=5.0, bg_hi=20.0):
    """Poisson ROIs of the astigmatic PSF; returns (rois, truth)."""
    cx = (s - 1) / 2.0
    x = cx + rng.uniform(-xy_spread, xy_spread, n)
    y = cx + rng.uniform(-xy_spread, xy_spread, n)
    z = rng.uniform(-z_range, z_range, n)
    photons = np.exp(rng.uniform(math.log(n_lo), math.log(n_hi), n))
    bg = rng.uniform(bg_lo, bg_hi, n)
    sx, sy = astig_sigmas(z, sigma0)
    gx = _int_gauss(x, sx, s)   # along jj
    gy = _int_gauss(y, sy, s)   # along ii
    model = bg[:, None, None] + photons[:, None, None] * gx[:, :, None] * gy[:, None, :]
    rois = rng.poisson(model).astype(np.float32)
    truth = dict(x=x, y=y, z_nm=z, z=z_to_param(z), N=photons, bg=bg)
    return rois, truth


def workload_3d(n=10000, s=13, iterations=30, stream=1):
    """Plain 3D astigmatic fit: n ROIs of s x s, 30 LM iterations."""
    rng = _rng(stream)
    rois, truth = rois3d(n, s, rng)
    return Workload(f"3d_{s}px", 6, iterations, coeff3d(), rois, truth)


def workload_3d_mixed(n=1_000_000, sizes=(11, 13, 17), ratio=(1, 2, 1), iterations=30,
                      stream=2):
    """Batched 3D: ROIs of several sizes (ratio 1:2:1); one Workload per size."""
    rng = _rng(stream)
    tot = sum(ratio)
    counts = [n * r // tot for r in ratio]
    counts[sizes.index(13) if 13 in sizes else 0] += n - sum(counts)
    out = []
    for s, c in zip(sizes, counts):
        rois, truth = rois3d(c, s, rng)
        out.append(Workload(f"3d_{s}px", 6, iterations, coeff3d(), rois, truth))
    return out


# ---------------------------------------------------------------------------
# 4D colour model (fit type 7)

def color_sigma(lam):
    """Base sigma (px) for colour coordinate lam in [0, 1]."""
    return 1.2 + 0.25 * np.asarray(lam, dtype=np.float64)


def psf4d_samples(n_lat=26, z_lo=-600.0, z_hi=600.0):
    """(W, Z, X, Y) stack; the colour axis is end-padded like the reference's
    colour demo (bspline_based_color_classification_v3.m:19-25): samples
    [l0, l0, l1/3, l2/3, l1, l1, l1], so colour lam sits at w = 2 + 3 lam."""
    lam_knots = np.array([0.0, 0.0, 1 / 3, 2 / 3, 1.0, 1.0, 1.0])
    stacks = []
    for lam in lam_knots:
        s3, z = psf3d_samples(n_lat, z_lo, z_hi, sigma0=float(color_sigma(lam)))
        stacks.append(s3)
    return np.stack(stacks, axis=0), z


def lam_to_w(lam):
    return 2.0 + 3.0 * np.asarray(lam)


def coeff4d(n_lat=26):
    key = ("4d", n_lat)
    if key not in _COEFF_CACHE:
        s, _ = psf4d_samples(n_lat)
        _COEFF_CACHE[key] = _coeff_f32(s)
    return _COEFF_CACHE[key]


def workload_4d(n=500_000, sizes=(13, 15), iterations=60, stream=3):
    """3D + colour: ROIs of 13 and 15 px (half each); one Workload per size."""
    rng = _rng(stream)
    out = []
    counts = [n // len(sizes)] * len(sizes)
    counts[0] += n - sum(counts)
    for s, c in zip(sizes, counts):
        cx = (s - 1) / 2.0
        x = cx + rng.uniform(-1.5, 1.5, c)
        y = cx + rng.uniform(-1.5, 1.5, c)
        z = rng.uniform(-600.0, 600.0, c)
        lam = rng.uniform(0.0, 1.0, c)
        photons = np.exp(rng.uniform(math.log(800.0), math.log(4000.0), c))
        bg = rng.uniform(5.0, 15.0, c)
        sx, sy = astig_sigmas(z, 1.0)
        sc = color_sigma(lam)
        gx = _int_gauss(x, sx * sc, s)
        gy = _int_gauss(y, sy * sc, s)
        model = bg[:, None, None] + photons[:, None, None] * gx[:, :, None] * gy[:, None, :]
        rois = rng.poisson(model).astype(np.float32)
        truth = dict(x=x, y=y, z_nm=z, z=z_to_param(z), lam=lam, w=lam_to_w(lam), N=photons, bg=bg)
        init_p = np.array([z_to_param(0.0), lam_to_w(0.5)], dtype=np.float32)
        out.append(Workload(f"4d_{s}px", 7, iterations, coeff4d(), rois, truth, init_p=init_p))
    return out


# ---------------------------------------------------------------------------
# 5D orientation model (fit type 8)

N_AZ = 18      # azimuth samples per period (20 deg)
N_POL = 9      # polar samples
POL_STEP = 10.0


def dipole_lobes(x, y, z_nm, phi, theta, s):
    """Three astigmatic lobes weighted by the dipole orientation.

    Lobe weights sin^2(t)cos^2(p), sin^2(t)sin^2(p), cos^2(t); every lobe is
    shifted laterally by 0.4 px * (sin t cos p, sin t sin p)."""
    st, ct = np.sin(theta), np.cos(theta)
    sp, cp = np.sin(phi), np.cos(phi)
    w = [st ** 2 * cp ** 2, st ** 2 * sp ** 2, ct ** 2]
    dx = 0.4 * st * cp
    dy = 0.4 * st * sp
    sx, sy = astig_sigmas(z_nm, 1.3)
    sig = [(sx, sy), (sy, sx), (0.5 * (sx + sy) * 1.1, 0.5 * (sx + sy) * 1.1)]
    out = 0.0
    for wi, (gsx, gsy) in zip(w, sig):
        gx = _int_gauss(x + dx, gsx, s)
        gy = _int_gauss(y + dy, gsy, s)
        out = out + wi[:, None, None] * gx[:, :, None] * gy[:, None, :]
    return out


def psf5d_samples(n_lat=34, z_lo=-400.0, z_hi=400.0, n_az=N_AZ, n_pol=N_POL):
    """(U, W, Z, X, Y) stack over one azimuth period and the polar grid."""
    nz = int(round((z_hi - z_lo) / Z_STEP_NM)) + 1
    zs = z_lo + Z_STEP_NM * np.arange(nz)
    c = (n_lat - 2) / 2.0
    out = np.zeros((n_pol, n_az, nz, n_lat, n_lat))
    for iu in range(n_pol):
        th = np.deg2rad(POL_STEP * iu)
        for iw in range(n_az):
            ph = 2 * np.pi * iw / n_az
            # lobes at every z of the grid, emitter at the sample centre
            lob = dipole_lobes(np.full(nz, c), np.full(nz, c), zs, np.full(nz, ph),
                               np.full(nz, th), n_lat)
            out[iu, iw] = lob
    return out, zs


def coeff5d(n_lat=34, z_lo=-400.0, z_hi=400.0, n_az=N_AZ, n_pol=N_POL):
    """5D coefficients (U, W, Z, X, Y) and the orientation-averaged 3D ones.

    The azimuth axis W is periodic: the fitter wraps w into (1, nW - 1] with
    period nW - 2 (CPUmleFit_LM.cpp:3436-3443), so the coefficients along W are
    the periodic interpolating spline laid out as c[m] = c_per[(m - 2) mod n_az]
    for m = 0 .. n_az + 4 (nW = n_az + 2). The polar axis U uses the mirror
    prefilter."""
    key = ("5d", n_lat, z_lo, z_hi, n_az, n_pol)
    if key not in _COEFF_CACHE:
        s, _ = psf5d_samples(n_lat, z_lo, z_hi, n_az, n_pol)
        c = s
        for ax in (2, 3, 4):           # Z, X, Y: mirror prefilter
            c = prefilter.filter_axis(c, ax)
        c = prefilter.filter_axis(c, 0)  # U: mirror
        c = prefilter.filter_axis_periodic(c, 1)  # W: periodic
        c = prefilter.mirror_pad(c, axes=(0, 2, 3, 4))
        m = np.arange(n_az + 5)
        c = np.take(c, (m - 2) % n_az, axis=1)
        c5 = np.ascontiguousarray(c.astype(np.float32))
        s3 = s.mean(axis=(0, 1))
        c3 = _coeff_f32(s3)
        _COEFF_CACHE[key] = (c5, c3)
    return _COEFF_CACHE[key]


def phi_to_w(phi):
    return np.asarray(phi) / (2 * np.pi / N_AZ) + 2.0


def theta_to_u(theta):
    return np.rad2deg(np.asarray(theta)) / POL_STEP + 1.0


def workload_5d(n=100_000, s=17, iterations=60, stream=5):
    rng = _rng(stream)
    c5, c3 = coeff5d()
    cx = (s - 1) / 2.0
    x = cx + rng.uniform(-1.0, 1.0, n)
    y = cx + rng.uniform(-1.0, 1.0, n)
    z = rng.uniform(-300.0, 300.0, n)
    phi = rng.uniform(0.0, 2 * np.pi, n)
    theta = np.deg2rad(rng.uniform(10.0, 70.0, n))
    photons = rng.uniform(2000.0, 8000.0, n)
    bg = rng.uniform(5.0, 20.0, n)
    model = bg[:, None, None] + photons[:, None, None] * dipole_lobes(x, y, z, phi, theta, s)
    rois = rng.poisson(model).astype(np.float32)
    truth = dict(x=x, y=y, z_nm=z, z=z_to_param(z, -400.0), phi=phi, w=phi_to_w(phi),
                 theta=theta, u=theta_to_u(theta), N=photons, bg=bg, g2=np.ones(n))
    init_p = np.array([z_to_param(0.0, -400.0), phi_to_w(np.pi), theta_to_u(np.deg2rad(40.0)),
                       0.7], dtype=np.float32)
    return Workload(f"5d_{s}px", 8, iterations, c5, rois, truth, init_p=init_p, coeff3=c3)


# ---------------------------------------------------------------------------
# 4Pi model (four interference channels, GPUmleFit_LM_4Pi_bspline)

N_PHI = 32                       # phase knots per period
PHI_STEP = 2 * np.pi / N_PHI
LAMBDA_NM = 668.0                # emission wavelength of the reference's demo
PHASE_SHIFTS = np.array([0.0, 0.5 * np.pi, np.pi, 1.5 * np.pi])


def modulation(z_nm):
    """Interference contrast of the synthetic 4Pi PSF (falls off with |z|)."""
    return 0.8 * np.exp(-(np.asarray(z_nm) / 900.0) ** 2)


def psf4pi_samples(n_lat=26, z_lo=-600.0, z_hi=600.0):
    """Phase-resolved PSF stack (W, Z, X, Y): the astigmatic PSF times
    1 + m(z) cos(phase), at phases 0 .. (N_PHI + 1) * PHI_STEP (one period plus
    one sample, as bspline_based_4piloc_v4.m:80-86 samples it)."""
    base, z = psf3d_samples(n_lat, z_lo, z_hi)
    ph = PHI_STEP * np.arange(N_PHI + 2)
    m = modulation(z)
    out = base[None] * (1.0 + m[None, :, None, None] * np.cos(ph)[:, None, None, None])
    return out, z


def coeff4pi(n_lat=26):
    """Mirror-prefiltered coefficients (W, Z, X, Y): W = N_PHI + 4 along the phase
    axis, so the fitter's period is W - 4 = N_PHI knots."""
    key = ("4pi", n_lat)
    if key not in _COEFF_CACHE:
        s, _ = psf4pi_samples(n_lat)
        _COEFF_CACHE[key] = _coeff_f32(s)
    return _COEFF_CACHE[key]


def phase_to_w(phi):
    """Phase (rad) to the fit's phase position: knot units with the +1 origin
    (simBSplinePSF.m: wc = Phi / dphidN + 1)."""
    return np.mod(np.asarray(phi), 2 * np.pi) / PHI_STEP + 1.0


def rois4pi(n, s, rng, z_range=500.0, n_lo=1000.0, n_hi=5000.0, bg_lo=10.0, bg_hi=30.0,
            xy_spread=1.0):
    """Poisson ROIs of the four channels, (4, N, s, s); photons and background
    per channel, shared by the channels; phase = 4 pi z / lambda."""
    cx = (s - 1) / 2.0
    x = cx + rng.uniform(-xy_spread, xy_spread, n)
    y = cx + rng.uniform(-xy_spread, xy_spread, n)
    z = rng.uniform(-z_range, z_range, n)
    phi = np.mod(4 * np.pi * z / LAMBDA_NM, 2 * np.pi)
    photons = np.exp(rng.uniform(math.log(n_lo), math.log(n_hi), n))
    bg = rng.uniform(bg_lo, bg_hi, n)
    sx, sy = astig_sigmas(z, 1.3)
    base = _int_gauss(x, sx, s)[:, :, None] * _int_gauss(y, sy, s)[:, None, :]
    m = modulation(z)
    rois = np.empty((4, n, s, s), np.float32)
    for c, sh in enumerate(PHASE_SHIFTS):
        mod = 1.0 + m * np.cos(phi + sh)
        model = bg[:, None, None] + photons[:, None, None] * mod[:, None, None] * base
        rois[c] = rng.poisson(model)
    truth = dict(x=x, y=y, z_nm=z, z=z_to_param(z), phi=phi, w=phase_to_w(phi), N=photons, bg=bg)
    return rois, truth


def workload_4pi(n=100_000, s=13, iterations=100, stream=6, start_phase=2 * np.pi):
    """4Pi fit as the reference's demo runs it: 13 px ROIs in four channels,
    100 iterations, z started mid-range and the phase at one start value."""
    rng = _rng(stream)
    rois, truth = rois4pi(n, s, rng)
    init_z = np.full(n, z_to_param(0.0), np.float32)
    init_phi = np.full(n, start_phase / PHI_STEP, np.float32)
    dT = np.zeros((n, 4, 6), np.float32)
    extra = dict(dT=dT, init_z=init_z, init_phi=init_phi,
                 phase_shift=(PHASE_SHIFTS / PHI_STEP).astype(np.float32))
    return Workload(f"4pi_{s}px", 9, iterations, coeff4pi(), rois, truth, extra=extra)


# ---------------------------------------------------------------------------
# 4Pi workload of the benchmark's stated 4Pi configuration: four channels
# I_c = G(x, y, z) [1 + 0.8 cos(psi + c pi/2)] with the interference phase
# psi = 2 pi z / 260 nm + phi, a per-ROI phase offset phi; 16 px ROIs; the
# coefficient grid samples 33 x 33 lateral, 61 z (-600..600 nm) and 16 phases
# per period, periodic in phase; per-channel lateral offsets uniform within
# +-0.5 px; photons split evenly over the channels.

N_PHI_C4 = 16
PHI_STEP_C4 = 2 * np.pi / N_PHI_C4
PHASE_PERIOD_NM_C4 = 260.0
C4_LAT = 33


def _c4_centre(s, n_lat=C4_LAT):
    """Sample index of the PSF centre for s px ROIs on an n_lat-sample lateral
    grid: pixel jj of an emitter at x sits at knot (s + 1) // 2 - x + jj +
    (nX - s) / 2 with nX = n_lat - 1 (CPUmleFit_LM.cpp:2512-2519), and sample j
    at knot j + 1."""
    return (s + 1) // 2 + (n_lat - 1 - s) / 2.0 - 1.0


def psf4pi_c4_samples(s=16, n_lat=C4_LAT, z_lo=-600.0, z_hi=600.0, n_phi=N_PHI_C4):
    """(W, Z, X, Y): the astigmatic PSF times 1 + 0.8 cos(phase) at n_phi
    phases over one period."""
    nz = int(round((z_hi - z_lo) / Z_STEP_NM)) + 1
    z = z_lo + Z_STEP_NM * np.arange(nz)
    c = _c4_centre(s, n_lat)
    sx, sy = astig_sigmas(z, 1.3)
    base = _int_gauss(np.full(nz, c), sx, n_lat)[:, :, None] * _int_gauss(np.full(nz, c), sy, n_lat)[:, None, :]
    ph = PHI_STEP_C4 * np.arange(n_phi)
    return base[None] * (1.0 + 0.8 * np.cos(ph))[:, None, None, None], z


def coeff4pi_c4(s=16, n_lat=C4_LAT, n_phi=N_PHI_C4):
    """Coefficients (W, Z, X, Y): mirror prefilter and pad along Z, X, Y; the
    periodic interpolating spline along the phase, laid out for the fitter's
    wrap (period W - 4 knots, phase position w in [1, 1 + period), sample j at
    w = j + 1): plane m holds the periodic coefficient (m - 1) mod n_phi, for
    m = 0 .. n_phi + 3."""
    key = ("4pi_c4", s, n_lat, n_phi)
    if key not in _COEFF_CACHE:
        smp, _ = psf4pi_c4_samples(s, n_lat, n_phi=n_phi)
        c = smp
        for ax in (1, 2, 3):
            c = prefilter.filter_axis(c, ax)
        c = prefilter.filter_axis_periodic(c, 0)
        c = prefilter.mirror_pad(c, axes=(1, 2, 3))
        m = np.arange(n_phi + 4)
        c = np.take(c, (m - 1) % n_phi, axis=0)
        _COEFF_CACHE[key] = np.ascontiguousarray(c.astype(np.float32))
    return _COEFF_CACHE[key]


def workload_4pi_c4(n=250_000, s=16, iterations=100, stream=7, z_range=500.0, chunk=65536):
    """The stated 4Pi configuration: n ROIs of 4 x s x s; x, y within +-1 px of
    the centre, z uniform within +-z_range nm, phase offset uniform on [0, 2 pi),
    total photons log-uniform 2000-10000 split evenly over the channels,
    background uniform 5-20 per pixel and channel, per-channel lateral offsets
    uniform within +-0.5 px (passed to the fit as dT). One start: z mid-range,
    phase at the first knot."""
    rng = _rng(stream)
    cx = (s - 1) / 2.0
    x = cx + rng.uniform(-1.0, 1.0, n)
    y = cx + rng.uniform(-1.0, 1.0, n)
    z = rng.uniform(-z_range, z_range, n)
    phi = rng.uniform(0.0, 2 * np.pi, n)
    psi = np.mod(2 * np.pi * z / PHASE_PERIOD_NM_C4 + phi, 2 * np.pi)
    n_tot = np.exp(rng.uniform(math.log(2000.0), math.log(10000.0), n))
    photons = n_tot / 4.0
    bg = rng.uniform(5.0, 20.0, n)
    dT = np.zeros((n, 4, 6), np.float32)
    dT[:, :, 0] = rng.uniform(-0.5, 0.5, (n, 4))
    dT[:, :, 1] = rng.uniform(-0.5, 0.5, (n, 4))
    sx, sy = astig_sigmas(z, 1.3)
    rois = np.empty((4, n, s, s), np.float32)
    for c in range(4):
        for b in range(0, n, chunk):
            e = min(n, b + chunk)
            gx = _int_gauss(x[b:e] + dT[b:e, c, 0], sx[b:e], s)
            gy = _int_gauss(y[b:e] + dT[b:e, c, 1], sy[b:e], s)
            mod = 1.0 + 0.8 * np.cos(psi[b:e] + c * 0.5 * np.pi)
            model = bg[b:e, None, None] + (photons[b:e] * mod)[:, None, None] * gx[:, :, None] * gy[:, None, :]
            rois[c, b:e] = rng.poisson(model)
    truth = dict(x=x, y=y, z_nm=z, z=z_to_param(z), phi=phi, psi=psi,
                 w=psi / PHI_STEP_C4 + 1.0, N=photons, bg=bg)
    init_z = np.full(n, z_to_param(0.0), np.float32)
    init_phi = np.full(n, 1.0, np.float32)
    shifts = (np.arange(4) * 0.5 * np.pi / PHI_STEP_C4).astype(np.float32)
    extra = dict(dT=dT, init_z=init_z, init_phi=init_phi, phase_shift=shifts)
    return Workload(f"4pi_c4_{s}px", 9, iterations, coeff4pi_c4(s), rois, truth, extra=extra)
