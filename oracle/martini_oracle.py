"""CPU FP64 oracle for MARTINI source insertion (test infrastructure only).

This module is the checker, not the product: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import
it.  It restates, in plain numpy/scipy FP64, the algorithm of the reference
package ``astromartini`` 2.1.18 (kyleaoman/martini) for the source-insertion
path ``Martini.insert_source_in_cube``.  Every function cites the reference
lines it follows (paths are relative to the reference project root).

Parity of this restatement is pinned against golden vectors produced by the
reference's own code (``tests/golden/make_golden.py`` runs the reference's
``_kernel_integral``, ``_init_sm_lengths`` selection, ``_prune_particles``,
``init_spectra`` and ``_evaluate_pixel_spectrum`` under a dimensionless units
shim, because astropy is not installed) and against the reference test-suite's
known answers (thermal width 9.0853727258 km/s at 1e4 K, kernel selection
[0, 0, 2, 1], unit spectrum sums, pixel coordinates).

Two insertion forms are provided:

* ``insert_perpixel`` -- the reference's own loop structure: one call of
  ``evaluate_pixel_spectrum`` per pixel, each scanning all particles with the
  Chebyshev-box mask (martini/martini.py:243-283, :327-343).  Its cost is
  O(N_pix * N); it is what the CPU baseline times.
* ``insert_scatter`` -- the same arithmetic reorganised per particle over its
  footprint box (identical mask predicate, identical weights and spectra), for
  parity checks at sizes where the per-pixel loop is too slow.
"""

from __future__ import annotations

import math
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
from scipy.optimize import fsolve
from scipy.special import erf

# Physical constants (CODATA 2018, the values astropy 5/6 ship; the reference
# test tests/test_spectral_models.py:43-48 expects 9.0853727258 km/s at 1e4 K).
K_B = 1.380649e-23  # J/K
M_P = 1.67262192369e-27  # kg
C_KMS = 299792.458  # km/s
HI_FREQ_HZ = 1.420405751e9  # martini/datacube.py:21
MHI_TO_JY = 2.36e5  # martini/spectral_models.py:127-145

# Kernel type codes shared with the CUDA path (include/martini_gb300.h).
KT_WENDLAND_C2 = 0
KT_WENDLAND_C6 = 1
KT_CUBIC_SPLINE = 2
KT_QUARTIC_SPLINE = 3
KT_GAUSSIAN = 4
KT_DIRAC = 5

GAUSS_SIG = 1.0 / (2.0 * np.sqrt(2.0 * np.log(2.0)))  # sph_kernels.py:1020


# ---------------------------------------------------------------------------
# Kernel functions and constants (martini/sph_kernels.py)
# ---------------------------------------------------------------------------


def kernel_profile(ktype: int, q: np.ndarray, truncate: float = 3.0) -> np.ndarray:
    """3D kernel W(q) normalised to unit volume.

    WendlandC2 sph_kernels.py:366-393, WendlandC6 :507-542, cubic spline
    :761-789, Gaussian :962-992, quartic spline :1438-1484.
    """
    q = np.asarray(q, dtype=np.float64)
    if ktype == KT_WENDLAND_C2:
        return np.where(q < 1, np.power(1 - q, 4) * (4 * q + 1), 0) * (21 / 2 / np.pi)
    if ktype == KT_WENDLAND_C6:
        return np.where(
            q < 1,
            np.power(1 - q, 8) * (1 + 8 * q + 25 * q**2 + 32 * q**3),
            0,
        ) * (1365 / 64 / np.pi)
    if ktype == KT_CUBIC_SPLINE:
        w = np.where(q < 0.5, 1 - 6 * q**2 + 6 * q**3, 2 * np.power(1 - q, 3))
        w = np.where(q > 1, 0.0, w)
        return w * (8 / np.pi)
    if ktype == KT_QUARTIC_SPLINE:
        w = np.zeros(np.shape(q))
        m1 = q < 0.2
        m2 = (q >= 0.2) & (q < 0.6)
        m3 = (q >= 0.6) & (q < 1)
        w = np.where(m1, (1 - q) ** 4 - 5 * (0.6 - q) ** 4 + 10 * (0.2 - q) ** 4, w)
        w = np.where(m2, (1 - q) ** 4 - 5 * (0.6 - q) ** 4, w)
        w = np.where(m3, (1 - q) ** 4, w)
        return w * (15625 / 512 / np.pi)
    if ktype == KT_GAUSSIAN:
        sig = GAUSS_SIG
        norm = gaussian_norm(truncate)
        return (
            np.where(
                q < truncate * sig,
                np.power(sig * np.sqrt(2 * np.pi), -3) * np.exp(-np.power(q / sig, 2) / 2),
                0,
            )
            / norm
        )
    raise ValueError(f"no profile for kernel type {ktype}")


def gaussian_norm(truncate: float) -> float:
    """Normalisation of the truncated Gaussian, sph_kernels.py:949-951."""
    return float(
        erf(truncate / np.sqrt(2))
        - 2 * truncate / np.sqrt(2 * np.pi) * np.exp(-np.power(truncate, 2) / 2)
    )


def find_fwhm(f) -> float:
    """FWHM of a peaked kernel by root finding, sph_kernels.py:14-48."""
    return 2 * fsolve(lambda q: f(q) - f(np.zeros(1)) / 2, 0.5)[0]


def kernel_constants(ktype: int, truncate: float = 3.0) -> dict:
    """size_in_fwhm, _rescale and validity limit of a simple kernel.

    Closed-form kernels rescale so that FWHM = 1 (sph_kernels.py:366-371,
    :507-511, :750-755, :1430-1435); the Gaussian keeps rescale 1 and sets
    size_in_fwhm = truncate / 2.3548 with a truncation-dependent minimum size
    (sph_kernels.py:931-954); DiracDelta has size_in_fwhm = 1 and a maximum
    size 0.5 px (sph_kernels.py:1104-1112).
    """
    if ktype == KT_DIRAC:
        return dict(ktype=ktype, truncate=0.0, size_in_fwhm=1.0, rescale=1.0,
                    min_valid=None, max_valid=0.5)
    if ktype == KT_GAUSSIAN:
        if truncate < 2:
            raise RuntimeError(
                "GaussianKernel with truncation <2sigma will cause large errors in total mass."
            )
        if truncate < 3:
            mv = 3.7
        elif truncate < 4:
            mv = 2.3357
        elif truncate < 5:
            mv = 1.1288
        elif truncate < 6:
            mv = 0.45
        else:
            mv = 0.336
        return dict(ktype=ktype, truncate=float(truncate),
                    size_in_fwhm=truncate / (2 * np.sqrt(2 * np.log(2))), rescale=1.0,
                    min_valid=mv, max_valid=None)
    min_valid = {KT_WENDLAND_C2: 1.51, KT_WENDLAND_C6: 1.29, KT_CUBIC_SPLINE: 1.16,
                 KT_QUARTIC_SPLINE: 1.2385}[ktype]
    # eval_kernel(r, 1) with rescale 1: W(q) / 1**3 (sph_kernels.py:192-219)
    fwhm = find_fwhm(lambda r: kernel_profile(ktype, r))
    return dict(ktype=ktype, truncate=0.0, size_in_fwhm=1 / fwhm, rescale=1.0 / fwhm,
                min_valid=min_valid, max_valid=None)


# Public adaptive kernel tuples, sph_kernels.py:1629-1635, :1689-1695,
# :1752-1758, :1824-1834, :1897-1903.
def adaptive_tuple(name: str, truncate: float = 3.0) -> list[dict]:
    primary = {
        "WendlandC2Kernel": (KT_WENDLAND_C2, 0.0),
        "WendlandC6Kernel": (KT_WENDLAND_C6, 0.0),
        "CubicSplineKernel": (KT_CUBIC_SPLINE, 0.0),
        "QuarticSplineKernel": (KT_QUARTIC_SPLINE, 0.0),
        "GaussianKernel": (KT_GAUSSIAN, truncate),
    }[name]
    return [
        kernel_constants(primary[0], primary[1] if primary[0] == KT_GAUSSIAN else 3.0),
        kernel_constants(KT_DIRAC),
        kernel_constants(KT_GAUSSIAN, 6.0),
    ]


def simple_tuple(ktype: int, truncate: float = 3.0) -> list[dict]:
    return [kernel_constants(ktype, truncate)]


def validate(kc: dict, h: np.ndarray) -> np.ndarray:
    """Validity of the kernel approximation, sph_kernels.py:443-478 (min size),
    :1167-1204 (DiracDelta max size)."""
    if kc["max_valid"] is not None:
        return h <= kc["max_valid"]
    return h >= kc["min_valid"]


def select_kernels(kernels: list[dict], h_px: np.ndarray):
    """Per-particle kernel choice, sph_kernels.py:1241-1274.

    Returns (kernel_indices, size_in_fwhm, rescale); index -1 (no valid
    kernel) takes kernels[0]'s size and rescale.  A single simple kernel
    returns index 0 everywhere (no adaptive selection, sph_kernels.py:85-119).
    """
    n = h_px.shape[0]
    if len(kernels) == 1:
        k = kernels[0]
        return (np.zeros(n, dtype=np.int64), np.full(n, k["size_in_fwhm"]),
                np.full(n, k["rescale"]))
    idx = -np.ones(n, dtype=np.int64)
    for ik, k in enumerate(kernels):
        idx[(idx == -1) & validate(k, h_px * k["rescale"])] = ik
    sizes = np.array([k["size_in_fwhm"] for k in kernels])
    rescales = np.array([k["rescale"] for k in kernels])
    size = sizes[idx]
    size[idx == -1] = sizes[0]
    resc = rescales[idx]
    resc[idx == -1] = rescales[0]
    return idx, size, resc


def sm_ranges(h_px: np.ndarray, size_in_fwhm) -> np.ndarray:
    """Footprint half-width in pixels, sph_kernels.py:257-262."""
    return np.ceil(h_px * size_in_fwhm)


# ---- pixel integrals (dij = particle - pixel, in px; h = rescaled length) --


def ki_wendland_c2(dij, h):
    """sph_kernels.py:400-441."""
    dr2 = np.power(dij, 2).sum(axis=0)
    out = np.zeros(h.shape)
    R2 = dr2 / (h * h)
    out[R2 == 0] = 2.0 / 3.0
    use = (R2 < 1) & (R2 != 0)
    r2 = R2[use]
    A = np.sqrt(1 - r2)
    out[use] = 5 * r2 * r2 * (0.5 * r2 + 3) * np.log((1 + A) / np.sqrt(r2)) + A * (
        -27.0 / 2.0 * r2 * r2 - 14.0 / 3.0 * r2 + 2.0 / 3.0
    )
    return out * (21 / 2 / np.pi) / np.power(h, 2)


def _c6_indef(R, z):
    """Antiderivative of the C6 kernel along the line of sight, with the
    reference's rounded coefficients (sph_kernels.py:575-674)."""
    q = np.sqrt(R**2 + z**2)
    L = np.log(q + z)
    return (
        -231 * R**10 * z - 385 * R**8 * z**3 - 1155 * R**8 * z - 462 * R**6 * z**5
        - 1540 * R**6 * z**3 - 462 * R**6 * z - 330 * R**4 * z**7 - 1386 * R**4 * z**5
        - 462 * R**4 * z**3 + 66 * R**4 * z - (128 + 1 / 3) * R**2 * z**9
        - 660 * R**2 * z**7 - 277.2 * R**2 * z**5 + 44 * R**2 * z**3
        + 8 / 3 * z**11 * q + (16 + 4 / 15) * R**2 * z**9 * q + 70.4 * z**9 * q
        + 360.8 * R**2 * z**7 * q + 132 * z**7 * q + 550 * R**2 * z**5 * q - 11 * R**2 * z
        + 7.21875 * R**12 * L + 24.7813 * R**10 * z * q + 173.25 * R**10 * L
        + 530.75 * R**8 * z * q + 288.75 * R**8 * L + 47.4792 * R**8 * z**3 * q
        + 767.25 * R**6 * z * q + 58.0167 * R**6 * z**5 * q + 819.5 * R**6 * z**3 * q
        + 41.7 * R**4 * z**7 * q + 752.4 * R**4 * z**5 * q + 896.5 * R**4 * z**3 * q
        - 21 * z**11 - (128 + 1 / 3) * z**9 - 66 * z**7 + 13.2 * z**5 - 11 / 3 * z**3 + z
    )


def ki_wendland_c6(dij, h):
    """sph_kernels.py:544-685."""
    dr2 = np.power(dij, 2).sum(axis=0)
    out = np.zeros(h.shape)
    R = np.sqrt(dr2) / h
    use = (R < 1) & (R != 0)
    norm = 1365 / 64 / np.pi
    zmax = np.sqrt(1 - R[use] ** 2)
    out[use] = norm * 2 * (_c6_indef(R[use], zmax) - _c6_indef(R[use], 0.0))
    out[R == 0] = norm * 2 * (4 / 15)
    return out / np.power(h, 2)


def ki_cubic_spline(dij, h):
    """sph_kernels.py:791-858 (dij is scaled by 2 on a copy)."""
    d = dij * 2
    dr2 = np.power(d, 2).sum(axis=0)
    out = np.zeros(h.shape)
    R2 = dr2 / (h * h)
    out[R2 == 0] = 11.0 / 16.0 + 0.25 * 0.25
    c1 = (R2 > 0) & (R2 <= 1)
    c2 = (R2 > 1) & (R2 <= 4)
    r1 = R2[c1]
    r2 = R2[c2]
    A1 = np.sqrt(1 - r1)
    B1 = np.sqrt(4 - r1)
    B2 = np.sqrt(4 - r2)
    I1 = (A1 - 0.5 * A1**3 - 1.5 * r1 * A1 + 3.0 / 32.0 * A1 * (3 * r1 + 2)
          + 9.0 / 32.0 * r1 * r1 * (np.log(1 + A1) - np.log(np.sqrt(r1))))
    I2 = (-B2 * (3 * r2 + 56) / 4.0
          - 3.0 / 8.0 * r2 * (r2 + 16) * np.log((2 + B2) / np.sqrt(r2))
          + 2 * (3 * r2 + 4) * B2 + 2 * B2**3)
    I3 = (-B1 * (3 * r1 + 56) / 4.0 + A1 * (4 * r1 + 50) / 8.0
          - 3.0 / 8.0 * r1 * (r1 + 16) * np.log((2 + B1) / (1 + A1))
          + 2 * (3 * r1 + 4) * (B1 - A1) + 2 * (B1**3 - A1**3))
    out[c1] = I1 + 0.25 * I3
    out[c2] = 0.25 * I2
    return out / 1.59689476201133 / np.power(h, 2) * 4


def _quartic_IA(R, z, A):
    """sph_kernels.py:1516-1547."""
    q = np.sqrt(z**2 + R**2)
    R2 = R**2
    return (A**4 * z - 2 * A**3 * z * q + 2 * A**2 * z * (3 * R2 + z**2)
            - A * R2 * (4 * A**2 + 3 * R2) * np.arcsinh(z / R) / 2
            - A * z * q * (5 * R2 + 2 * z**2) / 2 + R2 * R2 * z + 2 * R2 * z**3 / 3
            + z**5 / 5)


def ki_quartic_spline(dij, h):
    """sph_kernels.py:1486-1564."""
    dr = np.sqrt(np.power(dij, 2).sum(axis=0))
    out = np.zeros(h.shape)
    R = dr / h
    m1 = (R > 0) & (R < 0.2)
    out[m1] += 10 * _quartic_IA(R[m1], np.sqrt(0.2**2 - R[m1] ** 2), 0.2)
    m2 = (R > 0) & (R < 0.6)
    out[m2] -= 5 * _quartic_IA(R[m2], np.sqrt(0.6**2 - R[m2] ** 2), 0.6)
    m3 = (R > 0) & (R < 1.0)
    out[m3] += _quartic_IA(R[m3], np.sqrt(1 - R[m3] ** 2), 1.0)
    out[R == 0] = 384 / 3125
    out *= 2 * 15625 / 512 / np.pi
    return out / np.power(h, 2)


def ki_gaussian(dij, h, truncate):
    """sph_kernels.py:994-1044."""
    sig = GAUSS_SIG
    dr = np.sqrt(np.power(dij, 2).sum(axis=0))
    with np.errstate(invalid="ignore"):
        zmax = np.sqrt(truncate**2 - np.power(dr / h / sig, 2))
    zmax = np.where(truncate > dr / h / sig, zmax, 0)
    x0 = (dij[0] - 0.5) / h / np.sqrt(2) / sig
    x1 = (dij[0] + 0.5) / h / np.sqrt(2) / sig
    y0 = (dij[1] - 0.5) / h / np.sqrt(2) / sig
    y1 = (dij[1] + 0.5) / h / np.sqrt(2) / sig
    out = 0.25 * erf(zmax / np.sqrt(2)) * (erf(x1) - erf(x0)) * (erf(y1) - erf(y0))
    out[(dr - np.sqrt(0.5)) / h / sig > truncate] = 0
    return out / gaussian_norm(truncate)


def ki_dirac(dij, h):
    """sph_kernels.py:1136-1165: 1 px^-2 iff |dx| < 0.5 and |dy| < 0.5."""
    return np.where((np.abs(dij) < 0.5).all(axis=0), 1.0, 0.0)


def kernel_integral(kc: dict, dij: np.ndarray, h: np.ndarray) -> np.ndarray:
    t = kc["ktype"]
    if t == KT_WENDLAND_C2:
        return ki_wendland_c2(dij, h)
    if t == KT_WENDLAND_C6:
        return ki_wendland_c6(dij, h)
    if t == KT_CUBIC_SPLINE:
        return ki_cubic_spline(dij, h)
    if t == KT_QUARTIC_SPLINE:
        return ki_quartic_spline(dij, h)
    if t == KT_GAUSSIAN:
        return ki_gaussian(dij, h, kc["truncate"])
    if t == KT_DIRAC:
        return ki_dirac(dij, h)
    raise ValueError(t)


def px_weight(kernels: list[dict], kidx: np.ndarray, dij: np.ndarray,
              h_eff: np.ndarray) -> np.ndarray:
    """_px_weight + adaptive dispatch, sph_kernels.py:85-119, :1330-1363.

    ``h_eff`` is sm_lengths * rescale; index -1 uses kernels[0].
    """
    out = np.zeros(h_eff.shape)
    for ik in np.unique(kidx):
        kc = kernels[0] if ik == -1 else kernels[ik]
        m = kidx == ik
        out[m] = kernel_integral(kc, dij[:, m], h_eff[m])
    return out


# ---------------------------------------------------------------------------
# Channels and spectra (martini/datacube.py, martini/spectral_models.py)
# ---------------------------------------------------------------------------


def vrad_channel_edges(n_channels: int, channel_width_kms: float, centre_kms: float):
    """Velocity channel edges of a VRAD cube in km/s.

    WCS axis 3: crpix = Nc/2 + 0.5, cdelt = -|dv|, crval = centre
    (datacube.py:457-475); edges at pixel arange(Nc+1) - 0.5, origin 0
    (datacube.py:513-536).  Edges therefore decrease with channel index.
    """
    crpix = n_channels / 2.0 + 0.5
    k = np.arange(n_channels + 1) - 0.5
    return centre_kms + (-abs(channel_width_kms)) * (k + 1 - crpix)


def freq_channel_edges(n_channels: int, channel_width_hz: float, centre_hz: float):
    """Velocity (radio convention) edges of a FREQ cube in km/s.

    FREQ axis has cdelt = +|df| (datacube.py:468-475); converted with the
    radio Doppler convention v = c (1 - f / f0) (datacube.py:539-562).
    """
    crpix = n_channels / 2.0 + 0.5
    k = np.arange(n_channels + 1) - 0.5
    f = centre_hz + abs(channel_width_hz) * (k + 1 - crpix)
    return C_KMS * (1.0 - f / HI_FREQ_HZ)


def thermal_sigma_kms(T_K: np.ndarray) -> np.ndarray:
    """sqrt(k_B T / m_p) in km/s, spectral_models.py:465-485."""
    return np.sqrt(K_B * np.asarray(T_K, dtype=np.float64) / M_P) / 1e3


def gaussian_phi(a, b, v, sigma):
    """spectral_models.py:386-425: 0.5 [erf((b-v)/(sqrt2 s)) - erf((a-v)/(sqrt2 s))]."""
    tb = erf((b - v) / np.sqrt(2.0) / sigma)
    ta = erf((a - v) / np.sqrt(2.0) / sigma)
    return 0.5 * (tb - ta)


def dirac_phi(a, b, v):
    """spectral_models.py:544-570: H(v - a) H(b - v) with H(0) = 1."""
    return np.heaviside(v - a, 1.0) * np.heaviside(b - v, 1.0)


def channel_bounds(edges: np.ndarray):
    """Lower/upper edge per channel, spectral_models.py:180-187."""
    d = np.diff(edges)
    if np.all(d > 0):
        return edges[:-1], edges[1:]
    if np.all(d < 0):
        return edges[1:], edges[:-1]
    raise ValueError("Channel edges are not monotonic sequence.")


def init_spectra(model: str, mHI_Msun, distance_Mpc, v_kms, edges_kms, sigma_kms=None):
    """Per-particle channel spectra in Jy, spectral_models.py:63-200.

    S_p(c) = mHI_p / D_p^2 * phi_p(c) / |dv_c| / 2.36e5.
    """
    lo, hi = channel_bounds(edges_kms)
    v = np.asarray(v_kms, dtype=np.float64)[:, None]
    if model == "gaussian":
        s = np.asarray(sigma_kms, dtype=np.float64)
        s = s[:, None] if s.ndim == 1 else s
        phi = gaussian_phi(lo[None, :], hi[None, :], v, s)
    elif model == "dirac":
        phi = dirac_phi(lo[None, :], hi[None, :], v)
    else:
        raise ValueError(model)
    A = np.asarray(mHI_Msun, dtype=np.float64) * np.power(np.asarray(distance_Mpc, dtype=np.float64), -2)
    A = np.broadcast_to(A, v.shape[:1])
    widths = np.abs(np.diff(edges_kms))
    spectra = A[:, None] * phi
    spectra = spectra / widths
    return spectra / MHI_TO_JY


# ---------------------------------------------------------------------------
# Pruning and insertion (martini/martini.py)
# ---------------------------------------------------------------------------


def prune_mask(x, y, vchan, ranges, mHI, nx_pad, ny_pad, n_channels, half_width_kms,
               edges_kms, spatial=True, spectral=True, mass=True):
    """Accept mask of martini/martini.py:168-241."""
    hw = np.asarray(half_width_kms) / np.max(np.abs(np.diff(edges_kms)))
    rej = np.zeros(x.shape, dtype=bool)
    if spatial:
        rej |= (x + ranges < 0) | (y + ranges < 0)
        rej |= x - ranges > nx_pad
        rej |= y - ranges > ny_pad
        rej |= np.isnan(x) | np.isnan(y)
    if spectral:
        rej |= vchan + 4 * hw < 0
        rej |= vchan - 4 * hw > n_channels
    if mass:
        rej |= np.asarray(mHI) == 0
    return ~rej


def evaluate_pixel_spectrum(i, j, x, y, ranges, kernels, kidx, h_eff, spectra):
    """One pixel's spectrum in Jy/pix^2, martini/martini.py:243-283."""
    mask = (np.abs(i - x) <= ranges) & (np.abs(j - y) <= ranges)
    dij = np.vstack((x[mask] - i, y[mask] - j))
    w = px_weight(kernels, kidx[mask], dij, h_eff[mask])
    return (spectra[mask] * w[:, None]).sum(axis=0)


def insert_perpixel(nx, ny, x, y, ranges, kernels, kidx, h_eff, spectra, ncpu=1,
                    pixels=None):
    """The reference's per-pixel loop (martini/martini.py:327-362).

    Returns the (nx, ny, Nc) cube in Jy/pix^2, or, when ``pixels`` (a list of
    (i, j)) is given, the (len(pixels), Nc) spectra of just those pixels.
    ``ncpu > 1`` spreads pixels over a thread pool as the reference does
    (numpy releases the GIL inside its kernels).
    """
    ij = pixels if pixels is not None else [(i, j) for i in range(nx) for j in range(ny)]

    def f(p):
        return evaluate_pixel_spectrum(p[0], p[1], x, y, ranges, kernels, kidx, h_eff, spectra)

    if ncpu == 1:
        rows = [f(p) for p in ij]
    else:
        with ThreadPoolExecutor(max_workers=ncpu) as ex:
            rows = list(ex.map(f, ij, chunksize=max(1, len(ij) // (8 * ncpu))))
    out = np.array(rows).reshape(len(ij), spectra.shape[1])
    if pixels is not None:
        return out
    return out.reshape(nx, ny, spectra.shape[1])


def footprint_bounds(c, r, n):
    """Integer pixel range [lo, hi] with |i - c| <= r, clipped to [0, n-1].

    The Chebyshev-box mask of martini/martini.py:272-274 evaluated on an
    integer range: candidates from floor/ceil, then the exact FP64 predicate
    decides the ends.
    """
    lo = math.floor(c - r) - 1
    hi = math.ceil(c + r) + 1
    lo = max(lo, 0)
    hi = min(hi, n - 1)
    while lo <= hi and not (abs(lo - c) <= r):
        lo += 1
    while hi >= lo and not (abs(hi - c) <= r):
        hi -= 1
    return lo, hi


def insert_scatter(nx, ny, x, y, ranges, kernels, kidx, h_eff, spectra):
    """Same arithmetic as ``insert_perpixel``, accumulated per particle."""
    nc = spectra.shape[1]
    cube = np.zeros((nx, ny, nc))
    for p in range(x.shape[0]):
        if not (np.isfinite(x[p]) and np.isfinite(y[p])):
            continue
        ilo, ihi = footprint_bounds(x[p], ranges[p], nx)
        jlo, jhi = footprint_bounds(y[p], ranges[p], ny)
        if ilo > ihi or jlo > jhi:
            continue
        ii, jj = np.meshgrid(np.arange(ilo, ihi + 1), np.arange(jlo, jhi + 1), indexing="ij")
        dij = np.vstack(((x[p] - ii).ravel(), (y[p] - jj).ravel()))
        w = px_weight(kernels, np.full(dij.shape[1], kidx[p]), dij,
                      np.full(dij.shape[1], h_eff[p]))
        cube[ilo:ihi + 1, jlo:jhi + 1, :] += (w.reshape(ii.shape)[:, :, None]
                                              * spectra[p][None, None, :])
    return cube


def to_jy_per_arcsec2(cube_jy_per_pix2, px_size_arcsec):
    """Unit conversion of martini/martini.py:364-366 (datacube.py:189-194)."""
    return cube_jy_per_pix2 / px_size_arcsec**2


def flux_and_mass(cube_jy_per_pix2, padx, pady, edges_kms, distance_Mpc):
    """Inserted flux (Jy) and HI mass (Msun), martini/martini.py:367-392."""
    nx, ny = cube_jy_per_pix2.shape[:2]
    sl = (slice(padx, nx - padx), slice(pady, ny - pady))
    c = cube_jy_per_pix2[sl]
    flux = float(c.sum())
    per_chan = c.sum(axis=(0, 1))
    mass = MHI_TO_JY * distance_Mpc**2 * float(np.sum(per_chan * np.abs(np.diff(edges_kms))))
    return flux, mass


# ---------------------------------------------------------------------------
# Particle projection (martini/sources/sph_source.py:265-362)
# ---------------------------------------------------------------------------


def project_particles(xyz_kpc, vxyz_kms, distance_Mpc, ra_deg=0.0, dec_deg=0.0,
                      h=0.7, vpeculiar_kms=0.0):
    """Sky position and line-of-sight velocity of each particle.

    Rotation R_y(dec) R_z(-ra) applied to row vectors, translation to the
    source distance along the (ra, dec) direction, peculiar velocity along
    it and Hubble flow h*100*r per particle (sph_source.py:265-317; the
    expected transform is spelled out in tests/test_sources.py:255-316).
    Returns (ra_deg, dec_deg, vlos_kms, dist_Mpc).
    """
    ra = np.deg2rad(ra_deg)
    dec = np.deg2rad(dec_deg)
    Ry = np.array([[np.cos(dec), 0, np.sin(dec)], [0, 1, 0], [-np.sin(dec), 0, np.cos(dec)]])
    Rz = np.array([[np.cos(-ra), -np.sin(-ra), 0], [np.sin(-ra), np.cos(-ra), 0], [0, 0, 1]])
    rot = Ry.dot(Rz)
    u = np.array([np.cos(dec) * np.cos(ra), np.cos(dec) * np.sin(ra), np.sin(dec)])
    pos = np.asarray(xyz_kpc, dtype=np.float64).dot(rot) + u[None, :] * distance_Mpc * 1e3
    vel = (np.asarray(vxyz_kms, dtype=np.float64).dot(rot)
           + h * 100.0 * pos * 1e-3 + u[None, :] * vpeculiar_kms)
    d = np.sqrt((pos**2).sum(axis=1))
    vlos = (pos * vel).sum(axis=1) / d
    ra_p = np.rad2deg(np.arctan2(pos[:, 1], pos[:, 0])) % 360.0
    dec_p = np.rad2deg(np.arcsin(pos[:, 2] / d))
    return ra_p, dec_p, vlos, d * 1e-3


def tan_world2pix(ra_deg, dec_deg, crval_ra, crval_dec, crpix1, crpix2, cdelt1, cdelt2):
    """Gnomonic (TAN) projection to 0-based pixel coordinates.

    Restates the FITS WCS TAN convention (Calabretta & Greisen 2002) used by
    ``datacube.wcs`` (datacube.py:438-486) through ``wcs_world2pix``
    (sph_source.py:346-361).  Points on or behind the tangent plane's horizon
    give NaN, as wcslib flags them invalid.
    """
    a = np.deg2rad(ra_deg)
    d = np.deg2rad(dec_deg)
    a0 = np.deg2rad(crval_ra)
    d0 = np.deg2rad(crval_dec)
    cosc = np.sin(d) * np.sin(d0) + np.cos(d) * np.cos(d0) * np.cos(a - a0)
    with np.errstate(divide="ignore", invalid="ignore"):
        xi = np.rad2deg(np.cos(d) * np.sin(a - a0) / cosc)
        eta = np.rad2deg((np.sin(d) * np.cos(d0) - np.cos(d) * np.sin(d0) * np.cos(a - a0)) / cosc)
    px = crpix1 - 1 + xi / cdelt1
    py = crpix2 - 1 + eta / cdelt2
    bad = ~(cosc > 0)
    px = np.where(bad, np.nan, px)
    py = np.where(bad, np.nan, py)
    return px, py


def sm_lengths_px(hsm_kpc, dist_Mpc, px_size_arcsec):
    """arctan(hsm / D_particle) in pixels, sph_kernels.py:235-255."""
    ang = np.arctan(np.asarray(hsm_kpc) / (np.asarray(dist_Mpc) * 1e3))
    return np.rad2deg(ang) * 3600.0 / px_size_arcsec


# ---------------------------------------------------------------------------
# Seeded synthetic discs (the configurations' generator)
# ---------------------------------------------------------------------------


def disc_particles(n, seed, R_d=3.0, z_d=0.3, v_flat=200.0, v_disp=10.0,
                   mHI_med=1e5, mHI_dex=0.2, h_med=1.0, h_dex=0.3, T_med=1e4, T_dex=0.3,
                   h_loguniform=None):
    """Exponential disc: R ~ Gamma(2, R_d), z ~ N(0, z_d), circular speed
    v_flat * arctan(R / 1 kpc) / (pi / 2) plus isotropic N(0, v_disp);
    lognormal HI masses, smoothing lengths and temperatures.  One RNG, fixed
    draw order (phi, R, z, dispersion, mass, h, T).  The disc lies in the
    x-y plane with x along the line of sight before inclination.
    """
    rng = np.random.default_rng(seed)
    phi = rng.uniform(0, 2 * np.pi, n)
    R = rng.gamma(2.0, R_d, n)
    z = rng.normal(0.0, z_d, n)
    disp = rng.normal(0.0, v_disp, (n, 3))
    mHI = mHI_med * 10 ** (mHI_dex * rng.normal(0, 1, n))
    if h_loguniform is None:
        hsm = h_med * 10 ** (h_dex * rng.normal(0, 1, n))
    else:
        lo, hi = h_loguniform
        hsm = 10 ** rng.uniform(np.log10(lo), np.log10(hi), n)
    T = T_med * 10 ** (T_dex * rng.normal(0, 1, n))
    vphi = v_flat * np.arctan(R / 1.0) / (np.pi / 2)
    xyz = np.stack((R * np.cos(phi), R * np.sin(phi), z), axis=1)
    vxyz = np.stack((-vphi * np.sin(phi), vphi * np.cos(phi), np.zeros(n)), axis=1) + disp
    return dict(xyz=xyz, vxyz=vxyz, mHI=mHI, hsm=hsm, T=T, rng=rng)


def incline(xyz, vxyz, incl_deg):
    """Rotate a face-on (x-y plane) disc so its normal tilts by incl from the
    line of sight (x axis): rotation about y.  incl = 0 is face-on."""
    # face-on in the sky plane y-z means the disc normal is along x; the
    # generator's disc normal is z, so first map z -> x, then tilt about y.
    M0 = np.array([[0, 0, 1], [1, 0, 0], [0, 1, 0]], dtype=np.float64)  # (x,y,z)->(y,z,x)
    i = np.deg2rad(incl_deg)
    Ry = np.array([[np.cos(i), 0, np.sin(i)], [0, 1, 0], [-np.sin(i), 0, np.cos(i)]])
    M = Ry @ M0
    return xyz @ M.T, vxyz @ M.T


# ---------------------------------------------------------------------------
# Total flux per particle in C (FP64), for full-size parity
# ---------------------------------------------------------------------------

_CLIB = None


def _clib():
    """The oracle's C restatement (oracle/flux_total.c), built on first use."""
    global _CLIB
    if _CLIB is None:
        import ctypes as C
        from oracle import build as ob
        lib = C.CDLL(ob.build())
        dp = C.POINTER(C.c_double)
        lib.mgo_flux_total.restype = C.c_double
        lib.mgo_flux_total.argtypes = [C.c_int64, dp, dp, dp, dp, C.c_void_p, C.c_int,
                                       C.POINTER(C.c_int), dp, dp, C.c_int, C.c_int, C.c_int,
                                       C.c_int, C.c_int, C.c_void_p]
        lib.mgo_spectrum_sums.restype = None
        lib.mgo_spectrum_sums.argtypes = [C.c_int64, dp, C.c_void_p, C.c_double, dp, C.c_int,
                                          C.c_int, dp, C.c_int, dp]
        _CLIB = lib
    return _CLIB


def _f64(a):
    import ctypes as C
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(C.POINTER(C.c_double))


def spectrum_sums(model: str, v_kms, sigma_kms, amp, edges_kms, threads=None):
    """sum_c S_p(c) per particle in Jy, S_p(c) = amp_p phi_p(c) / |dv_c|
    (spectral_models.py:63-200; Gaussian :386-425, Dirac :544-570), in
    FP64 C.  ``sigma_kms`` is an array or a scalar (Gaussian only)."""
    import ctypes as C
    lib = _clib()
    v, vp = _f64(v_kms)
    a, ap = _f64(np.broadcast_to(amp, v.shape))
    e, ep = _f64(edges_kms)
    out = np.empty(v.shape[0])
    sig_arr, sig_ptr, sig_c = None, None, 0.0
    if model == "gaussian":
        if np.ndim(sigma_kms) == 0:
            sig_c = float(sigma_kms)
        else:
            sig_arr, _ = _f64(sigma_kms)
            sig_ptr = sig_arr.ctypes.data_as(C.c_void_p)
    lib.mgo_spectrum_sums(v.shape[0], vp, sig_ptr, sig_c, ap, 1 if model == "dirac" else 0,
                          e.shape[0] - 1, ep, threads or os.cpu_count() or 1,
                          out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def flux_total(x, y, ranges, kernels, kidx, h_eff, ssum, nx, ny, padx=0, pady=0,
               threads=None, return_wsum=False):
    """Total flux over the unpadded cube, sum_p (sum_box W_p) (sum_c S_p(c)),
    in FP64 C: the reference's per-pixel sums (martini/martini.py:243-283)
    added over the unpadded pixels (:367-375), reordered per particle.
    ``ssum`` comes from :func:`spectrum_sums`."""
    import ctypes as C
    lib = _clib()
    xs, xp = _f64(x)
    ys, yp = _f64(y)
    rs, rp = _f64(ranges)
    hs, hp = _f64(h_eff)
    ss, sp = _f64(ssum)
    n = xs.shape[0]
    ki = None if kidx is None else np.ascontiguousarray(kidx, dtype=np.int8)
    kt = (C.c_int * 4)(*[int(k["ktype"]) for k in kernels] + [0] * (4 - len(kernels)))
    tr = np.array([float(k.get("truncate", 3.0)) for k in kernels] + [3.0] * (4 - len(kernels)))
    wsum = np.empty(n) if return_wsum else None
    tot = lib.mgo_flux_total(n, xp, yp, rp, hp,
                             None if ki is None else ki.ctypes.data_as(C.c_void_p),
                             len(kernels), kt, tr.ctypes.data_as(C.POINTER(C.c_double)), sp,
                             int(nx), int(ny), int(padx), int(pady),
                             threads or os.cpu_count() or 1,
                             None if wsum is None else wsum.ctypes.data_as(C.c_void_p))
    return (tot, wsum) if return_wsum else tot


def pixel_spectra(pixels, x, y, ranges, kernels, kidx, h_eff, model, mHI, dist, v, edges,
                  sigma=None, threads=8):
    """The reference's per-pixel sum (``_evaluate_pixel_spectrum``,
    martini/martini.py:243-283) at each (i, j) of ``pixels``, FP64: the
    Chebyshev-box mask over all particles, the kernel weights of the masked
    ones (sph_kernels.py:85-119) and their spectra (spectral_models.py:63-200).
    Returns an array [len(pixels), nc] in Jy / pix^2."""
    nc = len(edges) - 1
    kidx = np.zeros(x.shape[0], np.int64) if kidx is None else np.asarray(kidx, np.int64)
    h_eff = np.asarray(h_eff, np.float64)

    def one(ij):
        i, j = ij
        m = (np.abs(x - i) <= ranges) & (np.abs(y - j) <= ranges)
        if not m.any():
            return np.zeros(nc)
        dij = np.vstack((x[m] - i, y[m] - j))
        wt = px_weight(kernels, kidx[m], dij, h_eff[m])
        sig = None
        if model == "gaussian":
            sig = np.broadcast_to(np.asarray(sigma, np.float64), x.shape)[m]
        sp = init_spectra(model, mHI[m], dist[m], v[m], edges, sig)
        return wt @ sp

    with ThreadPoolExecutor(threads) as ex:
        return np.stack(list(ex.map(one, pixels)))
