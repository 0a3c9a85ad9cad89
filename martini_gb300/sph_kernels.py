"""SPH kernels: the reference's classes, constants, validation and adaptive
selection; the pixel integrals themselves run on the GPU.

Mirrors martini/sph_kernels.py: ``_WendlandC2Kernel`` (:340-478),
``_WendlandC6Kernel`` (:481-721), ``_CubicSplineKernel`` (:724-894),
``_GaussianKernel`` (:897-1080), ``DiracDeltaKernel`` (:1083-1204),
``_QuarticSplineKernel`` (:1402-1600), ``_AdaptiveKernel`` (:1207-1399) and
the public adaptive kernels (:1603-1959).  Each kernel's ``size_in_fwhm``
and ``_rescale`` come from the same FWHM root find (sph_kernels.py:14-48).
"""

from __future__ import annotations

import numpy as np
from scipy.optimize import fsolve
from scipy.special import erf

from . import _native as N


def find_fwhm(f) -> float:
    """Twice the root of f(q) - f(0)/2 from q = 0.5 (sph_kernels.py:14-48)."""
    return 2 * fsolve(lambda q: f(q) - f(np.zeros(1)) / 2, 0.5)[0]


class _BaseSPHKernel:
    """Common state: sm_lengths (px), sm_ranges, rescale, validation."""

    size_in_fwhm = None
    native_type = None

    def __init__(self):
        self._rescale = 1.0
        self.sm_lengths = None
        self.sm_ranges = None

    # ---- kernel profile (for constants and users) --------------------------
    def kernel(self, q):
        raise NotImplementedError

    def eval_kernel(self, r, h):
        """Kernel value at r for FWHM h (sph_kernels.py:192-219)."""
        q = np.array(np.asarray(r, dtype=np.float64) / np.asarray(h, dtype=np.float64)
                     / self._rescale)
        scalar_input = q.ndim == 0
        W = self.kernel(q)
        W = W / np.power(np.asarray(h, dtype=np.float64) * self._rescale, 3)
        return W.item() if scalar_input else W

    # ---- set-up (sph_kernels.py:221-262) -------------------------------------
    def _init_sm_lengths(self, source, datacube):
        """Angular smoothing length in pixels: arctan(hsm / D_particle)."""
        if source.skycoords is None:
            raise RuntimeError("Initialize source skycoords before initializing smoothing lengths.")
        ang = np.arctan(source.hsm_g / (source.skycoords.distance * 1e3))
        self.sm_lengths = np.rad2deg(ang) * 3600.0 / datacube.px_size

    def _init_sm_ranges(self):
        self.sm_ranges = np.ceil(self.sm_lengths * self.size_in_fwhm)

    def _apply_mask(self, mask):
        self.sm_lengths = self.sm_lengths[mask]
        self.sm_ranges = self.sm_ranges[mask]

    def _validate_error(self, msg, sm_lengths, valid, noraise=False, quiet=False):
        if not quiet:
            print(f"    ---------{self.__class__.__name__} VALIDATION---------")
            print("    Median smoothing length: ", np.median(sm_lengths), "px")
            print("    Minimum smoothing length: ", np.min(sm_lengths), "px")
            print("    Maximum smoothing length: ", np.max(sm_lengths), "px")
            print("    ", np.sum(np.logical_not(valid)), "/", np.size(sm_lengths),
                  "smoothing lengths fail validation.")
        if not noraise:
            raise RuntimeError(msg)

    def _confirm_validation(self, noraise=False, quiet=False):
        return self._validate(self.sm_lengths, noraise=noraise, quiet=quiet)

    def _validate(self, sm_lengths, noraise=False, quiet=False):
        raise NotImplementedError

    # ---- device description ----------------------------------------------------
    def _device_kernels(self):
        """[(MG_KERNEL_*, truncate)] of the kernel table."""
        return [(self.native_type, 0.0)]

    def _device_arrays(self):
        """(h_eff = sm_lengths * rescale, kernel_index or None) per particle."""
        return self.sm_lengths * self._rescale, None


class _MinSizeKernel(_BaseSPHKernel):
    min_valid_size = None
    _label = ""

    def __init__(self):
        super().__init__()
        fwhm = find_fwhm(lambda r: self.eval_kernel(r, 1))
        self.size_in_fwhm = 1 / fwhm
        self._rescale /= fwhm

    def _validate(self, sm_lengths, noraise=False, quiet=False):
        valid = np.asarray(sm_lengths) >= self.min_valid_size
        if np.logical_not(valid).any():
            self._validate_error(
                f"martini.sph_kernels.{type(self).__name__}._validate:\n"
                f"SPH smoothing lengths must be >= {self.min_valid_size:f} px in size for "
                f"{self._label} kernel integral approximation accuracy within 1%.\nThis check "
                "may be disabled by calling martini.martini.Martini.insert_source_in_cube with "
                "'skip_validation=True', but use this with care.",
                sm_lengths, valid, noraise=noraise, quiet=quiet)
        return valid


class _WendlandC2Kernel(_MinSizeKernel):
    """Wendland C2: W(q) = 21/(2 pi) (1-q)^4 (4q+1), q < 1."""

    min_valid_size = 1.51
    native_type = N.MG_KERNEL_WENDLAND_C2
    _label = "WendlandC2"

    def kernel(self, q):
        return np.where(q < 1, np.power(1 - q, 4) * (4 * q + 1), 0) * (21 / 2 / np.pi)


class _WendlandC6Kernel(_MinSizeKernel):
    """Wendland C6: W(q) = 1365/(64 pi) (1-q)^8 (1 + 8q + 25q^2 + 32q^3), q < 1."""

    min_valid_size = 1.29
    native_type = N.MG_KERNEL_WENDLAND_C6
    _label = "WendlandC6"

    def kernel(self, q):
        return np.where(q < 1, np.power(1 - q, 8) * (1 + 8 * q + 25 * q**2 + 32 * q**3), 0) * (
            1365 / 64 / np.pi)


class _CubicSplineKernel(_MinSizeKernel):
    """Cubic spline (M4): 8/pi [1 - 6q^2 + 6q^3 | 2(1-q)^3], q < 1."""

    min_valid_size = 1.16
    native_type = N.MG_KERNEL_CUBIC_SPLINE
    _label = "CubicSplineKernel"

    def kernel(self, q):
        W = np.where(q < 0.5, 1 - 6 * np.power(q, 2) + 6 * np.power(q, 3), 2 * np.power(1 - q, 3))
        W = np.where(q > 1, 0.0, W)
        return W * (8 / np.pi)


class _QuarticSplineKernel(_MinSizeKernel):
    """Quartic spline (M5), 15625/(512 pi) times three shells."""

    min_valid_size = 1.2385
    native_type = N.MG_KERNEL_QUARTIC_SPLINE
    _label = "QuarticSplineKernel"

    def kernel(self, q):
        q = np.asarray(q, dtype=np.float64)
        W = np.zeros(q.shape)
        m1 = q < 0.2
        m2 = (q >= 0.2) & (q < 0.6)
        m3 = (q >= 0.6) & (q < 1)
        W = np.where(m1, (1 - q) ** 4 - 5 * (0.6 - q) ** 4 + 10 * (0.2 - q) ** 4, W)
        W = np.where(m2, (1 - q) ** 4 - 5 * (0.6 - q) ** 4, W)
        W = np.where(m3, (1 - q) ** 4, W)
        return W * (15625 / 512 / np.pi)


class _GaussianKernel(_BaseSPHKernel):
    """Truncated Gaussian with FWHM 1 (sph_kernels.py:897-1080)."""

    native_type = N.MG_KERNEL_GAUSSIAN

    def __init__(self, truncate: float = 3.0):
        self.truncate = float(truncate)
        if self.truncate < 2:
            raise RuntimeError("GaussianKernel with truncation <2sigma will cause large errors in "
                               "total mass.")
        if self.truncate < 3:
            self.min_valid_size = 3.7
        elif self.truncate < 4:
            self.min_valid_size = 2.3357
        elif self.truncate < 5:
            self.min_valid_size = 1.1288
        elif self.truncate < 6:
            self.min_valid_size = 0.45
        else:
            self.min_valid_size = 0.336
        self.norm = erf(self.truncate / np.sqrt(2)) - 2 * self.truncate / np.sqrt(
            2 * np.pi) * np.exp(-np.power(self.truncate, 2) / 2)
        super().__init__()
        self.size_in_fwhm = self.truncate / (2 * np.sqrt(2 * np.log(2)))

    def kernel(self, q):
        sig = 1 / (2 * np.sqrt(2 * np.log(2)))
        return np.where(q < self.truncate * sig,
                        np.power(sig * np.sqrt(2 * np.pi), -3) * np.exp(-np.power(q / sig, 2) / 2),
                        0) / self.norm

    def _validate(self, sm_lengths, noraise=False, quiet=False):
        valid = np.asarray(sm_lengths) >= self.min_valid_size
        if np.logical_not(valid).any():
            self._validate_error(
                "martini.sph_kernels._GaussianKernel._validate:\n"
                f"SPH smoothing lengths must be >= {self.min_valid_size:f} px in size for "
                "GaussianKernel kernel integral approximation accuracy within 1%.\nThis check "
                "may be disabled by calling martini.martini.Martini.insert_source_in_cube with "
                "'skip_validation=True', but use this with care. Note that the minimum size "
                "depends on the kernel truncation.", sm_lengths, valid, noraise=noraise,
                quiet=quiet)
        return valid

    def _device_kernels(self):
        return [(self.native_type, self.truncate)]


class DiracDeltaKernel(_BaseSPHKernel):
    """Point-like particles: weight 1 in the pixel within half a pixel."""

    max_valid_size = 0.5
    native_type = N.MG_KERNEL_DIRAC

    def __init__(self, size_in_fwhm: float = 1.0):
        super().__init__()
        self.size_in_fwhm = size_in_fwhm
        self._rescale = 1.0

    def kernel(self, q):
        return np.where(q, 0, np.inf)

    def _validate(self, sm_lengths, noraise=False, quiet=False):
        valid = np.asarray(sm_lengths) <= self.max_valid_size
        if np.logical_not(valid).any():
            self._validate_error(
                "martini.sph_kernels.DiracDeltaKernel._validate:\n"
                f"provided smoothing scale (FWHM) must be <= {self.max_valid_size:f} px in size "
                "for DiracDelta kernel to be a reasonable approximation. Call "
                "martini.martini.Martini.insert_source_in_cube with 'skip_validation=True' to "
                "override at the cost of accuracy, but use this with care.", sm_lengths, valid,
                noraise=noraise, quiet=quiet)
        return valid


class _AdaptiveKernel(_BaseSPHKernel):
    """Per-particle choice of the first kernel whose approximation is valid
    (sph_kernels.py:1207-1399); particles with none use kernels[0]."""

    def __init__(self, kernels):
        self.kernels = tuple(kernels)
        if len(self.kernels) > N.MG_MAX_KERNELS:
            raise ValueError(f"at most {N.MG_MAX_KERNELS} kernels")
        super().__init__()

    def _init_sm_lengths(self, source, datacube):
        super()._init_sm_lengths(source, datacube)
        idx = -np.ones(self.sm_lengths.shape, dtype=np.int64)
        for ik, K in enumerate(self.kernels):
            idx[(idx == -1) & K._validate(self.sm_lengths * K._rescale, noraise=True,
                                          quiet=True)] = ik
        self.kernel_indices = idx
        sizes = np.array([K.size_in_fwhm for K in self.kernels], dtype=np.float64)
        rescales = np.array([K._rescale for K in self.kernels], dtype=np.float64)
        self.size_in_fwhm = sizes[idx]
        self.size_in_fwhm[idx == -1] = sizes[0]
        self._rescale = rescales[idx]
        self._rescale[idx == -1] = rescales[0]

    def _apply_mask(self, mask):
        self.size_in_fwhm = self.size_in_fwhm[mask]
        self._rescale = self._rescale[mask]
        self.kernel_indices = self.kernel_indices[mask]
        super()._apply_mask(mask)

    def eval_kernel(self, r, h):
        return self.kernels[0].eval_kernel(r, h)

    def kernel(self, q):
        return self.kernels[0].kernel(q)

    def _validate(self, sm_lengths, noraise=False, quiet=False):
        valid = self.kernel_indices >= 0
        if np.logical_not(valid).any():
            self._validate_error(
                "martini.sph_kernels._AdaptiveKernel._validate:\nSome particles have no kernel "
                "candidate for which accuracy passes validation.\nThis check may be disabled "
                "by calling martini.martini.Martini.insert_source_in_cube with "
                "'skip_validation=True', but use this with care.\n", sm_lengths, valid,
                noraise=noraise, quiet=quiet)
        return valid

    def _device_kernels(self):
        out = []
        for K in self.kernels:
            out.extend(K._device_kernels())
        return out

    def _device_arrays(self):
        return self.sm_lengths * self._rescale, self.kernel_indices.astype(np.int8)


class WendlandC2Kernel(_AdaptiveKernel):
    """WendlandC2 falling back to DiracDelta and Gaussian(6) (sph_kernels.py:1603-1661)."""

    def __init__(self):
        super().__init__((_WendlandC2Kernel(), DiracDeltaKernel(), _GaussianKernel(truncate=6.0)))


class WendlandC6Kernel(_AdaptiveKernel):
    """WendlandC6 falling back to DiracDelta and Gaussian(6) (sph_kernels.py:1664-1721)."""

    def __init__(self):
        super().__init__((_WendlandC6Kernel(), DiracDeltaKernel(), _GaussianKernel(truncate=6.0)))


class CubicSplineKernel(_AdaptiveKernel):
    """Cubic spline falling back to DiracDelta and Gaussian(6) (sph_kernels.py:1724-1785)."""

    def __init__(self):
        super().__init__((_CubicSplineKernel(), DiracDeltaKernel(), _GaussianKernel(truncate=6.0)))


class GaussianKernel(_AdaptiveKernel):
    """Gaussian(truncate) falling back to DiracDelta and Gaussian(6) (sph_kernels.py:1788-1865)."""

    def __init__(self, truncate: float = 3.0):
        super().__init__((_GaussianKernel(truncate=truncate), DiracDeltaKernel(),
                          _GaussianKernel(truncate=6.0)))


class QuarticSplineKernel(_AdaptiveKernel):
    """Quartic spline falling back to DiracDelta and Gaussian(6) (sph_kernels.py:1868-1933)."""

    def __init__(self):
        super().__init__((_QuarticSplineKernel(), DiracDeltaKernel(),
                          _GaussianKernel(truncate=6.0)))


class AdaptiveKernel:
    """Removed in the reference's v2.0.3 (sph_kernels.py:1936-1959)."""

    def __init__(self, *args, **kwargs):
        raise NotImplementedError(
            "Pre-configured adaptive kernels have been implemented in v2.0.3, see the SPH "
            "Kernels page in the documentation for details. You most likely want to use "
            "WendlandC2Kernel(), WendlandC6Kernel(), CubicSplineKernel() or "
            "QuarticSplineKernel() where you previously used AdaptiveKernel(...).")


__all__ = ["_WendlandC2Kernel", "_WendlandC6Kernel", "_CubicSplineKernel", "_QuarticSplineKernel",
           "_GaussianKernel", "DiracDeltaKernel", "_AdaptiveKernel", "WendlandC2Kernel",
           "WendlandC6Kernel", "CubicSplineKernel", "GaussianKernel", "QuarticSplineKernel",
           "AdaptiveKernel", "find_fwhm"]

