"""Spectral line models: the reference's classes; spectra are evaluated on
the GPU inside the insertion kernel (and materialised by ``mg_spectra`` only
when ``.spectra`` is read).

Mirrors martini/spectral_models.py: ``GaussianSpectrum`` (:304-485) with a
fixed width or the thermal width sqrt(k_B T / m_p) (:465-485), and
``DiracDeltaSpectrum`` (:488-587).  Per particle the amplitude is
mHI / D^2 / 2.36e5 (Jy km/s; :63-147) and the channel spectrum is that
amplitude times the line profile integrated over the channel, divided by the
channel width.
"""

from __future__ import annotations

import numpy as np

from . import _native as N
from . import units as u


class _BaseSpectrum:
    native_model = None

    def __init__(self, ncpu=None, spec_dtype=np.float64):
        self.ncpu = ncpu if ncpu is not None else 1
        self.spec_dtype = spec_dtype
        self._spectra = None
        self._owner = None

    def half_width(self, source):
        raise NotImplementedError

    def _device_sigma(self, source):
        """(per-particle sigma km/s or None, constant sigma)."""
        return None, 0.0

    @property
    def spectra(self):
        """Per-particle channel spectra (N, Nc) in Jy, computed on the GPU on
        first access after ``init_spectra``; None before."""
        if self._spectra is None and self._owner is not None:
            self._spectra = self._owner._materialise_spectra().astype(self.spec_dtype)
        return self._spectra

    @spectra.setter
    def spectra(self, value):
        self._spectra = value

    def init_spectra(self, source, datacube):
        """Bind the model to its source and cube; the spectra are evaluated on
        the GPU when needed (spectral_models.py:63-147 evaluates them here)."""
        edges = datacube.velocity_channel_edges
        d = np.diff(edges)
        if not (np.all(d > 0) or np.all(d < 0)):
            raise ValueError("Channel edges are not monotonic sequence.")
        self._spectra = None


class GaussianSpectrum(_BaseSpectrum):
    """Gaussian line of fixed ``sigma`` (km/s) or ``sigma="thermal"``."""

    native_model = N.MG_SPECTRUM_GAUSSIAN

    def __init__(self, sigma=7.0, ncpu=None, spec_dtype=np.float64):
        self.sigma_mode = sigma if isinstance(sigma, str) else u.value(sigma, "km/s")
        super().__init__(ncpu=ncpu, spec_dtype=spec_dtype)

    def half_width(self, source):
        """1D velocity dispersion in km/s (spectral_models.py:465-485)."""
        if isinstance(self.sigma_mode, str):
            if self.sigma_mode != "thermal":
                raise ValueError("sigma must be a velocity or 'thermal'")
            return np.sqrt(u.K_B * np.asarray(source.T_g, dtype=np.float64) / u.M_P) / 1e3
        return self.sigma_mode

    def _device_sigma(self, source):
        s = np.asarray(self.half_width(source), dtype=np.float64)
        if s.ndim == 0:
            return None, float(s)
        return s.astype(np.float32), 0.0


class DiracDeltaSpectrum(_BaseSpectrum):
    """All of a particle's flux in the channel containing its velocity (both
    channels when it sits exactly on an edge, spectral_models.py:544-570)."""

    native_model = N.MG_SPECTRUM_DIRAC

    def half_width(self, source):
        return 0.0


__all__ = ["GaussianSpectrum", "DiracDeltaSpectrum"]
