"""Radio telescope beams (martini/beams.py) for the GPU beam convolution.

``GaussianBeam`` keeps the reference's constructor and its beam image: the
2D Gaussian of ``f_kernel`` (beams.py:231-276) sampled on a 0.1-pixel grid,
fitted with a bicubic spline and integrated over each pixel of a
(2 size + 1)^2 image, size = ceil(bmaj * truncate / px + 1)
(beams.py:103-160, :277-295).  The image is host set-up work, done once per
cube; the convolution itself runs in the CUDA library (mg_convolve_beam).
"""

from __future__ import annotations

import numpy as np
import scipy.interpolate

from . import units as u


class _BaseBeam:
    def __init__(self, bmaj=15.0, bmin=None, bpa=0.0):
        self.bmaj = u.scalar(bmaj, "arcsec")
        self.bmin = self.bmaj if bmin is None else u.scalar(bmin, "arcsec")
        self.bpa = u.scalar(bpa, "deg")
        self.px_size = None
        self.kernel = None
        # FWHM -> Gaussian-equivalent area, pi bmaj bmin / (4 ln 2) (beams.py:84)
        self.area = np.pi * self.bmaj * self.bmin / 4 / np.log(2)  # arcsec^2

    def needs_pad(self):
        """Pad of the cube the convolution needs (beams.py:88-101)."""
        if self.kernel is None:
            raise RuntimeError("Beam kernel not initialized.")
        return self.kernel.shape[0] // 2, self.kernel.shape[1] // 2

    def init_kernel(self, datacube):
        """The pixel-integrated beam image (beams.py:103-160)."""
        self.px_size = datacube.px_size
        self.vel = datacube.spectral_centre
        self.ra = datacube.ra
        self.dec = datacube.dec
        npx_x, npx_y = self.kernel_size_px()
        px = self.px_size
        px_edges_x = np.arange(-npx_x - 0.5, npx_x + 0.50001, 1) * px
        px_edges_y = np.arange(-npx_y - 0.5, npx_y + 0.50001, 1) * px
        fine_x = np.arange(-npx_x - 0.5, npx_x + 0.501, 0.1) * px
        fine_y = np.arange(-npx_y - 0.5, npx_y + 0.501, 0.1) * px
        rbs = scipy.interpolate.RectBivariateSpline(
            fine_x, fine_y, self.f_kernel()(*np.meshgrid(fine_x, fine_y, indexing="ij")),
            kx=3, ky=3)
        xgrid, ygrid = np.meshgrid(px_edges_x, px_edges_y)
        self.kernel = np.vectorize(rbs.integral)(xgrid[1:, :-1], xgrid[1:, 1:], ygrid[:-1, 1:],
                                                 ygrid[1:, 1:])

    def f_kernel(self):
        raise NotImplementedError

    def kernel_size_px(self):
        raise NotImplementedError


class GaussianBeam(_BaseBeam):
    """Gaussian beam with FWHMs ``bmaj``, ``bmin`` (arcsec), position angle
    ``bpa`` (deg, East of North), truncated at ``truncate`` FWHM."""

    def __init__(self, bmaj=15.0, bmin=None, bpa=0.0, truncate: float = 4.0):
        self.truncate = truncate
        super().__init__(bmaj=bmaj, bmin=bmin, bpa=bpa)

    def f_kernel(self):
        """Beam amplitude (arcsec^-2) at offsets (x, y) in arcsec (beams.py:231-276)."""
        def fwhm_to_sigma(fwhm):
            return fwhm / (2.0 * np.sqrt(2.0 * np.log(2.0)))

        smaj = fwhm_to_sigma(self.bmaj)
        smin = fwhm_to_sigma(self.bmin)
        pa = np.deg2rad(self.bpa)
        a = np.cos(pa) ** 2 / (2.0 * smin ** 2) + np.sin(pa) ** 2 / (2.0 * smaj ** 2)
        b = -np.sin(2.0 * pa) / (4 * smin ** 2) + np.sin(2.0 * pa) / (4 * smaj ** 2)
        c = np.sin(pa) ** 2 / (2.0 * smin ** 2) + np.cos(pa) ** 2 / (2.0 * smaj ** 2)
        A = 1.0 / (2.0 * np.pi * smin * smaj)
        return lambda x, y: A * np.exp(-a * x ** 2 - 2.0 * b * x * y - c * y ** 2)

    def kernel_size_px(self):
        size = np.ceil(self.bmaj * self.truncate / self.px_size + 1)
        return size, size


__all__ = ["GaussianBeam"]
