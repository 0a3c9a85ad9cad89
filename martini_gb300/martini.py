"""``Martini`` with the reference's constructor and insertion call, running
the insertion on the GPU.

Mirrors martini/martini.py: ``_BaseMartini.__init__`` (:118-151: beam pad,
sky and pixel coordinates, smoothing lengths, pruning), ``_prune_particles``
(:168-241), ``_insert_source_in_cube`` (:285-407) and
``Martini.insert_source_in_cube`` (:827-861), ``reset`` (:409-425) and
``init_spectra`` (:153-166).  The per-pixel loop of :327-362 is replaced by
one call of the CUDA library; the cube is accumulated into the host array
(``_array +=``, as :338) and converted to Jy/arcsec^2 (:364-366).
"""

from __future__ import annotations

import numpy as np

from . import _native as N
from .datacube import DataCube
from .engine import DeviceParticles, InsertionEngine

MHI_TO_JY = 2.36e5  # Msun / (Mpc^2 Jy km/s), martini/spectral_models.py:127-145

FORMS = {"fp32": N.MG_FORM_FP32, "bf16x3": N.MG_FORM_BF16X3, "f16x3": N.MG_FORM_F16X3}


class _BaseMartini:
    def __init__(self, *, source, datacube: DataCube, beam=None, noise=None, sph_kernel,
                 spectral_model, quiet: bool = False, _prune_kwargs: dict | None = None,
                 form: str = "fp32", device=None):
        self.quiet = quiet
        self.source = source
        self._datacube = datacube
        self.beam = beam
        self.noise = noise
        self.sph_kernel = sph_kernel
        self.spectral_model = spectral_model
        if form not in FORMS:
            raise ValueError(f"form must be one of {sorted(FORMS)}")
        self.form = form
        self._device = device
        self._engine = None
        if self.beam is not None:
            self.beam.init_kernel(self._datacube)
            self._datacube.add_pad(self.beam.needs_pad())
        self.source._init_skycoords()
        self.source._init_pixcoords(self._datacube)
        self.sph_kernel._init_sm_lengths(source=self.source, datacube=self._datacube)
        self.sph_kernel._init_sm_ranges()
        self._prune_particles(**(_prune_kwargs or {}))

    # ---- set-up ------------------------------------------------------------------
    def _prune_particles(self, spatial: bool = True, spectral: bool = True, mass: bool = True,
                         obj_type_str: str = "data cube"):
        """Drop particles that cannot contribute (martini/martini.py:168-241)."""
        src, dc, k = self.source, self._datacube, self.sph_kernel
        if not self.quiet:
            print(f"Source module contained {src.npart} particles with total HI mass of "
                  f"{src.mHI_g.sum():.2e} solMass.")
        hw = np.asarray(self.spectral_model.half_width(src)) / np.max(
            np.abs(np.diff(dc.velocity_channel_edges)))
        x, y, z = src.pixcoords
        r = k.sm_ranges
        reject = np.zeros(src.npart, dtype=bool)
        if spatial:
            reject |= (x + r < 0) | (y + r < 0)
            reject |= x - r > dc.n_px_x + dc.padx * 2
            reject |= y - r > dc.n_px_y + dc.pady * 2
            reject |= np.isnan(x) | np.isnan(y)
        if spectral:
            reject |= z + 4 * hw < 0
            reject |= z - 4 * hw > dc.n_channels
        if mass:
            reject |= src.mHI_g == 0
        accept = ~reject
        src.apply_mask(accept)
        k._apply_mask(accept)
        if not self.quiet:
            print(f"Pruned particles that will not contribute to {obj_type_str}, {src.npart} "
                  f"particles remaining with total HI mass of {src.mHI_g.sum():.2e} solMass.")

    def init_spectra(self):
        """Bind the spectral model (spectra are evaluated on the GPU)."""
        if not self.quiet:
            print("Initializing spectra...")
        self.spectral_model.init_spectra(self.source, self._datacube)
        self.spectral_model._owner = self
        if not self.quiet:
            print("Spectra initialized.")

    # ---- device inputs ------------------------------------------------------------
    @property
    def engine(self) -> InsertionEngine:
        if self._engine is None:
            self._engine = InsertionEngine(self._device)
        return self._engine

    def _device_inputs(self):
        import torch
        src, k, sm = self.source, self.sph_kernel, self.spectral_model
        h_eff, kidx = k._device_arrays()
        sig, sig_const = sm._device_sigma(src)
        amp = src.mHI_g * np.power(src.skycoords.distance, -2.0) / MHI_TO_JY
        dev = self.engine.device
        parts = DeviceParticles.from_host(
            dev, src.pixcoords[0], src.pixcoords[1], k.sm_ranges, h_eff, kidx,
            v=src.skycoords.radial_velocity, sigma=sig, amp=amp)
        edges = torch.from_numpy(np.ascontiguousarray(self._datacube.velocity_channel_edges,
                                                      dtype=np.float64)).to(dev)
        return parts, k._device_kernels(), sm.native_model, sig_const, edges

    def _materialise_spectra(self):
        parts, _, model, sig_const, edges = self._device_inputs()
        return self.engine.spectra(parts, model, sig_const, self._datacube.n_channels,
                                   edges).cpu().numpy()

    # ---- insertion ------------------------------------------------------------------
    def _insert_source_in_cube(self, skip_validation: bool = False, progressbar=None,
                               ncpu: int = 1, quiet=None):
        """Populate the DataCube with flux from the source particles.

        ``progressbar`` and ``ncpu`` are accepted for compatibility; the GPU
        path has no per-pixel loop to report on or thread over.
        """
        if self.spectral_model._owner is not self:
            self.init_spectra()
        self.sph_kernel._confirm_validation(noraise=skip_validation, quiet=self.quiet)
        dc = self._datacube
        parts, kernels, model, sig_const, edges = self._device_inputs()
        nx, ny, nc = dc._array.shape[:3]
        cube, flux = self.engine.insert(parts, kernels, model, sig_const, nx, ny, nc, edges,
                                        padx=dc.padx, pady=dc.pady, form=FORMS[self.form])
        add = cube.cpu().numpy().astype(np.float64)
        flux = flux.cpu().numpy()
        if dc.stokes_axis:
            add = add[..., np.newaxis]
        px2 = dc.px_size**2
        if dc._array_unit == "Jy/pix2":
            dc._array += add
            dc._array /= px2
        else:
            dc._array += add / px2
        dc._array_unit = "Jy/arcsec2"
        self._last_flux = flux
        inserted_flux = float(flux[0])
        inserted_mass = MHI_TO_JY * self.source.distance**2 * float(
            np.sum(flux[1:] * np.abs(np.diff(dc.velocity_channel_edges))))
        self.inserted_flux_density = inserted_flux
        self.inserted_mass = inserted_mass
        if (quiet is None and not self.quiet) or (quiet is not None and not quiet):
            arr = dc._array
            pos = arr[arr > 0]
            print("Source inserted.",
                  f"  Flux density in cube: {inserted_flux:.2e} Jy",
                  f"  Mass in cube (assuming distance {self.source.distance:.2f} Mpc and a "
                  f"spatially resolved source): {inserted_mass:.2e} solMass",
                  f"    [{inserted_mass / self.source.input_mass * 100:.0f}% of initial source "
                  "mass]",
                  f"  Maximum pixel: {arr.max():.2e} Jy / arcsec2",
                  "  Median non-zero pixel: "
                  f"{(np.median(pos) if pos.size else 0.0):.2e} Jy / arcsec2", sep="\n")

    def reset(self):
        """Zero the cube, keeping its shape and padding (martini/martini.py:409-425)."""
        dc = self._datacube
        dc._array = np.zeros(dc._array.shape)
        dc._array_unit = "Jy/pix2"


class Martini(_BaseMartini):
    """Synthetic HI data cubes from SPH particles, inserted on the GPU.

    Same constructor as the reference plus two keywords: ``form`` ("fp32",
    the FP32 CUDA-core contraction, or "bf16x3", the BF16 hi+lo tensor-core
    form) and ``device``.
    """

    def __init__(self, *, source, datacube, beam=None, noise=None, sph_kernel, spectral_model,
                 quiet: bool = False, form: str = "fp32", device=None):
        super().__init__(source=source, datacube=datacube, beam=beam, noise=noise,
                         sph_kernel=sph_kernel, spectral_model=spectral_model, quiet=quiet,
                         form=form, device=device)

    @property
    def datacube(self) -> DataCube:
        return self._datacube

    def insert_source_in_cube(self, skip_validation: bool = False, progressbar=None,
                              ncpu: int = 1):
        """Populate the DataCube with flux from the particles in the source
        (martini/martini.py:827-861)."""
        super()._insert_source_in_cube(skip_validation=skip_validation, progressbar=progressbar,
                                       ncpu=ncpu)
