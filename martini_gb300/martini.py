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

FORMS = {"fp32": N.MG_FORM_FP32, "bf16x3": N.MG_FORM_BF16X3, "f16x3": N.MG_FORM_F16X3,
         "bf16x6": N.MG_FORM_BF16X6}
# the chosen form: exact three-piece BF16 split on the tensor cores, within
# 1e-5 of peak and 1e-6 of flux of the FP64 reference arithmetic
DEFAULT_FORM = "bf16x6"


class _BaseMartini:
    def __init__(self, *, source, datacube: DataCube, beam=None, noise=None, sph_kernel,
                 spectral_model, quiet: bool = False, _prune_kwargs: dict | None = None,
                 form: str = DEFAULT_FORM, device=None):
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
        # this insertion's FP64 flux sums over the unpadded cube (total, then
        # per channel), from the GPU
        self._last_flux = flux
        # the summary sums the whole converted array, prior contents
        # included, over the unpadded pixels when both pads are non-zero
        # (martini/martini.py:367-392)
        pad_mask = (np.s_[dc.padx:-dc.padx, dc.pady:-dc.pady, ...]
                    if dc.padx > 0 and dc.pady > 0 else np.s_[...])
        in_jy = dc._array[pad_mask] * px2
        inserted_flux = float(np.sum(in_jy))
        per_channel = in_jy.sum(axis=(0, 1)).reshape(-1)
        inserted_mass = MHI_TO_JY * self.source.distance**2 * float(
            np.sum(per_channel * np.abs(np.diff(dc.velocity_channel_edges))))
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

    Same constructor as the reference plus two keywords: ``form`` and
    ``device``.  ``form`` selects the contraction: "bf16x6" (default; the
    exact three-piece BF16 split, six tensor-core products), "f16x3" (scaled
    FP16 hi + lo, three products), "fp32" (FP32 on CUDA cores) or "bf16x3"
    (BF16 hi + lo, three products: about 1e-5 relative per term, so it can
    miss the 1e-5-of-peak bar on cubes dominated by a few particles).
    """

    def __init__(self, *, source, datacube, beam=None, noise=None, sph_kernel, spectral_model,
                 quiet: bool = False, form: str = DEFAULT_FORM, device=None):
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

    def _wcs_cards(self):
        """Axis cards of the cube's WCS (datacube.py:438-486): RA---TAN and
        DEC--TAN in deg, VRAD in m/s or FREQ in Hz."""
        dc = self._datacube
        freq = dc._freq_channel_mode
        cards = [("CDELT1", -dc.px_size / 3600.0), ("CRPIX1", dc.n_px_x / 2.0 + 0.5 + dc.padx),
                 ("CRVAL1", float(dc.ra)), ("CTYPE1", "RA---TAN"), ("CUNIT1", "deg"),
                 ("CDELT2", dc.px_size / 3600.0), ("CRPIX2", dc.n_px_y / 2.0 + 0.5 + dc.pady),
                 ("CRVAL2", float(dc.dec)), ("CTYPE2", "DEC--TAN"), ("CUNIT2", "deg"),
                 ("CDELT3", abs(dc.channel_width) if freq else -abs(dc.channel_width) * 1e3),
                 ("CRPIX3", dc.n_channels / 2.0 + 0.5),
                 ("CRVAL3", float(dc.spectral_centre) * (1.0 if freq else 1e3)),
                 ("CTYPE3", "FREQ" if freq else "VRAD"), ("CUNIT3", "Hz" if freq else "m/s")]
        return cards

    def write_fits(self, filename: str, overwrite: bool = True, obj_name: str = "MOCK",
                   channels=None, dtype=None):
        """Write the cube to a FITS file (martini/martini.py:939-1051): the pad is
        dropped, '.fits' appended if absent, the reference's header cards."""
        import time as _time
        from . import __version__
        from .fits import write_primary
        dc = self._datacube
        dc.drop_pad()
        filename = filename + ".fits" if "fits" not in filename.split(".") else filename
        arr = dc._array
        unit = {"Jy/pix2": "Jy pix-2", "Jy/arcsec2": "Jy arcsec-2", "Jy/beam": "Jy/beam"}.get(
            dc._array_unit, dc._array_unit)
        cards = [("EXTEND", True)] + self._wcs_cards()
        if dc.stokes_axis:
            cards += [("CDELT4", 1.0), ("CRPIX4", 1.0), ("CRVAL4", 1.0), ("CTYPE4", "STOKES"),
                      ("CUNIT4", "PAR")]
        now = _time.time()
        mjd = now / 86400.0 + 40587.0
        cards += [("EPOCH", 2000), ("INSTRUME", "MARTINI", f"martini_gb300 {__version__}"),
                  ("BSCALE", 1.0), ("BZERO", 0.0), ("DATAMAX", float(np.max(arr))),
                  ("DATAMIN", float(np.min(arr))), ("ORIGIN", "martini_gb300"),
                  ("OBJECT", obj_name[:16])]
        if self.beam is not None:
            cards.append(("BPA", float(self.beam.bpa)))
        cards += [("OBSERVER", "K. Oman"), ("BUNIT", unit),
                  ("DATE-OBS", _time.strftime("%Y-%m-%dT%H:%M:%S", _time.gmtime(now))),
                  ("MJD-OBS", mjd)]
        if self.beam is not None:
            cards += [("BMAJ", self.beam.bmaj / 3600.0), ("BMIN", self.beam.bmin / 3600.0)]
        cards += [("BTYPE", "Intensity"), ("SPECSYS", "ICRS"), ("RESTFRQ", 1420405751.768)]
        data = arr.T
        if dtype is not None:
            data = data.astype(dtype, copy=False)
        write_primary(filename, cards, data, overwrite=overwrite)

    def write_beam_fits(self, filename: str, overwrite: bool = True, channels=None):
        """Write the beam image to a FITS file (martini/martini.py:1053-1105)."""
        from . import __version__
        from .fits import write_primary
        if self.beam is None:
            raise ValueError("Martini.write_beam_fits: Called with beam set to 'None'.")
        filename = filename if filename[-5:] == ".fits" else filename + ".fits"
        k = np.asarray(self.beam.kernel, dtype=np.float64)
        w = dict((c[0], c[1]) for c in self._wcs_cards())
        cards = [("EXTEND", True), ("BSCALE", 1.0), ("BZERO", 0.0), ("BUNIT", ""),
                 ("CRPIX1", k.shape[0] // 2 + 1), ("CDELT1", w["CDELT1"]), ("CRVAL1", w["CRVAL1"]),
                 ("CTYPE1", w["CTYPE1"]), ("CUNIT1", w["CUNIT1"]),
                 ("CRPIX2", k.shape[1] // 2 + 1), ("CDELT2", w["CDELT2"]), ("CRVAL2", w["CRVAL2"]),
                 ("CTYPE2", w["CTYPE2"]), ("CUNIT2", w["CUNIT2"]),
                 ("CRPIX3", 1), ("CDELT3", w["CDELT3"]), ("CRVAL3", w["CRVAL3"]),
                 ("CTYPE3", w["CTYPE3"]), ("CUNIT3", w["CUNIT3"]), ("SPECSYS", "ICRS"),
                 ("BMAJ", self.beam.bmaj / 3600.0), ("BMIN", self.beam.bmin / 3600.0),
                 ("BPA", float(self.beam.bpa)), ("BTYPE", "beam"), ("EPOCH", 2000),
                 ("OBSERVER", "K. Oman"), ("OBJECT", "MOCKBEAM"),
                 ("INSTRUME", "MARTINI", f"martini_gb300 {__version__}"),
                 ("DATAMAX", float(k.max())), ("DATAMIN", float(k.min())),
                 ("ORIGIN", "martini_gb300")]
        write_primary(filename, cards, k[np.newaxis, ...].transpose(0, 2, 1),
                      overwrite=overwrite)

    def convolve_beam(self):
        """Convolve the cube with the beam on the GPU, drop the pad and convert
        to Jy/beam (martini/martini.py:863-901)."""
        import warnings

        import torch
        from .engine import convolve_beam
        if self.beam is None:
            warnings.warn("Skipping beam convolution, no beam object provided to Martini.")
            return
        dc = self._datacube
        px, py = self.beam.needs_pad()
        if dc.padx < px or dc.pady < py:
            raise ValueError("datacube padding insufficient for beam convolution (perhaps you "
                             "loaded a datacube state with datacube.load_state that was "
                             "previously initialized by martini with a smaller beam?)")
        arr = dc._array[..., 0] if dc.stokes_axis else dc._array
        if dc._array_unit == "Jy/pix2":
            arr = arr / dc.px_size ** 2
        cube = torch.from_numpy(np.ascontiguousarray(arr, dtype=np.float32)).to(
            self.engine.device)
        out = convolve_beam(self.engine, cube, dc.padx, dc.pady, self.beam.kernel,
                            self.beam.area).cpu().numpy().astype(np.float64)
        dc._array = out[..., np.newaxis] if dc.stokes_axis else out
        dc.padx, dc.pady = 0, 0
        dc._array_unit = "Jy/beam"
        if not self.quiet:
            a = dc._array
            pos = a[a > 0]
            print("Beam convolved.",
                  f"  Data cube RMS after beam convolution: {np.std(a):.2e} Jy / beam",
                  f"  Maximum pixel: {a.max():.2e} Jy / beam",
                  "  Median non-zero pixel: "
                  f"{(np.median(pos) if pos.size else 0.0):.2e} Jy / beam", sep="\n")


class GlobalProfile(_BaseMartini):
    """The spatially integrated spectrum of a source, on the GPU
    (martini/martini.py:1369-1738).

    Every particle contributes its whole line unless it falls outside the
    band (spectral and mass pruning only, no spatial aperture); positions
    still set each particle's line of sight.  Same constructor as the
    reference; ``spectrum`` is in Jy.
    """

    def __init__(self, *, source, spectral_model, n_channels: int, channel_width,
                 spectral_centre=0.0, quiet: bool = False, channels=None, device=None):
        from .sph_kernels import DiracDeltaKernel
        datacube = DataCube(n_px_x=1, n_px_y=1, n_channels=n_channels, px_size=3600.0,
                            channel_width=channel_width, spectral_centre=spectral_centre)
        super().__init__(source=source, datacube=datacube, beam=None, noise=None,
                         sph_kernel=DiracDeltaKernel(size_in_fwhm=np.inf),
                         spectral_model=spectral_model, quiet=quiet,
                         _prune_kwargs=dict(spatial=False, spectral=True, mass=True,
                                            obj_type_str="spectrum"),
                         form="fp32", device=device)
        self.source.pixcoords[:2] = 0

    def insert_source_in_spectrum(self):
        """Form the spectrum (martini/martini.py:1551-1596): sum of the lines of
        every particle in the band, in Jy; the one-pixel cube holds it in
        Jy/arcsec^2 as the reference's does."""
        import torch
        from .engine import DeviceParticles, global_profile
        if self.spectral_model._owner is not self:
            self.init_spectra()
        src, dc, sm = self.source, self._datacube, self.spectral_model
        sig, sig_const = sm._device_sigma(src)
        amp = src.mHI_g * np.power(src.skycoords.distance, -2.0) / MHI_TO_JY
        n = src.npart
        zeros = np.zeros(n)
        dev = self.engine.device
        parts = DeviceParticles.from_host(dev, zeros, zeros, zeros, zeros.astype(np.float32),
                                          v=src.skycoords.radial_velocity, sigma=sig, amp=amp)
        edges = torch.from_numpy(np.ascontiguousarray(dc.velocity_channel_edges,
                                                      dtype=np.float64)).to(dev)
        spec = global_profile(self.engine, parts, sm.native_model, sig_const, dc.n_channels,
                              edges).cpu().numpy()
        self._spectrum = spec
        px2 = dc.px_size ** 2
        add = (spec / px2).reshape(1, 1, -1)
        if dc.stokes_axis:
            add = add[..., np.newaxis]
        if dc._array_unit == "Jy/pix2":
            dc._array = dc._array / px2
        dc._array = dc._array + add
        dc._array_unit = "Jy/arcsec2"
        if not self.quiet:
            flux = float(spec.sum())
            mass = MHI_TO_JY * src.distance ** 2 * flux * dc.channel_width
            print("Source inserted.",
                  f"  Flux density in spectrum: {flux:.2e} Jy",
                  f"  Mass in spectrum (assuming distance {src.distance:.2f} Mpc): {mass:.2e} "
                  "solMass",
                  f"    [{mass / src.input_mass * 100:.0f}% of initial source mass]", sep="\n")

    @property
    def spectrum(self):
        """Spatially integrated spectrum (Jy), formed on first access."""
        if not hasattr(self, "_spectrum"):
            self.insert_source_in_spectrum()
        return self._spectrum

    @property
    def channel_edges(self):
        return self._datacube.channel_edges

    @property
    def channel_mids(self):
        return self._datacube.channel_mids

    @property
    def frequency_channel_edges(self):
        return self._datacube.frequency_channel_edges

    @property
    def frequency_channel_mids(self):
        return self._datacube.frequency_channel_mids

    @property
    def velocity_channel_edges(self):
        return self._datacube.velocity_channel_edges

    @property
    def velocity_channel_mids(self):
        return self._datacube.velocity_channel_mids
