"""DataCube with the reference's constructor and channel grid (no astropy).

Mirrors ``martini.datacube.DataCube`` (martini/datacube.py:49-886): the cube
array ``_array`` of shape (n_px_x + 2 padx, n_px_y + 2 pady, n_channels[, 1])
in Jy/pix^2 (float64 on the host), the WCS parameters that place particles
on it (datacube.py:438-486), the channel edges (datacube.py:513-562) and
padding (datacube.py:669-729).  Units are tracked in ``_array_unit``.
"""

from __future__ import annotations

import numpy as np

from . import units as u


class DataCube:
    """Spectral data cube: pixel grid, channel grid and the flux array.

    Parameters follow the reference.  Without astropy, ``px_size`` is in
    arcsec, ``ra``/``dec`` in degrees, and ``channel_width`` /
    ``spectral_centre`` in km/s, or in Hz when ``freq_channels=True``.
    Astropy Quantities are accepted and converted (a frequency
    ``channel_width`` selects frequency channels, as in datacube.py:190-197).
    """

    def __init__(self, *, n_px_x: int, n_px_y: int, n_channels: int, px_size, channel_width,
                 spectral_centre=0.0, ra=0.0, dec=0.0, stokes_axis: bool = False,
                 coordinate_frame=None, specsys: str = "icrs", freq_channels: bool = False,
                 velocity_centre=None):
        if velocity_centre is not None:
            spectral_centre = velocity_centre
        if coordinate_frame is not None and type(coordinate_frame).__name__ != "ICRS":
            raise NotImplementedError("only the ICRS coordinate frame is supported")
        if specsys not in ("icrs", None):
            raise NotImplementedError("only specsys='icrs' is supported")
        self.stokes_axis = bool(stokes_axis)
        self.specsys = specsys
        self.n_px_x, self.n_px_y, self.n_channels = int(n_px_x), int(n_px_y), int(n_channels)
        self.px_size = u.scalar(px_size, "arcsec")
        ptype = u.physical_type(channel_width)
        if ptype is not None:
            freq_channels = ptype == "frequency"
            if ptype not in ("frequency", "speed"):
                raise ValueError("Channel width must have frequency or velocity units.")
        self._freq_channel_mode = bool(freq_channels)
        if self._freq_channel_mode:
            self.channel_width = abs(u.scalar(channel_width, "Hz"))
            if u.physical_type(spectral_centre) == "speed":
                self.spectral_centre = float(u.radio_frequency_hz(u.scalar(spectral_centre, "km/s")))
            else:
                self.spectral_centre = u.scalar(spectral_centre, "Hz")
        else:
            self.channel_width = abs(u.scalar(channel_width, "km/s"))
            if u.physical_type(spectral_centre) == "frequency":
                self.spectral_centre = float(u.radio_velocity_kms(u.scalar(spectral_centre, "Hz")))
            else:
                self.spectral_centre = u.scalar(spectral_centre, "km/s")
        self.ra = u.scalar(ra, "deg")
        self.dec = u.scalar(dec, "deg")
        self.padx = 0
        self.pady = 0
        shape = (self.n_px_x, self.n_px_y, self.n_channels) + ((1,) if self.stokes_axis else ())
        self._array = np.zeros(shape)
        self._array_unit = "Jy/pix2"

    # ---- WCS (datacube.py:438-486) -----------------------------------------
    @property
    def crpix(self):
        """1-based reference pixels of the RA, Dec and spectral axes."""
        return (self.n_px_x / 2.0 + 0.5 + self.padx, self.n_px_y / 2.0 + 0.5 + self.pady,
                self.n_channels / 2.0 + 0.5)

    @property
    def cdelt(self):
        """Axis increments: deg, deg, and Hz (FREQ) or km/s (VRAD, negative)."""
        spec = self.channel_width if self._freq_channel_mode else -self.channel_width
        return (-self.px_size / 3600.0, self.px_size / 3600.0, spec)

    @property
    def crval(self):
        return (self.ra, self.dec, self.spectral_centre)

    # ---- channels (datacube.py:494-562) --------------------------------------
    def _spectral_world(self, pix0):
        crpix = self.crpix[2]
        return self.crval[2] + self.cdelt[2] * (np.asarray(pix0, dtype=np.float64) + 1 - crpix)

    @property
    def channel_edges(self):
        """Channel edges in the spectral axis' unit (Hz or km/s)."""
        return self._spectral_world(np.arange(self.n_channels + 1) - 0.5)

    @property
    def channel_mids(self):
        return self._spectral_world(np.arange(self.n_channels))

    @property
    def velocity_channel_edges(self):
        """Channel edges as radio velocities, km/s (decreasing for default cubes)."""
        e = self.channel_edges
        return u.radio_velocity_kms(e) if self._freq_channel_mode else e

    @property
    def velocity_channel_mids(self):
        m = self.channel_mids
        return u.radio_velocity_kms(m) if self._freq_channel_mode else m

    @property
    def frequency_channel_edges(self):
        e = self.channel_edges
        return e if self._freq_channel_mode else u.radio_frequency_hz(e)

    @property
    def frequency_channel_mids(self):
        m = self.channel_mids
        return m if self._freq_channel_mode else u.radio_frequency_hz(m)

    def spectral_pixel(self, v_kms):
        """0-based spectral pixel coordinate of a radio velocity (km/s)."""
        world = u.radio_frequency_hz(v_kms) if self._freq_channel_mode else np.asarray(v_kms)
        return (self.crpix[2] - 1) + (world - self.crval[2]) / self.cdelt[2]

    # ---- array management ----------------------------------------------------
    @property
    def shape(self):
        return self._array.shape

    def add_pad(self, pad):
        """Grow the spatial axes by pad[0], pad[1] on each side (datacube.py:669-708)."""
        if self.padx > 0 or self.pady > 0:
            raise RuntimeError("Tried to add padding to already padded datacube array.")
        px, py = int(pad[0]), int(pad[1])
        shape = (self.n_px_x + 2 * px, self.n_px_y + 2 * py, self.n_channels) + (
            (1,) if self.stokes_axis else ())
        new = np.zeros(shape)
        new[px:shape[0] - px, py:shape[1] - py, ...] = self._array
        self._array = new
        self.padx, self.pady = px, py

    def drop_pad(self):
        """Remove the padding (datacube.py:710-729)."""
        if self.padx == 0 and self.pady == 0:
            return
        self._array = self._array[self.padx:-self.padx or None, self.pady:-self.pady or None, ...]
        self.padx, self.pady = 0, 0

    def copy(self):
        c = DataCube(n_px_x=self.n_px_x, n_px_y=self.n_px_y, n_channels=self.n_channels,
                     px_size=self.px_size, channel_width=self.channel_width,
                     spectral_centre=self.spectral_centre, ra=self.ra, dec=self.dec,
                     stokes_axis=self.stokes_axis, freq_channels=self._freq_channel_mode)
        c.padx, c.pady = self.padx, self.pady
        c._array = self._array.copy()
        c._array_unit = self._array_unit
        return c

    def __repr__(self):
        return (f"DataCube({self.n_px_x}x{self.n_px_y}x{self.n_channels}, px {self.px_size}\", "
                f"channel {self.channel_width} {'Hz' if self._freq_channel_mode else 'km/s'})")
