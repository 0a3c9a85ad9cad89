"""SPH particle source with the reference's constructor and sky projection.

Mirrors ``martini.sources.SPHSource`` (martini/sources/sph_source.py:53-1016)
for what the insertion path needs: particle arrays, rotation, placement at a
distance and sky position, Hubble flow plus peculiar velocity
(sph_source.py:265-326), projection to pixel coordinates through the cube's
TAN/VRAD (or FREQ) WCS (sph_source.py:328-362) and masking
(sph_source.py:364-393).  Set-up arithmetic is FP64 numpy on the host, as in
the reference's ``Martini.__init__``; the insertion itself runs on the GPU.
"""

from __future__ import annotations

import numpy as np

from . import units as u


class SPHSource:
    """HI source made of SPH particles.

    Without astropy: ``distance`` in Mpc, ``vpeculiar`` in km/s, ``ra``/``dec``
    in degrees, ``T_g`` in K, ``mHI_g`` in Msun, ``xyz_g``/``hsm_g`` in kpc,
    ``vxyz_g`` in km/s.  ``rotation`` may be a ``scipy.spatial.transform.Rotation``
    or a 3x3 matrix applied to column vectors.
    """

    def __init__(self, *, distance, vpeculiar=0.0, rotation=None, L_coords=None, ra=0.0, dec=0.0,
                 h: float = 0.7, T_g=None, mHI_g, xyz_g, vxyz_g, hsm_g=None,
                 coordinate_axis=None, coordinate_frame=None):
        if L_coords is not None:
            raise NotImplementedError(
                "L_coords alignment is not provided; pass an explicit rotation instead")
        if coordinate_frame is not None and type(coordinate_frame).__name__ != "ICRS":
            raise NotImplementedError("only the ICRS coordinate frame is supported")
        xyz = u.value(xyz_g, "kpc")
        vxyz = u.value(vxyz_g, "km/s")
        if coordinate_axis is None:
            if xyz.shape[0] == 3 and xyz.shape[1] != 3:
                coordinate_axis = 0
            elif xyz.shape[0] != 3 and xyz.shape[1] == 3:
                coordinate_axis = 1
            elif xyz.shape == (3, 3):
                raise RuntimeError("martini.sources.SPHSource: cannot guess coordinate_axis with "
                                   "shape (3, 3), provide explicitly.")
            else:
                raise RuntimeError("martini.sources.SPHSource: incorrect coordinate shape (not "
                                   "(3, N) or (N, 3)).")
        if xyz.shape != vxyz.shape:
            raise ValueError("martini.sources.SPHSource: xyz_g and vxyz_g must have matching "
                             "shapes.")
        if coordinate_axis == 0:
            xyz, vxyz = xyz.T, vxyz.T
        self.xyz_g = np.ascontiguousarray(xyz, dtype=np.float64)
        self.vxyz_g = np.ascontiguousarray(vxyz, dtype=np.float64)
        self.h = float(h)
        self.T_g = None if T_g is None else u.value(T_g, "K")
        n = self.xyz_g.shape[0]
        m = u.value(mHI_g, "Msun")
        self.mHI_g = np.broadcast_to(m, (n,)).astype(np.float64) if m.ndim == 0 else m
        self.input_mass = float(np.sum(self.mHI_g))
        hs = None if hsm_g is None else u.value(hsm_g, "kpc")
        self.hsm_g = None if hs is None else (np.broadcast_to(hs, (n,)).astype(np.float64)
                                              if hs.ndim == 0 else hs)
        self.npart = n
        self.ra = u.scalar(ra, "deg")
        self.dec = u.scalar(dec, "deg")
        self.distance = u.scalar(distance, "Mpc")
        self.vpeculiar = u.scalar(vpeculiar, "km/s")
        self.vhubble = self.h * 100.0 * self.distance
        self.vsys = self.vhubble + self.vpeculiar
        self._rotation = np.eye(3)
        if rotation is not None:
            self.rotate(rotation)
        self.skycoords = None
        self.pixcoords = None

    def rotate(self, rotation):
        """Rotate positions and velocities (sph_source.py:442-526)."""
        mat = rotation.as_matrix() if hasattr(rotation, "as_matrix") else np.asarray(rotation)
        self.xyz_g = self.xyz_g @ mat.T
        self.vxyz_g = self.vxyz_g @ mat.T
        self._rotation = mat @ self._rotation

    def _init_skycoords(self):
        """Sky position, distance and line-of-sight velocity of each particle.

        Rotation R_y(dec) R_z(-ra) on row vectors, translation by the source
        distance along (ra, dec), peculiar velocity along that direction and
        Hubble flow h * 100 km/s/Mpc * r per particle (sph_source.py:265-317);
        radial velocity = v . r / |r|.
        """
        ra = np.deg2rad(self.ra)
        dec = np.deg2rad(self.dec)
        cr, sr, cd, sd = np.cos(ra), np.sin(ra), np.cos(dec), np.sin(dec)
        rot = np.array([[cd, 0.0, sd], [0.0, 1.0, 0.0], [-sd, 0.0, cd]]) @ np.array(
            [[cr, sr, 0.0], [-sr, cr, 0.0], [0.0, 0.0, 1.0]])
        unit = np.array([cd * cr, cd * sr, sd])
        pos = self.xyz_g @ rot + unit * (self.distance * 1e3)
        vel = self.vxyz_g @ rot + (self.h * 100.0 * 1e-3) * pos + unit * self.vpeculiar
        d = np.sqrt(np.einsum("ij,ij->i", pos, pos))
        with np.errstate(invalid="ignore", divide="ignore"):
            vlos = np.einsum("ij,ij->i", pos, vel) / d
            dec_p = np.rad2deg(np.arcsin(pos[:, 2] / d))
        ra_p = np.rad2deg(np.arctan2(pos[:, 1], pos[:, 0])) % 360.0
        self.skycoords = _SkyCoords(ra_p, dec_p, d * 1e-3, vlos)

    def _init_pixcoords(self, datacube, origin: int = 0):
        """pixcoords (3, N): TAN projection onto the cube's WCS and spectral
        pixel of the radial velocity (sph_source.py:328-362)."""
        if self.skycoords is None:
            raise RuntimeError("Initialize source.skycoords before calling _init_pixcoords.")
        sc = self.skycoords
        (c1, c2, _), (d1, d2, _), (v1, v2, _) = datacube.crpix, datacube.cdelt, datacube.crval
        a = np.deg2rad(sc.ra)
        d = np.deg2rad(sc.dec)
        a0 = np.deg2rad(v1)
        d0 = np.deg2rad(v2)
        cosc = np.sin(d) * np.sin(d0) + np.cos(d) * np.cos(d0) * np.cos(a - a0)
        with np.errstate(divide="ignore", invalid="ignore"):
            xi = np.rad2deg(np.cos(d) * np.sin(a - a0) / cosc)
            eta = np.rad2deg((np.sin(d) * np.cos(d0) - np.cos(d) * np.sin(d0) * np.cos(a - a0))
                             / cosc)
        x = c1 - 1 + origin + xi / d1
        y = c2 - 1 + origin + eta / d2
        behind = ~(cosc > 0)  # wcslib flags these invalid -> NaN
        x[behind] = np.nan
        y[behind] = np.nan
        z = datacube.spectral_pixel(sc.radial_velocity) + origin
        self.pixcoords = np.vstack((x, y, z))

    def apply_mask(self, mask):
        """Keep particles where mask is True (sph_source.py:364-393)."""
        mask = np.asarray(mask, dtype=bool)
        if mask.size != self.npart:
            raise ValueError("Mask must have same length as particle arrays.")
        if mask.sum() == 0:
            raise RuntimeError("No non-zero mHI source particles in target region.")
        self.npart = int(mask.sum())
        if self.T_g is not None and np.ndim(self.T_g):
            self.T_g = self.T_g[mask]
        self.mHI_g = self.mHI_g[mask]
        self.xyz_g = self.xyz_g[mask]
        self.vxyz_g = self.vxyz_g[mask]
        if self.hsm_g is not None:
            self.hsm_g = self.hsm_g[mask]
        if self.skycoords is not None:
            self.skycoords = self.skycoords[mask]
        if self.pixcoords is not None:
            self.pixcoords = self.pixcoords[:, mask]


class _SkyCoords:
    """ra/dec (deg), distance (Mpc) and radial_velocity (km/s) per particle."""

    def __init__(self, ra, dec, distance, radial_velocity):
        self.ra, self.dec = ra, dec
        self.distance = distance
        self.radial_velocity = radial_velocity

    def __getitem__(self, m):
        return _SkyCoords(self.ra[m], self.dec[m], self.distance[m], self.radial_velocity[m])
