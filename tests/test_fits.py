"""FITS output (Martini.write_fits / write_beam_fits, martini/martini.py:939-1105)
written without astropy: standard 2880-byte blocks, the reference's header
cards, and the data with NAXIS1 = RA varying fastest (the reference writes
the cube transposed)."""

import os

import numpy as np


def _martini(tmpdir_beam=True):
    from martini_gb300 import DataCube, Martini, SPHSource
    from martini_gb300 import spectral_models as S
    from martini_gb300 import sph_kernels as K
    from martini_gb300 import workloads as W
    from martini_gb300.beams import GaussianBeam
    g = W.disc(2000, 4)
    xyz, vxyz = W.incline(g["xyz"], g["vxyz"], 40.0)
    src = SPHSource(distance=3.0, ra=30.0, dec=-10.0, T_g=g["T"], mHI_g=g["mHI"], xyz_g=xyz,
                    vxyz_g=vxyz, hsm_g=g["hsm"])
    dc = DataCube(n_px_x=20, n_px_y=16, n_channels=12, px_size=10.0, channel_width=4.0,
                  spectral_centre=src.vsys, ra=30.0, dec=-10.0)
    return Martini(source=src, datacube=dc, beam=GaussianBeam(bmaj=25.0) if tmpdir_beam else None,
                   sph_kernel=K.CubicSplineKernel(), spectral_model=S.GaussianSpectrum(7.0),
                   quiet=True)


def test_write_fits_header_and_axis_order(tmp_path):
    from martini_gb300.fits import BLOCK, read_primary
    m = _martini()
    dc = m.datacube
    rng = np.random.default_rng(0)
    dc._array = rng.random(dc._array.shape)
    dc._array_unit = "Jy/beam"
    unpadded = dc._array[dc.padx:dc._array.shape[0] - dc.padx,
                         dc.pady:dc._array.shape[1] - dc.pady].copy()
    fn = str(tmp_path / "cube")
    m.write_fits(fn, obj_name="TESTGALAXY")
    path = fn + ".fits"
    assert os.path.getsize(path) % BLOCK == 0
    hdr, data = read_primary(path)
    assert hdr["SIMPLE"] is True and hdr["BITPIX"] == -64 and hdr["NAXIS"] == 3
    assert (hdr["NAXIS1"], hdr["NAXIS2"], hdr["NAXIS3"]) == (20, 16, 12)
    assert hdr["CTYPE1"] == "RA---TAN" and hdr["CTYPE2"] == "DEC--TAN" and hdr["CTYPE3"] == "VRAD"
    assert hdr["CUNIT3"] == "m/s" and hdr["CDELT3"] == -4000.0
    assert abs(hdr["CDELT1"] + 10.0 / 3600) < 1e-15 and hdr["CRPIX1"] == 10.5
    assert hdr["CRVAL1"] == 30.0 and hdr["CRVAL2"] == -10.0
    assert hdr["BUNIT"] == "Jy/beam" and hdr["OBJECT"] == "TESTGALAXY"
    assert abs(hdr["BMAJ"] - 25.0 / 3600) < 1e-15 and hdr["RESTFRQ"] == 1420405751.768
    assert hdr["DATAMAX"] == unpadded.max()
    # data[c][j][i] == cube[i][j][c]
    np.testing.assert_array_equal(data, unpadded.T)


def test_write_beam_fits(tmp_path):
    from martini_gb300.fits import read_primary
    m = _martini()
    fn = str(tmp_path / "beam")
    m.write_beam_fits(fn)
    hdr, data = read_primary(fn + ".fits")
    k = m.beam.kernel
    assert data.shape == (1, k.shape[1], k.shape[0])
    np.testing.assert_array_equal(data[0], k.T)
    assert hdr["OBJECT"] == "MOCKBEAM" and hdr["CRPIX1"] == k.shape[0] // 2 + 1


def test_write_fits_float32(tmp_path):
    from martini_gb300.fits import read_primary
    m = _martini(tmpdir_beam=False)
    m.datacube._array = np.arange(np.prod(m.datacube._array.shape), dtype=np.float64).reshape(
        m.datacube._array.shape)
    fn = str(tmp_path / "c32.fits")
    m.write_fits(fn, dtype=np.float32)
    hdr, data = read_primary(fn)
    assert hdr["BITPIX"] == -32
    np.testing.assert_array_equal(data, m.datacube._array.T.astype(np.float32))
