"""Beam convolution (Martini.convolve_beam, martini/martini.py:863-901;
beam image martini/beams.py:103-160, :231-295).

CPU: the beam image integrates to ~1 and agrees with direct 2D quadrature
of the beam over pixels.  GPU: mg_convolve_beam equals scipy's fftconvolve
of each channel ("same" mode, the reference's call), pad dropped and scaled
by the beam area, for the shared-memory path and the large-beam path, and
through the Martini API.
"""

import numpy as np
import pytest
from scipy import integrate
from scipy.signal import fftconvolve


def _beam(bmaj=30.0, bmin=20.0, bpa=30.0, px=10.0):
    from martini_gb300 import DataCube
    from martini_gb300.beams import GaussianBeam
    b = GaussianBeam(bmaj=bmaj, bmin=bmin, bpa=bpa)
    b.init_kernel(DataCube(n_px_x=16, n_px_y=16, n_channels=4, px_size=px, channel_width=4.0))
    return b


def test_beam_image_normalised_and_matches_quadrature():
    b = _beam()
    k = b.kernel
    n = k.shape[0]
    assert k.shape == (n, n) and n % 2 == 1
    assert b.needs_pad() == (n // 2, n // 2)
    assert abs(k.sum() - 1.0) < 1e-4
    f = b.f_kernel()
    h = n // 2
    for (r, c) in [(h, h), (h + 1, h), (h, h + 2), (h - 2, h + 1)]:
        # image rows run along y, columns along x (the reference's meshgrid)
        x0, x1 = (c - h - 0.5) * b.px_size, (c - h + 0.5) * b.px_size
        y0, y1 = (r - h - 0.5) * b.px_size, (r - h + 0.5) * b.px_size
        val, _ = integrate.dblquad(lambda y, x: f(x, y), x0, x1, y0, y1, epsabs=1e-12)
        assert abs(k[r, c] - val) <= 1e-6 * k.max()


def _gpu_conv(cube, pad, kern, scale):
    import torch
    from martini_gb300.engine import InsertionEngine, convolve_beam
    eng = InsertionEngine("cuda:0")
    t = torch.from_numpy(cube.astype(np.float32)).to(eng.device)
    return convolve_beam(eng, t, pad[0], pad[1], kern, scale).cpu().numpy()


def _ref_conv(cube, pad, kern, scale):
    out = np.stack([fftconvolve(cube[..., c], kern, mode="same")
                    for c in range(cube.shape[2])], axis=2)
    return out[pad[0]:cube.shape[0] - pad[0], pad[1]:cube.shape[1] - pad[1]] * scale


@pytest.mark.gpu
@pytest.mark.parametrize("shape,kshape", [((60, 52, 40), (7, 9)), ((70, 64, 33), (27, 27)),
                                          ((150, 140, 5), (61, 61))],
                         ids=["small", "beam27", "large_direct"])
def test_convolution_matches_fftconvolve(shape, kshape):
    rng = np.random.default_rng(1)
    cube = rng.random(shape)
    cube[rng.random(shape) < 0.7] = 0.0
    kern = rng.random(kshape)
    kern /= kern.sum()
    pad = (kshape[0] // 2, kshape[1] // 2)
    got = _gpu_conv(cube, pad, kern, 3.5)
    ref = _ref_conv(cube.astype(np.float32).astype(np.float64), pad,
                    kern.astype(np.float32).astype(np.float64), 3.5)
    assert got.shape == ref.shape
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()


@pytest.mark.gpu
def test_martini_convolve_beam_end_to_end():
    from martini_gb300 import DataCube, Martini, SPHSource
    from martini_gb300 import spectral_models as S
    from martini_gb300 import sph_kernels as K
    from martini_gb300 import workloads as W
    from martini_gb300.beams import GaussianBeam
    g = W.disc(5000, 8)
    xyz, vxyz = W.incline(g["xyz"], g["vxyz"], 50.0)
    src = SPHSource(distance=3.0, T_g=g["T"], mHI_g=g["mHI"], xyz_g=xyz, vxyz_g=vxyz,
                    hsm_g=g["hsm"])
    dc = DataCube(n_px_x=48, n_px_y=48, n_channels=32, px_size=10.0, channel_width=4.0,
                  spectral_centre=src.vsys)
    beam = GaussianBeam(bmaj=30.0, bmin=30.0)
    m = Martini(source=src, datacube=dc, beam=beam, sph_kernel=K.CubicSplineKernel(),
                spectral_model=S.GaussianSpectrum(7.0), quiet=True)
    m.insert_source_in_cube()
    padded = m.datacube._array.copy()
    pad = (m.datacube.padx, m.datacube.pady)
    m.convolve_beam()
    got = m.datacube._array
    assert m.datacube._array_unit == "Jy/beam" and got.shape == (48, 48, 32)
    ref = _ref_conv(padded.astype(np.float32).astype(np.float64), pad,
                    beam.kernel.astype(np.float32).astype(np.float64), beam.area)
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()
