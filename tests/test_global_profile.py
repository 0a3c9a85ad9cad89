"""GlobalProfile: the spatially integrated spectrum (martini/martini.py:1369-1738).

The reference inserts every particle in the band into a one-pixel cube with
an infinite-range DiracDeltaKernel, so the spectrum is the sum of the
particles' channel spectra.  Checked against the oracle's spectra, against
the one-pixel cube through mg_insert (the reference's own construction),
and for mass recovery (tests/test_martini.py requires the mass within 1 %).
"""

import numpy as np
import pytest

from oracle import martini_oracle as orc


def _profile(spec, n=20000, seed=3):
    from martini_gb300 import GlobalProfile, SPHSource
    from martini_gb300 import spectral_models as S
    from martini_gb300 import workloads as W
    g = W.disc(n, seed)
    xyz, vxyz = W.incline(g["xyz"], g["vxyz"], 60.0)
    src = SPHSource(distance=3.0, T_g=g["T"], mHI_g=g["mHI"], xyz_g=xyz, vxyz_g=vxyz,
                    hsm_g=g["hsm"])
    sm = S.DiracDeltaSpectrum() if spec == "dirac" else S.GaussianSpectrum(spec)
    return GlobalProfile(source=src, spectral_model=sm, n_channels=160, channel_width=4.0,
                         spectral_centre=src.vsys, quiet=True)


def test_profile_setup_keeps_every_particle_in_the_band():
    m = _profile(7.0)
    src = m.source
    # no spatial pruning: every particle is kept unless it is out of band
    assert src.npart > 0.99 * 20000
    assert np.all(src.pixcoords[:2] == 0)
    edges = m.velocity_channel_edges
    assert edges.shape == (161,) and np.all(np.diff(edges) < 0)
    np.testing.assert_allclose(m.velocity_channel_mids, 0.5 * (edges[1:] + edges[:-1]))


@pytest.mark.gpu
@pytest.mark.parametrize("spec", [7.0, "thermal", "dirac"])
def test_profile_matches_oracle_and_one_pixel_cube(spec):
    import torch
    from martini_gb300 import _native as N
    from martini_gb300.engine import DeviceParticles, InsertionEngine
    m = _profile(spec)
    got = m.spectrum
    src = m.source
    model = "dirac" if spec == "dirac" else "gaussian"
    sig = (orc.thermal_sigma_kms(src.T_g) if spec == "thermal"
           else np.full(src.npart, 7.0) if model == "gaussian" else None)
    edges = m.velocity_channel_edges
    ref = orc.init_spectra(model, src.mHI_g, src.skycoords.distance,
                           src.skycoords.radial_velocity, edges, sig).sum(axis=0)
    peak = np.abs(ref).max()
    assert np.abs(got - ref).max() <= 1e-5 * peak
    assert abs(got.sum() - ref.sum()) <= 1e-6 * ref.sum()
    # the reference's construction: a 1 x 1 cube, DiracDeltaKernel of infinite range
    eng = InsertionEngine("cuda:0")
    n = src.npart
    zeros = np.zeros(n)
    parts = DeviceParticles.from_host(eng.device, zeros, zeros, np.full(n, np.inf),
                                      np.ones(n, np.float32), None,
                                      v=src.skycoords.radial_velocity,
                                      sigma=None if sig is None else sig.astype(np.float32),
                                      amp=src.mHI_g / src.skycoords.distance**2 / orc.MHI_TO_JY)
    smodel = N.MG_SPECTRUM_DIRAC if model == "dirac" else N.MG_SPECTRUM_GAUSSIAN
    cube, _ = eng.insert(parts, [(N.MG_KERNEL_DIRAC, 0.0)], smodel, 0.0, 1, 1, 160,
                         torch.from_numpy(np.ascontiguousarray(edges)).to(eng.device))
    one = cube.cpu().numpy()[0, 0].astype(np.float64)
    assert np.abs(one - got).max() <= 1e-5 * peak


@pytest.mark.gpu
def test_profile_recovers_the_source_mass():
    m = _profile(7.0)
    spec = m.spectrum
    src = m.source
    mass = orc.MHI_TO_JY * src.distance**2 * spec.sum() * 4.0
    assert abs(mass - src.input_mass) / src.input_mass < 0.01
