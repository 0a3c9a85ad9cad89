"""Host-side set-up of the drop-in API (projection, kernel selection,
pruning, channel grid) against the oracle's restatement (CPU only)."""

import numpy as np
import pytest

from martini_gb300 import DataCube, SPHSource
from martini_gb300.martini import _BaseMartini
from martini_gb300 import sph_kernels as K
from martini_gb300 import spectral_models as S
from oracle import martini_oracle as orc


def disc_source(n=2000, seed=3, D=3.0, incl=60.0, **kw):
    g = orc.disc_particles(n, seed=seed, **kw)
    xyz, vxyz = orc.incline(g["xyz"], g["vxyz"], incl)
    return g, xyz, vxyz, SPHSource(distance=D, T_g=g["T"], mHI_g=g["mHI"], xyz_g=xyz,
                                    vxyz_g=vxyz, hsm_g=g["hsm"])


class _NoGPU(_BaseMartini):
    """_BaseMartini set-up only (no insertion)."""


@pytest.mark.parametrize("ra,dec", [(0.0, 0.0), (30.0, -30.0), (200.0, 45.0)])
def test_pixcoords_match_oracle(ra, dec):
    g, xyz, vxyz, _ = disc_source()
    src = SPHSource(distance=3.0, ra=ra, dec=dec, T_g=g["T"], mHI_g=g["mHI"], xyz_g=xyz,
                    vxyz_g=vxyz, hsm_g=g["hsm"], vpeculiar=50.0)
    dc = DataCube(n_px_x=64, n_px_y=48, n_channels=32, px_size=10.0, channel_width=4.0,
                  spectral_centre=src.vsys, ra=ra, dec=dec)
    src._init_skycoords()
    src._init_pixcoords(dc)
    ra_p, dec_p, v, d = orc.project_particles(xyz, vxyz, 3.0, ra, dec, 0.7, 50.0)
    x, y = orc.tan_world2pix(ra_p, dec_p, ra, dec, 32.5, 24.5, -10 / 3600, 10 / 3600)
    vchan = 15.5 + (v - src.vsys) / -4.0
    np.testing.assert_allclose(src.pixcoords[0], x, atol=1e-9)
    np.testing.assert_allclose(src.pixcoords[1], y, atol=1e-9)
    np.testing.assert_allclose(src.pixcoords[2], vchan, atol=1e-9)
    np.testing.assert_allclose(src.skycoords.radial_velocity, v, rtol=1e-13)


def test_pixcoords_known_answer():
    """tests/test_sources.py:335-380 of the reference."""
    D = 1e-3 / np.deg2rad(1 / 3600.0)
    yz = np.linspace(-2.5, 2.5, 6)
    src = SPHSource(distance=D, h=0.0, T_g=np.ones(6) * 1e4, mHI_g=np.ones(6) * 1e4,
                    xyz_g=np.vstack((np.zeros(6), yz, yz)).T,
                    vxyz_g=np.vstack((np.linspace(-2.5, 2.5, 6), np.zeros(6), np.zeros(6))).T,
                    hsm_g=np.ones(6))
    dc = DataCube(n_px_x=6, n_px_y=6, n_channels=6, px_size=1.0, channel_width=1.0)
    src._init_skycoords()
    src._init_pixcoords(dc)
    exp = np.vstack((np.arange(6)[::-1], np.arange(6), np.arange(6)[::-1]))
    np.testing.assert_allclose(src.pixcoords, exp, atol=1e-4)


def test_channel_edges():
    dc = DataCube(n_px_x=4, n_px_y=4, n_channels=16, px_size=15.0, channel_width=4.0,
                  spectral_centre=210.0)
    np.testing.assert_allclose(dc.velocity_channel_edges, orc.vrad_channel_edges(16, 4.0, 210.0))
    dcf = DataCube(n_px_x=4, n_px_y=4, n_channels=16, px_size=15.0, channel_width=20e3,
                   spectral_centre=1.4194e9, freq_channels=True)
    np.testing.assert_allclose(dcf.velocity_channel_edges,
                               orc.freq_channel_edges(16, 20e3, 1.4194e9), rtol=1e-14)


@pytest.mark.parametrize("name", ["WendlandC2Kernel", "WendlandC6Kernel", "CubicSplineKernel",
                                  "QuarticSplineKernel", "GaussianKernel"])
def test_kernel_setup_matches_oracle(name):
    g, xyz, vxyz, src = disc_source(h_med=0.3, h_dex=0.6)
    dc = DataCube(n_px_x=64, n_px_y=64, n_channels=32, px_size=10.0, channel_width=4.0,
                  spectral_centre=src.vsys)
    k = getattr(K, name)()
    src._init_skycoords()
    src._init_pixcoords(dc)
    k._init_sm_lengths(src, dc)
    k._init_sm_ranges()
    ra, dec, v, d = orc.project_particles(xyz, vxyz, 3.0)
    hpx = orc.sm_lengths_px(g["hsm"], d, 10.0)
    np.testing.assert_allclose(k.sm_lengths, hpx, rtol=1e-14)
    idx, size, resc = orc.select_kernels(orc.adaptive_tuple(name), hpx)
    np.testing.assert_array_equal(k.kernel_indices, idx)
    np.testing.assert_array_equal(k.sm_ranges, orc.sm_ranges(hpx, size))
    np.testing.assert_allclose(k._rescale, resc, rtol=1e-15)
    assert set(np.unique(idx)) >= {0, 1, 2}


def test_adaptive_known_answer():
    src = SPHSource(distance=3.0, mHI_g=np.ones(4) * 1e4, xyz_g=np.ones((4, 3)) * 1e-3,
                    vxyz_g=np.zeros((4, 3)), hsm_g=np.array([3.0, 1.0, 0.55, 0.1]))
    px = np.rad2deg(np.arctan(1.0 / 3000.0)) * 3600  # 1 kpc pixels at 3 Mpc
    dc = DataCube(n_px_x=10, n_px_y=10, n_channels=8, px_size=px, channel_width=4.0)
    src._init_skycoords()
    for cls in (K.WendlandC2Kernel, K.WendlandC6Kernel, K.CubicSplineKernel,
                K.QuarticSplineKernel):
        k = cls()
        k._init_sm_lengths(src, dc)
        assert list(k.kernel_indices) == [0, 0, 2, 1]
    k = K.GaussianKernel(truncate=3.0)
    k._init_sm_lengths(src, dc)
    assert list(k.kernel_indices) == [0, 2, 2, 1]


@pytest.mark.parametrize("spectral", ["gaussian", "dirac", "thermal"])
def test_pruning_matches_oracle(spectral):
    g, xyz, vxyz, src = disc_source(n=3000)
    dc = DataCube(n_px_x=32, n_px_y=32, n_channels=16, px_size=10.0, channel_width=4.0,
                  spectral_centre=src.vsys)
    sm = {"gaussian": S.GaussianSpectrum(7.0), "dirac": S.DiracDeltaSpectrum(),
          "thermal": S.GaussianSpectrum("thermal")}[spectral]
    m = _NoGPU(source=src, datacube=dc, sph_kernel=K.CubicSplineKernel(), spectral_model=sm,
               quiet=True)
    ra, dec, v, d = orc.project_particles(xyz, vxyz, 3.0)
    x, y = orc.tan_world2pix(ra, dec, 0.0, 0.0, 16.5, 16.5, -10 / 3600, 10 / 3600)
    vchan = 7.5 + (v - 210.0) / -4.0
    hpx = orc.sm_lengths_px(g["hsm"], d, 10.0)
    _, size, _ = orc.select_kernels(orc.adaptive_tuple("CubicSplineKernel"), hpx)
    hw = {"gaussian": 7.0, "dirac": 0.0, "thermal": orc.thermal_sigma_kms(g["T"])}[spectral]
    keep = orc.prune_mask(x, y, vchan, orc.sm_ranges(hpx, size), g["mHI"], 32, 32, 16, hw,
                          dc.velocity_channel_edges)
    assert m.source.npart == keep.sum()
    np.testing.assert_allclose(m.source.pixcoords[0], x[keep], atol=1e-9)


def test_prune_all_raises():
    src = SPHSource(distance=3.0, mHI_g=np.zeros(2), xyz_g=np.zeros((2, 3)),
                    vxyz_g=np.zeros((2, 3)), hsm_g=np.ones(2))
    dc = DataCube(n_px_x=8, n_px_y=8, n_channels=8, px_size=10.0, channel_width=4.0,
                  spectral_centre=src.vsys)
    with pytest.raises(RuntimeError, match="No non-zero mHI source particles"):
        _NoGPU(source=src, datacube=dc, sph_kernel=K.CubicSplineKernel(),
               spectral_model=S.GaussianSpectrum(), quiet=True)


def test_validation_raises_like_reference():
    src = SPHSource(distance=3.0, mHI_g=np.ones(1) * 1e4, xyz_g=np.ones((1, 3)) * 1e-3,
                    vxyz_g=np.zeros((1, 3)), hsm_g=np.ones(1) * 0.2)
    dc = DataCube(n_px_x=16, n_px_y=16, n_channels=16, px_size=15.0, channel_width=4.0,
                  spectral_centre=src.vsys)
    m = _NoGPU(source=src, datacube=dc, sph_kernel=K._WendlandC2Kernel(),
               spectral_model=S.GaussianSpectrum(), quiet=True)
    with pytest.raises(RuntimeError, match="use this with care"):
        m.sph_kernel._confirm_validation(quiet=True)
    m.sph_kernel._confirm_validation(noraise=True, quiet=True)


def test_thermal_width_known_answer():
    src = SPHSource(distance=3.0, T_g=np.array([1e4]), mHI_g=np.ones(1), xyz_g=np.zeros((1, 3)),
                    vxyz_g=np.zeros((1, 3)), hsm_g=np.ones(1))
    assert S.GaussianSpectrum("thermal").half_width(src)[0] == pytest.approx(9.0853727258,
                                                                              rel=1e-10)


def test_gaussian_truncation_below_two_raises():
    with pytest.raises(RuntimeError, match="truncation <2sigma"):
        K._GaussianKernel(truncate=1.0)


def test_kernel_table_of_adaptive_and_single_kernels():
    """kernel_table maps kernel objects to the C ABI's rows, adaptive tuples in
    order (WendlandC2 -> Dirac -> Gaussian(6), sph_kernels.py:1629-1635)."""
    from martini_gb300 import _native as N
    from martini_gb300 import sph_kernels as K
    rows = N.kernel_table(K.WendlandC2Kernel())
    assert rows == [(N.MG_KERNEL_WENDLAND_C2, 0.0), (N.MG_KERNEL_DIRAC, 0.0),
                    (N.MG_KERNEL_GAUSSIAN, 6.0)]
    assert N.kernel_table(K.DiracDeltaKernel()) == [(N.MG_KERNEL_DIRAC, 0.0)]
    p = N.Problem()
    N.set_kernels(p, rows)
    assert p.n_kernels == 3 and p.kernels[2].type == N.MG_KERNEL_GAUSSIAN
    assert abs(p.kernels[2].truncate - 6.0) < 1e-6


def test_population_configs_are_seeded_and_in_range():
    """The disc population's draws (log N, cos i, v_flat, cube) are fixed by
    the seed: 2000 galaxies, 288,528,250 particles, every value in range."""
    from martini_gb300 import workloads as W
    cf = W.population_configs()
    assert len(cf) == 2000
    assert sum(c["n"] for c in cf) == 288_528_250
    assert all(1000 <= c["n"] <= 1_000_000 for c in cf)
    assert all(0.0 <= c["incl"] <= 90.0 for c in cf)
    assert all(50.0 <= c["disc"]["v_flat"] <= 300.0 for c in cf)
    assert {(c["nx"], c["nc"]) for c in cf} == set(W.POPULATION["cubes"])
    assert W.population_configs(5) == cf[:5]
    g = W.build_population(2)
    assert len(g) == 2 and all(x["n"] > 0 for x in g)


def _ref_rotmat(ra_deg, dec_deg):
    """The rotation the reference's tests expect: R_y(dec) . R_z(-ra), on
    row vectors (tests/test_sources.py:233-262)."""
    ra, dec = np.deg2rad(ra_deg), np.deg2rad(dec_deg)
    R_y = np.array([[np.cos(dec), 0, np.sin(dec)], [0, 1, 0], [-np.sin(dec), 0, np.cos(dec)]])
    R_z = np.array([[np.cos(-ra), -np.sin(-ra), 0], [np.sin(-ra), np.cos(-ra), 0], [0, 0, 1]])
    return R_y.dot(R_z)


def _sky(pos, vel):
    d = np.sqrt((pos ** 2).sum(axis=1))
    return (np.rad2deg(np.arctan2(pos[:, 1], pos[:, 0])) % 360.0,
            np.rad2deg(np.arcsin(pos[:, 2] / d)), d, (pos * vel).sum(axis=1) / d)


@pytest.mark.parametrize("ra", [0.0, 30.0, -30.0])
@pytest.mark.parametrize("dec", [0.0, 30.0, -30.0])
@pytest.mark.parametrize("distance", [0.0, 3.0])
@pytest.mark.parametrize("vpeculiar", [0.0, 100.0])
def test_sky_placement_known_answer(ra, dec, distance, vpeculiar):
    """tests/test_sources.py:268-316 (and :231-266 at distance 0, h = 0):
    positions rotate by R_y(dec) R_z(-ra), translate by the distance along
    the rotated x axis, and velocities gain the peculiar velocity along it
    and the Hubble flow h 100 km/s/Mpc times each particle's distance."""
    xyz = np.arange(1, 4, dtype=float).reshape(1, 3) * np.array([[1.0], [2.0]])
    vxyz = np.arange(1, 4, dtype=float).reshape(1, 3) * np.array([[1.0], [-1.0]])
    src = SPHSource(xyz_g=xyz, vxyz_g=vxyz, mHI_g=np.ones(2), ra=ra, dec=dec,
                    distance=distance, vpeculiar=vpeculiar)
    src._init_skycoords()
    rot = _ref_rotmat(ra, dec)
    direction = rot.T.dot(np.array([[1.0], [0.0], [0.0]]))
    pos = xyz.dot(rot) + direction.T * distance * 1e3             # kpc
    dist = np.sqrt((pos ** 2).sum(axis=1))
    vel = (vxyz.dot(rot) + pos / dist[:, None] * (0.7 * 100 * dist * 1e-3)[:, None]
           + (direction * vpeculiar).T)
    ra_e, dec_e, d_e, v_e = _sky(pos, vel)
    np.testing.assert_allclose(src.skycoords.ra, ra_e, atol=1e-9)
    np.testing.assert_allclose(src.skycoords.dec, dec_e, atol=1e-9)
    np.testing.assert_allclose(src.skycoords.distance, d_e * 1e-3, rtol=1e-12)
    np.testing.assert_allclose(src.skycoords.radial_velocity, v_e, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("ra", [0.0, 30.0, -30.0])
@pytest.mark.parametrize("dec", [0.0, 30.0, -30.0])
def test_sky_location_known_answer(ra, dec):
    """tests/test_sources.py:381-395: a particle at the origin lands at the
    source's (ra, dec); on a cube centred there (datacube.py:438-486) its
    pixel is the reference pixel, and a particle 1 kpc along +y (+RA on the
    sky, RA pixel axis decreasing) one arcsec-at-D away lands one pixel off."""
    D = 1e-3 / np.deg2rad(1 / 3600.0)  # 1 kpc subtends 1 arcsec
    src = SPHSource(xyz_g=np.array([[0.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]]),
                    vxyz_g=np.zeros((3, 3)), mHI_g=np.ones(3), ra=ra, dec=dec, distance=D, h=0.0,
                    coordinate_axis=1)
    src._init_skycoords()
    assert src.skycoords.ra[0] == pytest.approx(ra % 360.0, abs=1e-9)
    assert src.skycoords.dec[0] == pytest.approx(dec, abs=1e-9)
    dc = DataCube(n_px_x=8, n_px_y=8, n_channels=4, px_size=1.0, channel_width=1.0, ra=ra,
                  dec=dec)
    src._init_pixcoords(dc)
    np.testing.assert_allclose(src.pixcoords[:2, 0], [3.5, 3.5], atol=1e-9)
    # offsets of 1 arcsec along the source's sky axes, to TAN's second order
    np.testing.assert_allclose(src.pixcoords[:2, 1], [2.5, 3.5], atol=1e-4)
    np.testing.assert_allclose(src.pixcoords[:2, 2], [3.5, 4.5], atol=1e-4)
