"""GPU set-up (mg_setup) against the host set-up of the drop-in classes.

The host path (SPHSource._init_skycoords / _init_pixcoords, the kernel's
_init_sm_lengths / _init_sm_ranges, Martini._prune_particles) follows the
reference in FP64 numpy; mg_setup does the same per particle in FP64 on the
GPU.  Both must keep the same particles in the same order with the same
integer footprint ranges and kernel choices, pixel coordinates and
velocities to 1e-9, and give the same cube when inserted.
"""

import numpy as np
import pytest
import torch

from oracle import martini_oracle as orc

pytestmark = pytest.mark.gpu


def _source(n, seed, T=True):
    from martini_gb300 import SPHSource
    from martini_gb300 import workloads as W
    g = W.disc(n, seed, h_med=0.8, h_dex=0.4)
    xyz, vxyz = W.incline(g["xyz"], g["vxyz"], 55.0)
    return SPHSource(distance=4.0, vpeculiar=30.0, ra=15.0, dec=-30.0, T_g=g["T"] if T else None,
                     mHI_g=g["mHI"], xyz_g=xyz, vxyz_g=vxyz, hsm_g=g["hsm"])


CASES = {
    "vrad_adaptive_thermal_pad": dict(freq=False, kernel="WendlandC2Kernel", spec="thermal", pad=3),
    "freq_single_cubic_fixed": dict(freq=True, kernel="_CubicSplineKernel", spec=8.0, pad=0),
    "vrad_adaptive_c6_dirac": dict(freq=False, kernel="WendlandC6Kernel", spec="dirac", pad=0),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_gpu_setup_matches_host_setup(case):
    from martini_gb300 import DataCube
    from martini_gb300 import sph_kernels as K
    from martini_gb300 import spectral_models as S
    from martini_gb300 import units as u
    from martini_gb300.engine import InsertionEngine, setup_on_gpu
    from martini_gb300.martini import _BaseMartini
    c = CASES[case]
    n = 20000

    def make():
        src = _source(n, 11, T=c["spec"] == "thermal")
        if c["freq"]:
            dc = DataCube(n_px_x=96, n_px_y=80, n_channels=48, px_size=12.0,
                          channel_width=4.0 * 1420405751.768 / 299792.458, freq_channels=True,
                          spectral_centre=float(u.radio_frequency_hz(src.vsys)), ra=15.0,
                          dec=-30.0)
        else:
            dc = DataCube(n_px_x=96, n_px_y=80, n_channels=48, px_size=12.0, channel_width=4.0,
                          spectral_centre=src.vsys, ra=15.0, dec=-30.0)
        if c["pad"]:
            dc.add_pad((c["pad"], c["pad"]))
        kern = getattr(K, c["kernel"])()
        sm = (S.DiracDeltaSpectrum() if c["spec"] == "dirac" else S.GaussianSpectrum(c["spec"]))
        return src, dc, kern, sm

    # host path, as Martini.__init__
    src, dc, kern, sm = make()
    m = _BaseMartini.__new__(_BaseMartini)
    m.quiet, m.source, m._datacube, m.sph_kernel, m.spectral_model = True, src, dc, kern, sm
    src._init_skycoords()
    src._init_pixcoords(dc)
    kern._init_sm_lengths(source=src, datacube=dc)
    kern._init_sm_ranges()
    m._prune_particles()
    h_eff, kidx = kern._device_arrays()
    sig, sig_const = sm._device_sigma(src)
    amp = src.mHI_g * np.power(src.skycoords.distance, -2.0) / orc.MHI_TO_JY

    # GPU path from a fresh, unpruned source
    src2, dc2, kern2, sm2 = make()
    eng = InsertionEngine("cuda:0")
    parts, table, model, sconst = setup_on_gpu(eng, src2, dc2, kern2, sm2)
    assert parts.n == src.npart
    np.testing.assert_allclose(parts.x.cpu().numpy(), src.pixcoords[0], rtol=0, atol=1e-9)
    np.testing.assert_allclose(parts.y.cpu().numpy(), src.pixcoords[1], rtol=0, atol=1e-9)
    np.testing.assert_allclose(parts.v.cpu().numpy(), src.skycoords.radial_velocity, rtol=0,
                               atol=1e-9)
    np.testing.assert_array_equal(parts.sm_range.cpu().numpy(), kern.sm_ranges)
    np.testing.assert_allclose(parts.h_eff.cpu().numpy(), h_eff.astype(np.float32), rtol=2e-7)
    if kidx is None:
        assert parts.kernel_index is None
    else:
        np.testing.assert_array_equal(parts.kernel_index.cpu().numpy(), kidx)
    np.testing.assert_allclose(parts.amp.cpu().numpy(), amp, rtol=1e-12)
    if sig is not None:
        np.testing.assert_allclose(parts.sigma.cpu().numpy(), sig, rtol=2e-7)
    assert table == kern._device_kernels() and model == sm.native_model
    assert sconst == sig_const

    # same cube from either set-up
    edges = torch.from_numpy(np.ascontiguousarray(dc.velocity_channel_edges)).to(eng.device)
    nx, ny = dc._array.shape[:2]
    from martini_gb300.engine import DeviceParticles
    hp = DeviceParticles.from_host(eng.device, src.pixcoords[0], src.pixcoords[1],
                                   kern.sm_ranges, h_eff, kidx, v=src.skycoords.radial_velocity,
                                   sigma=sig, amp=amp)
    ref, _ = eng.insert(hp, table, model, sig_const, nx, ny, dc.n_channels, edges,
                        padx=dc.padx, pady=dc.pady)
    got, _ = eng.insert(parts, table, model, sconst, nx, ny, dc.n_channels, edges,
                        padx=dc.padx, pady=dc.pady)
    ref, got = ref.cpu().numpy(), got.cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-6 * np.abs(ref).max()
