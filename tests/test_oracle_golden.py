"""The FP64 oracle against golden vectors from the reference's own code and
against the reference test-suite's known answers (CPU only)."""

import glob
import os

import numpy as np
import pytest

from oracle import martini_oracle as orc
from tests.helpers import golden_cases

GOLD = os.path.join(os.path.dirname(__file__), "golden")

KERNEL_KEYS = {
    "_WendlandC2Kernel": (orc.KT_WENDLAND_C2, 0.0),
    "_WendlandC6Kernel": (orc.KT_WENDLAND_C6, 0.0),
    "_CubicSplineKernel": (orc.KT_CUBIC_SPLINE, 0.0),
    "_QuarticSplineKernel": (orc.KT_QUARTIC_SPLINE, 0.0),
    "_GaussianKernel_2": (orc.KT_GAUSSIAN, 2.0),
    "_GaussianKernel_3": (orc.KT_GAUSSIAN, 3.0),
    "_GaussianKernel_4": (orc.KT_GAUSSIAN, 4.0),
    "_GaussianKernel_5": (orc.KT_GAUSSIAN, 5.0),
    "_GaussianKernel_6": (orc.KT_GAUSSIAN, 6.0),
    "DiracDeltaKernel": (orc.KT_DIRAC, 0.0),
}


@pytest.fixture(scope="module")
def kv():
    return np.load(os.path.join(GOLD, "kernel_vectors.npz"))


@pytest.mark.parametrize("key", sorted(KERNEL_KEYS))
def test_kernel_integral_matches_reference(kv, key):
    kt, trunc = KERNEL_KEYS[key]
    kc = orc.kernel_constants(kt, trunc if trunc else 3.0)
    dij = np.vstack((kv["dx"], kv["dy"]))
    w = orc.kernel_integral(kc, dij, kv["h"].copy())
    ref = kv["w_" + key]
    scale = np.abs(ref).max()
    np.testing.assert_allclose(w, ref, rtol=1e-12, atol=1e-14 * scale)


@pytest.mark.parametrize("key", sorted(KERNEL_KEYS))
def test_kernel_constants_match_reference(kv, key):
    kt, trunc = KERNEL_KEYS[key]
    kc = orc.kernel_constants(kt, trunc if trunc else 3.0)
    assert kc["size_in_fwhm"] == pytest.approx(float(kv["size_" + key]), rel=1e-14)
    assert kc["rescale"] == pytest.approx(float(kv["rescale_" + key]), rel=1e-14)


@pytest.mark.parametrize("name", ["WendlandC2Kernel", "WendlandC6Kernel", "CubicSplineKernel",
                                  "QuarticSplineKernel", "GaussianKernel"])
def test_adaptive_selection_matches_reference(kv, name):
    h = kv["sel_h"]
    idx, size, resc = orc.select_kernels(orc.adaptive_tuple(name), h)
    np.testing.assert_array_equal(idx, kv["sel_idx_" + name])
    np.testing.assert_allclose(size, kv["sel_size_" + name], rtol=1e-15)
    np.testing.assert_allclose(resc, kv["sel_rescale_" + name], rtol=1e-15)
    np.testing.assert_array_equal(orc.sm_ranges(h, size), kv["sel_ranges_" + name])


def test_adaptive_selection_known_answer():
    """tests/test_sph_kernels.py:293-334: h = (3, 1, 0.55, 0.1) px."""
    h = np.array([3.0, 1.0, 0.55, 0.1])
    for name in ("WendlandC2Kernel", "WendlandC6Kernel", "CubicSplineKernel",
                 "QuarticSplineKernel"):
        idx, _, _ = orc.select_kernels(orc.adaptive_tuple(name), h)
        assert list(idx) == [0, 0, 2, 1]
    idx, _, _ = orc.select_kernels(orc.adaptive_tuple("GaussianKernel", 3.0), h)
    assert list(idx) == [0, 2, 2, 1]


def test_thermal_sigma_known_answer():
    """tests/test_spectral_models.py:43-48."""
    assert orc.thermal_sigma_kms(np.array([1e4]))[0] == pytest.approx(9.0853727258, rel=1e-10)


@pytest.mark.parametrize("tag", ["vrad", "incr", "freq"])
@pytest.mark.parametrize("model", ["gaussian", "dirac"])
def test_spectra_match_reference(tag, model):
    sv = np.load(os.path.join(GOLD, "spectra_vectors.npz"))
    sig = orc.thermal_sigma_kms((sv[f"sigma_{tag}"] * 1e3) ** 2 * orc.M_P / orc.K_B)
    s = orc.init_spectra(model, sv[f"mHI_{tag}"], sv[f"dist_{tag}"], sv[f"v_{tag}"],
                         sv[f"edges_{tag}"], sig)
    ref = sv[f"{model}_{tag}"]
    np.testing.assert_allclose(s, ref, rtol=1e-12, atol=1e-15 * np.abs(ref).max())


def test_spectrum_flux_known_answer():
    """tests/test_spectral_models.py:16-33, :101-119: flux = mHI / 2.36e5 at 1 Mpc."""
    edges = orc.vrad_channel_edges(64, 4.0, 210.0)
    for model, sig in (("gaussian", 7.0), ("gaussian", orc.thermal_sigma_kms(1e4)),
                       ("dirac", None)):
        s = orc.init_spectra(model, np.array([1e4]), np.array([1.0]), np.array([210.3]),
                             edges, None if sig is None else np.array([sig]))
        assert s[0].sum() * 4.0 == pytest.approx(1e4 / 2.36e5, rel=1e-5)
    # a Dirac line exactly on a channel edge lands in both channels (H(0) = 1)
    s = orc.init_spectra("dirac", np.array([1e4]), np.array([1.0]), np.array([210.0]), edges)
    assert s[0].sum() * 4.0 == pytest.approx(2 * 1e4 / 2.36e5, rel=1e-12)


def test_channel_edges_nonmonotonic_raises():
    with pytest.raises(ValueError, match="not monotonic"):
        orc.channel_bounds(np.array([1.0, 2.0, 1.5]))


def _pipeline(d):
    """Run the oracle on a golden case's inputs, as the reference does."""
    kname = str(d["kernel"])
    karg = float(d["kernel_arg"])
    if kname.startswith("_") or kname == "DiracDeltaKernel":
        kt = {"_WendlandC2Kernel": orc.KT_WENDLAND_C2, "_WendlandC6Kernel": orc.KT_WENDLAND_C6,
              "_CubicSplineKernel": orc.KT_CUBIC_SPLINE,
              "_QuarticSplineKernel": orc.KT_QUARTIC_SPLINE,
              "_GaussianKernel": orc.KT_GAUSSIAN, "DiracDeltaKernel": orc.KT_DIRAC}[kname]
        kernels = orc.simple_tuple(kt, karg if np.isfinite(karg) else 3.0)
    else:
        kernels = orc.adaptive_tuple(kname, karg if np.isfinite(karg) else 3.0)
    h = d["h_px"]
    kidx, size, resc = orc.select_kernels(kernels, h)
    ranges = orc.sm_ranges(h, size)
    spectral = str(d["spectral"])
    if spectral == "gaussian":
        sig = (orc.thermal_sigma_kms(d["T"]) if d["T"].size else d["sigma"])
        hw = sig
    else:
        sig = None
        hw = 0.0
    pad = int(d["pad"])
    nx, ny, nc = int(d["nx"]), int(d["ny"]), int(d["nc"])
    keep = orc.prune_mask(d["x"], d["y"], d["vchan"], ranges, d["mHI"], nx + 2 * pad,
                          ny + 2 * pad, nc, hw, d["edges"])
    sl = lambda a: a[keep] if np.ndim(a) else a  # noqa: E731
    spectra = orc.init_spectra(spectral, d["mHI"][keep], d["dist"][keep], d["v"][keep],
                               d["edges"], None if sig is None else sl(sig))
    args = (d["x"][keep], d["y"][keep], ranges[keep], kernels, kidx[keep], (h * resc)[keep],
            spectra)
    return keep, spectra, args, (nx + 2 * pad, ny + 2 * pad)


CASES = sorted(os.path.basename(p)[5:-4] for p in glob.glob(os.path.join(GOLD, "cube_*.npz")))


@pytest.mark.parametrize("case", CASES)
def test_cube_matches_reference(case):
    d = np.load(os.path.join(GOLD, f"cube_{case}.npz"))
    keep, spectra, args, (nx, ny) = _pipeline(d)
    assert keep.sum() == int(d["n_after"])
    np.testing.assert_array_equal(args[0], d["kept_x"])
    np.testing.assert_allclose(spectra, d["spectra"], rtol=1e-12,
                               atol=1e-15 * np.abs(d["spectra"]).max())
    ref = d["cube"]
    peak = np.abs(ref).max()
    scat = orc.insert_scatter(nx, ny, *args)
    np.testing.assert_allclose(scat, ref, rtol=0, atol=1e-12 * peak)
    if nx * ny <= 400:
        pp = orc.insert_perpixel(nx, ny, *args)
        np.testing.assert_allclose(pp, ref, rtol=0, atol=1e-13 * peak)


def test_pixcoords_known_answer():
    """tests/test_sources.py:335-380: particles 1 kpc apart at the distance
    where 1 kpc subtends 1 arcsec land on integer pixels."""
    D = 1e-3 / np.deg2rad(1 / 3600.0)  # Mpc
    yz = np.linspace(-2.5, 2.5, 6)
    xyz = np.vstack((np.zeros(6), yz, yz)).T
    vxyz = np.vstack((np.linspace(-2.5, 2.5, 6), np.zeros(6), np.zeros(6))).T
    ra, dec, v, _ = orc.project_particles(xyz, vxyz, D, h=0.0)
    px = 1.0 / 3600.0
    x, y = orc.tan_world2pix(ra, dec, 0.0, 0.0, 3.5, 3.5, -px, px)
    vchan = (6 / 2 + 0.5 - 1) + (v - 0.0) / (-1.0)
    np.testing.assert_allclose(x, np.arange(6)[::-1], atol=1e-4)
    np.testing.assert_allclose(y, np.arange(6), atol=1e-4)
    np.testing.assert_allclose(vchan, np.arange(6)[::-1], atol=1e-4)


def test_projection_behind_observer_is_nan():
    """tests/test_martini.py:546-584: a particle 180 deg from the cube centre."""
    ra, dec, v, _ = orc.project_particles(np.array([[0.0, 0, 0], [-20e3, 0, 0]]),
                                          np.zeros((2, 3)), 10.0)
    x, y = orc.tan_world2pix(ra, dec, 180.0, 0.0, 1.5, 1.5, -1 / 360, 1 / 360)
    assert np.isnan(x[0]) and np.isnan(y[0])
    assert np.isfinite(x[1]) and np.isfinite(y[1])


@pytest.mark.parametrize("case", golden_cases())
def test_c_flux_total_matches_golden_cube(case):
    """The per-particle FP64 flux total in C (sum_p (sum_box W_p) sum_c S_p)
    equals the sum of the reference-generated cube over its unpadded pixels,
    and its spectrum sums equal the reference's init_spectra row sums."""
    from tests.helpers import case_inputs, load_case
    d = load_case(case)
    c = case_inputs(d)
    sig = c["sigma"] if c["spectral"] == "gaussian" else None
    ss = orc.spectrum_sums(c["spectral"], c["v"], sig, c["amp"], c["edges"])
    sp = orc.init_spectra(c["spectral"], c["mHI"], c["dist"], c["v"], c["edges"], sig)
    np.testing.assert_allclose(ss, sp.sum(axis=1), rtol=1e-12, atol=1e-15 * np.abs(ss).max())
    tot = orc.flux_total(c["x"], c["y"], c["ranges"], c["kernels"], c["kidx"], c["h_eff"], ss,
                         c["nx"], c["ny"], c["pad"], c["pad"])
    ref = d["cube"]
    pad = c["pad"]
    expect = ref[pad:ref.shape[0] - pad, pad:ref.shape[1] - pad].sum()
    assert abs(tot - expect) <= 1e-11 * abs(expect)
