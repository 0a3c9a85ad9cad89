"""GPU parity: the CUDA insertion against the reference's golden cubes and
the FP64 oracle.  Tolerances: max |cube - ref| / peak(ref) <= 1e-5 and
|flux - ref flux| / ref flux <= 1e-6 for every form that claims them: FP32,
the scaled FP16 split (f16x3) and the exact three-piece BF16 split (bf16x6).
The two-piece BF16 split (bf16x3, ~16 bits per operand) is checked against
the same bar in an expected-failure test: it meets it on most cubes but not
on every one."""

import numpy as np
import pytest
import torch

from tests.helpers import case_inputs, golden_cases, load_case, native_kernel_table
from oracle import martini_oracle as orc

pytestmark = pytest.mark.gpu

TOL_PEAK = 1e-5
TOL_FLUX = 1e-6


@pytest.fixture(scope="module")
def engine():
    from martini_gb300.engine import InsertionEngine
    return InsertionEngine("cuda:0")


def run_gpu(engine, c, form=0, plan=True):
    from martini_gb300 import _native as N
    from martini_gb300.engine import DeviceParticles
    dev = engine.device
    parts = DeviceParticles.from_host(dev, c["x"], c["y"], c["ranges"], c["h_eff"], c["kidx"],
                                      v=c["v"], sigma=c["sigma"], amp=c["amp"])
    model = N.MG_SPECTRUM_GAUSSIAN if c["spectral"] == "gaussian" else N.MG_SPECTRUM_DIRAC
    edges = torch.from_numpy(np.ascontiguousarray(c["edges"], dtype=np.float64)).to(dev)
    cube, flux = engine.insert(parts, native_kernel_table(c["kernels"]), model, 0.0, c["nx"],
                               c["ny"], c["nc"], edges, padx=c["pad"], pady=c["pad"], form=form,
                               plan=plan)
    return cube.cpu().numpy().astype(np.float64), flux.cpu().numpy()


def assert_close(got, ref, flux=None, pad=0, tol=TOL_PEAK, ftol=TOL_FLUX):
    peak = np.abs(ref).max()
    err = np.abs(got - ref).max() / peak
    assert err <= tol, f"max err / peak = {err:.3e}"
    if flux is not None:
        sl = (slice(pad, ref.shape[0] - pad), slice(pad, ref.shape[1] - pad))
        tot = ref[sl].sum()
        ferr = abs(flux[0] - tot) / tot
        assert ferr <= ftol, f"flux rel err = {ferr:.3e}"
        np.testing.assert_allclose(flux[1:], ref[sl].sum(axis=(0, 1)), rtol=1e-5,
                                   atol=1e-6 * np.abs(ref[sl].sum(axis=(0, 1))).max())


# MG_FORM_FP32, MG_FORM_F16X3, MG_FORM_BF16X6: every form held to the bar
FORMS = [0, 2, 3]
FORM_IDS = ["fp32", "f16x3", "bf16x6"]
FORM_TOL = {0: TOL_PEAK, 2: TOL_PEAK, 3: TOL_PEAK}
FLUX_TOL = {0: TOL_FLUX, 2: TOL_FLUX, 3: TOL_FLUX}
TC_FORMS = [2, 3]
TC_IDS = ["f16x3", "bf16x6"]


@pytest.mark.parametrize("form", FORMS, ids=FORM_IDS)
@pytest.mark.parametrize("case", golden_cases())
def test_golden_cube(engine, case, form):
    d = load_case(case)
    c = case_inputs(d)
    assert len(c["x"]) == int(d["n_after"])
    got, flux = run_gpu(engine, c, form=form)
    assert_close(got, d["cube"], flux, c["pad"], tol=FORM_TOL[form], ftol=FLUX_TOL[form])


@pytest.mark.xfail(strict=False, reason="the two-piece BF16 split keeps ~16 bits per operand "
                   "(up to 3 * 2^-18 = 1.1e-5 relative per term): a cube whose peak or flux "
                   "sits in a few one-particle voxels can miss 1e-5 of peak / 1e-6 of flux")
def test_golden_cubes_bf16x3_at_the_bar(engine):
    """MG_FORM_BF16X3 against every golden cube at the real bar."""
    worst = []
    for case in golden_cases():
        d = load_case(case)
        c = case_inputs(d)
        got, flux = run_gpu(engine, c, form=1)
        ref = d["cube"]
        peak = np.abs(ref).max()
        pad = c["pad"]
        tot = ref[pad:ref.shape[0] - pad, pad:ref.shape[1] - pad].sum()
        worst.append((np.abs(got - ref).max() / peak, abs(flux[0] - tot) / tot, case))
    e, f, case = max(worst)
    assert e <= TOL_PEAK, f"{case}: max err / peak {e:.3e}"
    assert max(w[1] for w in worst) <= TOL_FLUX


def test_martini_api_matches_oracle():
    """Martini(...).insert_source_in_cube() end to end against the oracle."""
    from martini_gb300 import DataCube, Martini, SPHSource
    from martini_gb300.sph_kernels import WendlandC2Kernel
    from martini_gb300.spectral_models import GaussianSpectrum
    g = orc.disc_particles(4000, seed=11, h_med=0.6)
    xyz, vxyz = orc.incline(g["xyz"], g["vxyz"], 50.0)
    src = SPHSource(distance=3.0, T_g=g["T"], mHI_g=g["mHI"], xyz_g=xyz, vxyz_g=vxyz,
                    hsm_g=g["hsm"])
    dc = DataCube(n_px_x=48, n_px_y=40, n_channels=40, px_size=10.0, channel_width=4.0,
                  spectral_centre=src.vsys)
    m = Martini(source=src, datacube=dc, sph_kernel=WendlandC2Kernel(),
                spectral_model=GaussianSpectrum(sigma="thermal"), quiet=True)
    m.insert_source_in_cube()
    k = m.sph_kernel
    spectra = orc.init_spectra("gaussian", src.mHI_g, src.skycoords.distance,
                               src.skycoords.radial_velocity, dc.velocity_channel_edges,
                               orc.thermal_sigma_kms(src.T_g))
    ref = orc.insert_scatter(48, 40, src.pixcoords[0], src.pixcoords[1], k.sm_ranges,
                             orc.adaptive_tuple("WendlandC2Kernel"), k.kernel_indices,
                             k.sm_lengths * k._rescale, spectra) / 100.0
    assert dc._array_unit == "Jy/arcsec2"
    assert_close(dc._array, ref)
    assert m.inserted_flux_density == pytest.approx(ref.sum() * 100.0, rel=TOL_FLUX)


def test_insert_accumulates_into_existing_array():
    """_array += (martini/martini.py:338): prior contents are kept."""
    from martini_gb300 import DataCube, Martini, SPHSource
    from martini_gb300.sph_kernels import CubicSplineKernel
    from martini_gb300.spectral_models import GaussianSpectrum
    g = orc.disc_particles(500, seed=2)
    src = SPHSource(distance=3.0, mHI_g=g["mHI"], xyz_g=g["xyz"], vxyz_g=g["vxyz"],
                    hsm_g=g["hsm"])
    dc = DataCube(n_px_x=16, n_px_y=16, n_channels=16, px_size=15.0, channel_width=4.0,
                  spectral_centre=src.vsys)
    m = Martini(source=src, datacube=dc, sph_kernel=CubicSplineKernel(),
                spectral_model=GaussianSpectrum(), quiet=True)
    m.insert_source_in_cube()
    once = dc._array.copy()
    f1, m1 = m.inserted_flux_density, m.inserted_mass
    m.insert_source_in_cube()
    np.testing.assert_allclose(dc._array, 2 * once, rtol=1e-12)
    # the summary sums the whole array, the first insertion included
    # (martini/martini.py:367-392)
    assert m.inserted_flux_density == pytest.approx(2 * f1, rel=1e-12)
    assert m.inserted_mass == pytest.approx(2 * m1, rel=1e-12)
    assert f1 == pytest.approx(float(m._last_flux[0]), rel=1e-6)
    m.reset()
    assert dc._array.sum() == 0
    m.insert_source_in_cube()
    np.testing.assert_allclose(dc._array, once, rtol=1e-12)


def test_spectra_materialised_match_oracle(engine):
    from martini_gb300 import _native as N
    from martini_gb300.engine import DeviceParticles
    sv = np.load("tests/golden/spectra_vectors.npz")
    for tag in ("vrad", "incr", "freq"):
        v, sig, mHI, dist = sv[f"v_{tag}"], sv[f"sigma_{tag}"], sv[f"mHI_{tag}"], sv[f"dist_{tag}"]
        edges = sv[f"edges_{tag}"]
        n = v.size
        parts = DeviceParticles.from_host(engine.device, np.zeros(n), np.zeros(n), np.ones(n),
                                          np.ones(n), None, v=v, sigma=sig,
                                          amp=mHI / dist**2 / orc.MHI_TO_JY)
        e = torch.from_numpy(edges).to(engine.device)
        for model, key in ((N.MG_SPECTRUM_GAUSSIAN, "gaussian"), (N.MG_SPECTRUM_DIRAC, "dirac")):
            got = engine.spectra(parts, model, 0.0, edges.size - 1, e).cpu().numpy()
            ref = sv[f"{key}_{tag}"]
            np.testing.assert_allclose(got, ref, rtol=0, atol=1e-6 * np.abs(ref).max())


def test_empty_and_outside(engine):
    from martini_gb300 import _native as N
    from martini_gb300.engine import DeviceParticles
    edges = torch.from_numpy(orc.vrad_channel_edges(8, 4.0, 100.0)).to(engine.device)
    for x in (np.zeros(0), np.array([-50.0, 80.0, np.nan])):
        n = x.size
        parts = DeviceParticles.from_host(engine.device, x, np.zeros(n), np.full(n, 2.0),
                                          np.full(n, 1.5), None, v=np.full(n, 100.0),
                                          sigma=np.full(n, 5.0), amp=np.ones(n))
        cube, flux = engine.insert(parts, [(N.MG_KERNEL_WENDLAND_C2, 0.0)],
                                   N.MG_SPECTRUM_GAUSSIAN, 0.0, 12, 10, 8, edges)
        assert float(cube.abs().max()) == 0.0
        assert float(flux[0]) == 0.0


def test_nonmonotonic_edges_raise(engine):
    from martini_gb300 import _native as N
    from martini_gb300.engine import DeviceParticles
    e = orc.vrad_channel_edges(8, 4.0, 100.0)
    e[4] = e[2]
    parts = DeviceParticles.from_host(engine.device, np.array([3.0]), np.array([3.0]),
                                      np.array([2.0]), np.array([1.5]), None,
                                      v=np.array([100.0]), sigma=np.array([5.0]),
                                      amp=np.array([1.0]))
    with pytest.raises(ValueError, match="not monotonic"):
        engine.insert(parts, [(N.MG_KERNEL_WENDLAND_C2, 0.0)], N.MG_SPECTRUM_GAUSSIAN, 0.0, 8, 8,
                      8, torch.from_numpy(e).to(engine.device))


def test_workspace_overflow_is_reported(engine):
    """A workspace sized for fewer pairs than the data need: no write past it,
    MG_ERR_WORKSPACE from mg_check."""
    import ctypes as C
    from martini_gb300 import _native as N
    from martini_gb300.engine import DeviceParticles
    rng = np.random.default_rng(0)
    n = 200
    parts = DeviceParticles.from_host(engine.device, rng.uniform(0, 32, n), rng.uniform(0, 32, n),
                                      np.full(n, 12.0), np.full(n, 7.0), None,
                                      v=np.full(n, 100.0), sigma=np.full(n, 5.0), amp=np.ones(n))
    edges = torch.from_numpy(orc.vrad_channel_edges(8, 4.0, 100.0)).to(engine.device)
    cube = torch.empty((32, 32, 8), dtype=torch.float32, device=engine.device)
    prob = engine.problem(parts, [(N.MG_KERNEL_WENDLAND_C2, 0.0)], N.MG_SPECTRUM_GAUSSIAN, 0.0,
                          32, 32, 8, 0, 0, edges, cube, None, N.MG_FORM_FP32)
    info = engine.plan(prob)
    small = C.c_size_t()
    N.check(engine.lib.mg_workspace_size(C.byref(prob), info.n_pairs // 2, 0, C.byref(small)))
    ws = torch.zeros(small.value, dtype=torch.uint8, device=engine.device)
    s = torch.cuda.current_stream().cuda_stream
    N.check(engine.lib.mg_insert(C.byref(prob), C.c_void_p(ws.data_ptr()), ws.numel(),
                                 info.n_pairs // 2, 0, C.c_void_p(s)))
    assert engine.lib.mg_check(C.c_void_p(ws.data_ptr()), C.c_void_p(s)) == N.MG_ERR_WORKSPACE


@pytest.mark.parametrize("form", FORMS, ids=FORM_IDS)
def test_flux_conservation_medium(engine, form):
    """A 20k-particle WendlandC2 disc on 128^2 x 64: full-cube parity."""
    rng_seed = 21
    g = orc.disc_particles(20000, seed=rng_seed, h_med=1.0)
    xyz, vxyz = orc.incline(g["xyz"], g["vxyz"], 60.0)
    ra, dec, v, d = orc.project_particles(xyz, vxyz, 3.0)
    x, y = orc.tan_world2pix(ra, dec, 0.0, 0.0, 64.5, 64.5, -10 / 3600, 10 / 3600)
    hpx = orc.sm_lengths_px(g["hsm"], d, 10.0)
    kernels = orc.adaptive_tuple("WendlandC2Kernel")
    kidx, size, resc = orc.select_kernels(kernels, hpx)
    ranges = orc.sm_ranges(hpx, size)
    edges = orc.vrad_channel_edges(64, 4.0, 210.0)
    sig = orc.thermal_sigma_kms(g["T"])
    vchan = 31.5 + (v - 210.0) / -4.0
    keep = orc.prune_mask(x, y, vchan, ranges, g["mHI"], 128, 128, 64, sig, edges)
    c = dict(x=x[keep], y=y[keep], ranges=ranges[keep], h_eff=(hpx * resc)[keep],
             kidx=kidx[keep], v=v[keep], sigma=sig[keep],
             amp=(g["mHI"] / d**2 / orc.MHI_TO_JY)[keep], kernels=kernels, spectral="gaussian",
             edges=edges, nx=128, ny=128, nc=64, pad=0)
    spectra = orc.init_spectra("gaussian", g["mHI"][keep], d[keep], v[keep], edges, sig[keep])
    ref = orc.insert_scatter(128, 128, c["x"], c["y"], c["ranges"], kernels, c["kidx"],
                             c["h_eff"], spectra)
    got, flux = run_gpu(engine, c, form=form)
    assert_close(got, ref, flux, tol=FORM_TOL[form], ftol=FLUX_TOL[form])


@pytest.mark.parametrize("form", FORMS, ids=FORM_IDS)
def test_insertion_is_deterministic(engine, form):
    """Stable sort + fixed split-K order: two runs give identical bits."""
    d = load_case("cfg1_disc_cubic")
    c = case_inputs(d)
    a, fa = run_gpu(engine, c, form=form)
    b, fb = run_gpu(engine, c, form=form, plan=False)
    assert np.array_equal(a, b)
    assert np.array_equal(fa, fb)


@pytest.mark.parametrize("form", FORMS, ids=FORM_IDS)
def test_split_k_large_tile_matches_oracle(engine, form):
    """Thousands of particles on one tile: several K chunks per segment, the
    split-K partial reduction, against the oracle."""
    rng = np.random.default_rng(17)
    n = 9000
    x = rng.normal(6.0, 1.5, n)
    y = rng.normal(9.0, 2.5, n)
    h = 10 ** rng.uniform(0.2, 0.6, n)
    kernels = orc.adaptive_tuple("WendlandC2Kernel")
    kidx, size, resc = orc.select_kernels(kernels, h)
    ranges = orc.sm_ranges(h, size)
    edges = orc.vrad_channel_edges(96, 4.0, 300.0)
    v = rng.uniform(150, 450, n)
    sig = rng.uniform(4, 12, n)
    mHI = 10 ** rng.uniform(4, 5, n)
    c = dict(x=x, y=y, ranges=ranges, h_eff=h * resc, kidx=kidx, v=v, sigma=sig,
             amp=mHI / 9.0 / orc.MHI_TO_JY, kernels=kernels, spectral="gaussian", edges=edges,
             nx=20, ny=24, nc=96, pad=0)
    spectra = orc.init_spectra("gaussian", mHI, np.full(n, 3.0), v, edges, sig)
    ref = orc.insert_scatter(20, 24, x, y, ranges, kernels, kidx, h * resc, spectra)
    got, flux = run_gpu(engine, c, form=form)
    assert_close(got, ref, flux, tol=FORM_TOL[form], ftol=FLUX_TOL[form])


@pytest.mark.parametrize("form", TC_FORMS, ids=TC_IDS)
def test_spectrum_store_matches_in_kernel_lines(engine, form):
    """The tensor-core forms read Gaussian lines from the per-particle
    spectrum store when the workspace has room for it (mg_plan's size) and
    evaluate them in the contraction otherwise (a workspace of exactly
    mg_workspace_size).  Both use the same arithmetic: identical cubes."""
    import ctypes as C
    from martini_gb300 import _native as N
    from martini_gb300.engine import DeviceParticles
    rng = np.random.default_rng(5)
    n, nx, ny, nc = 4000, 48, 40, 96
    kernels = orc.adaptive_tuple("WendlandC2Kernel")
    h = 10 ** rng.uniform(-0.3, 0.8, n)
    kidx, size, resc = orc.select_kernels(kernels, h)
    parts = DeviceParticles.from_host(engine.device, rng.normal(24, 9, n), rng.normal(20, 8, n),
                                      orc.sm_ranges(h, size), h * resc, kidx,
                                      v=rng.normal(200, 60, n), sigma=rng.uniform(3, 20, n),
                                      amp=10 ** rng.uniform(-7, -5, n))
    edges = torch.from_numpy(orc.vrad_channel_edges(nc, 4.0, 200.0)).to(engine.device)
    table = native_kernel_table(kernels)
    s = C.c_void_p(torch.cuda.current_stream(engine.device).cuda_stream)
    cubes = []
    for with_store in (True, False):
        cube = torch.empty((nx, ny, nc), dtype=torch.float32, device=engine.device)
        prob = engine.problem(parts, table, N.MG_SPECTRUM_GAUSSIAN, 0.0, nx, ny, nc, 0, 0, edges,
                              cube, None, form)
        info = engine.plan(prob)
        exact = C.c_size_t()
        N.check(engine.lib.mg_workspace_size(C.byref(prob), info.n_pairs, info.n_partial_items,
                                             C.byref(exact)))
        assert info.workspace_bytes > exact.value  # room for the store
        nbytes = info.workspace_bytes if with_store else exact.value
        ws = torch.empty(nbytes, dtype=torch.uint8, device=engine.device)
        N.check(engine.lib.mg_insert(C.byref(prob), C.c_void_p(ws.data_ptr()), nbytes,
                                     info.n_pairs, info.n_partial_items, s))
        N.check(engine.lib.mg_check(C.c_void_p(ws.data_ptr()), s))
        cubes.append(cube.cpu().numpy())
    assert np.abs(cubes[0]).max() > 0
    np.testing.assert_array_equal(cubes[0], cubes[1])


@pytest.mark.parametrize("form", FORMS, ids=FORM_IDS)
@pytest.mark.parametrize("shape", [(2048, 2048), (4096, 2048)], ids=["2048x2048", "4096x2048"])
def test_large_sparse_tile_grids(engine, shape, form):
    """Tile grids too large for the shared-memory coverage histogram of the
    binning kernel (2048 x 2048: 129 x 257 difference array) and for the
    shared-memory prefix sums of the tile plan (4096 x 2048: 257 x 257)
    take the global-memory paths: same cube as the oracle."""
    nx, ny = shape
    nc = 4
    rng = np.random.default_rng(17)
    n = 400
    kernels = orc.adaptive_tuple("WendlandC2Kernel")
    h = 10 ** rng.uniform(0.0, 1.3, n)
    kidx, size, resc = orc.select_kernels(kernels, h)
    x = rng.uniform(-10, nx + 10, n)
    y = rng.uniform(-10, ny + 10, n)
    edges = orc.vrad_channel_edges(nc, 4.0, 100.0)
    sig = rng.uniform(3, 6, n)
    v = rng.normal(100, 4, n)
    mhi = 10 ** rng.uniform(4, 5, n)
    dist = np.full(n, 3.0)
    c = dict(x=x, y=y, ranges=orc.sm_ranges(h, size), h_eff=h * resc, kidx=kidx, v=v, sigma=sig,
             amp=mhi / dist**2 / orc.MHI_TO_JY, kernels=kernels, spectral="gaussian",
             edges=edges, nx=nx, ny=ny, nc=nc, pad=0)
    spectra = orc.init_spectra("gaussian", mhi, dist, v, edges, sig)
    ref = orc.insert_scatter(nx, ny, x, y, c["ranges"], kernels, kidx, c["h_eff"], spectra)
    got, flux = run_gpu(engine, c, form=form)
    assert_close(got, ref, flux, tol=FORM_TOL[form], ftol=FLUX_TOL[form])


@pytest.mark.parametrize("form", FORMS, ids=FORM_IDS)
@pytest.mark.parametrize("nc", [300, 512])
def test_wide_band(engine, form, nc):
    """Bands wider than 256 channels (the 2 km/s, 512-channel configuration):
    the tensor-core forms hold the whole band in TMEM (KC = 32 stages, no
    master accumulator); the FP32 form uses many 64-channel blocks."""
    g = orc.disc_particles(6000, seed=33, h_med=0.7)
    xyz, vxyz = orc.incline(g["xyz"], g["vxyz"], 60.0)
    ra, dec, v, d = orc.project_particles(xyz, vxyz, 10.0)
    x, y = orc.tan_world2pix(ra, dec, 0.0, 0.0, 32.5, 32.5, -10 / 3600, 10 / 3600)
    hpx = orc.sm_lengths_px(g["hsm"], d, 10.0)
    kernels = orc.adaptive_tuple("WendlandC2Kernel")
    kidx, size, resc = orc.select_kernels(kernels, hpx)
    ranges = orc.sm_ranges(hpx, size)
    vc = 700.0
    edges = orc.vrad_channel_edges(nc, 2.0, vc)
    sig = orc.thermal_sigma_kms(g["T"])
    vchan = (nc - 1) / 2 + (v - vc) / -2.0
    keep = orc.prune_mask(x, y, vchan, ranges, g["mHI"], 64, 64, nc, sig, edges)
    c = dict(x=x[keep], y=y[keep], ranges=ranges[keep], h_eff=(hpx * resc)[keep],
             kidx=kidx[keep], v=v[keep], sigma=sig[keep],
             amp=(g["mHI"] / d**2 / orc.MHI_TO_JY)[keep], kernels=kernels, spectral="gaussian",
             edges=edges, nx=64, ny=64, nc=nc, pad=0)
    spectra = orc.init_spectra("gaussian", g["mHI"][keep], d[keep], v[keep], edges, sig[keep])
    ref = orc.insert_scatter(64, 64, c["x"], c["y"], c["ranges"], kernels, c["kidx"],
                             c["h_eff"], spectra)
    got, flux = run_gpu(engine, c, form=form)
    assert_close(got, ref, flux, tol=FORM_TOL[form], ftol=FLUX_TOL[form])


@pytest.mark.parametrize("form", FORMS, ids=FORM_IDS)
def test_accumulate_two_spectral_groups(engine, form):
    """Two particle groups with different spectral models (Gaussian lines and
    Dirac lines) inserted into one cube: the second call adds to the first
    (accumulate mode, the reference's `_array +=`); the flux covers both.
    Also checks that accumulate keeps what the cube held before."""
    from martini_gb300 import _native as N
    from martini_gb300.engine import DeviceParticles
    rng = np.random.default_rng(41)
    n, nx, ny, nc = 3000, 40, 36, 48
    kernels = orc.adaptive_tuple("WendlandC2Kernel")
    h = 10 ** rng.uniform(-0.3, 0.8, n)
    kidx, size, resc = orc.select_kernels(kernels, h)
    x, y = rng.normal(20, 7, n), rng.normal(18, 6, n)
    ranges = orc.sm_ranges(h, size)
    v, sig = rng.normal(250, 30, n), rng.uniform(4, 10, n)
    mhi = 10 ** rng.uniform(4, 5, n)
    amp = mhi / 9.0 / orc.MHI_TO_JY
    edges = orc.vrad_channel_edges(nc, 4.0, 250.0)
    dirac = rng.random(n) < 0.2
    groups = [(~dirac, N.MG_SPECTRUM_GAUSSIAN, "gaussian"), (dirac, N.MG_SPECTRUM_DIRAC, "dirac")]
    ref = np.zeros((nx, ny, nc))
    for m, _, model in groups:
        sp = orc.init_spectra(model, mhi[m], np.full(m.sum(), 3.0), v[m], edges,
                              sig[m] if model == "gaussian" else None)
        ref += orc.insert_scatter(nx, ny, x[m], y[m], ranges[m], kernels, kidx[m], (h * resc)[m],
                                  sp)
    base = np.linspace(0.0, 1e-3, nx * ny * nc).reshape(nx, ny, nc).astype(np.float32)
    cube = torch.from_numpy(base).to(engine.device)
    table = native_kernel_table(kernels)
    e = torch.from_numpy(edges).to(engine.device)
    for m, model, _ in groups:
        parts = DeviceParticles.from_host(engine.device, x[m], y[m], ranges[m], (h * resc)[m],
                                          kidx[m], v=v[m], sigma=sig[m], amp=amp[m])
        _, flux = engine.insert(parts, table, model, 0.0, nx, ny, nc, e, form=form, cube=cube,
                                accumulate=True)
    got = cube.cpu().numpy().astype(np.float64) - base
    peak = np.abs(ref).max()
    assert np.abs(got - ref).max() / peak <= FORM_TOL[form]
    tot = ref.sum() + base.astype(np.float64).sum()
    assert abs(flux.cpu().numpy()[0] - tot) / tot <= TOL_FLUX


@pytest.mark.parametrize("form", FORMS, ids=FORM_IDS)
def test_batch_of_cubes_matches_oracle(engine, form):
    """Seven cubes of different shapes, pads and channel grids in one
    mg_insert_batched call (one binning pass, one contraction queue),
    including an empty cube and one whose particles all miss it: each cube
    equals its own oracle insertion."""
    from martini_gb300 import _native as N
    from martini_gb300.engine import DeviceParticles, insert_batch
    rng = np.random.default_rng(77)
    kernels = orc.adaptive_tuple("WendlandC2Kernel")
    shapes = [(16, 16, 24, 0), (40, 24, 48, 2), (24, 48, 64, 0), (8, 8, 16, 0), (64, 40, 300, 0),
              (32, 32, 32, 4), (20, 28, 40, 0)]
    items, refs = [], []
    for k, (nx, ny, nc, pad) in enumerate(shapes):
        n = [400, 1500, 2500, 0, 2000, 800, 300][k]
        h = 10 ** rng.uniform(-0.4, 0.8, n)
        kidx, size, resc = orc.select_kernels(kernels, h)
        if k == 6:  # every particle misses the cube
            x, y = rng.uniform(nx + 40, nx + 60, n), rng.uniform(0, ny, n)
        else:
            x, y = rng.normal(nx / 2, nx / 5, n), rng.normal(ny / 2, ny / 5, n)
        vc = 100.0 + 50 * k
        edges = orc.vrad_channel_edges(nc, 4.0 if k % 2 == 0 else 3.0, vc)
        v, sig = rng.normal(vc, 15, n), rng.uniform(3, 9, n)
        mhi = 10 ** rng.uniform(4, 5, n)
        spectra = orc.init_spectra("gaussian", mhi, np.full(n, 3.0), v, edges, sig)
        ranges = orc.sm_ranges(h, size)
        refs.append(orc.insert_scatter(nx, ny, x, y, ranges, kernels, kidx, h * resc, spectra))
        parts = DeviceParticles.from_host(engine.device, x, y, ranges, h * resc, kidx, v=v, sigma=sig,
                                          amp=mhi / 9.0 / orc.MHI_TO_JY)
        items.append(dict(parts=parts, edges=torch.from_numpy(edges).to(engine.device), nx=nx,
                          ny=ny, nc=nc, padx=pad, pady=pad))
    outs = insert_batch(engine, items, native_kernel_table(kernels), N.MG_SPECTRUM_GAUSSIAN,
                        form=form)
    for k, ((cube, flux), ref) in enumerate(zip(outs, refs)):
        got = cube.cpu().numpy().astype(np.float64)
        pad = shapes[k][3]
        if np.abs(ref).max() == 0:
            assert np.abs(got).max() == 0, f"cube {k}"
            assert flux.cpu().numpy()[0] == 0.0
            continue
        assert_close(got, ref, flux.cpu().numpy(), pad=pad, tol=FORM_TOL[form], ftol=FLUX_TOL[form])


def test_cuda_graph_replay_matches_direct_run(engine):
    """mg_insert captured in a CUDA graph (no host synchronisation or
    allocation inside) and replayed gives the same bits as a direct run,
    split-K partials included."""
    from martini_gb300 import _native as N
    from martini_gb300.engine import DeviceParticles, InsertionEngine
    rng = np.random.default_rng(9)
    n, nx, ny, nc = 30000, 48, 40, 64
    kernels = orc.adaptive_tuple("WendlandC2Kernel")
    h = 10 ** rng.uniform(-0.2, 0.9, n)
    kidx, size, resc = orc.select_kernels(kernels, h)
    parts = DeviceParticles.from_host(engine.device, rng.normal(24, 6, n), rng.normal(20, 5, n),
                                      orc.sm_ranges(h, size), h * resc, kidx,
                                      v=rng.normal(200, 30, n), sigma=rng.uniform(4, 10, n),
                                      amp=10 ** rng.uniform(-7, -6, n))
    edges = torch.from_numpy(orc.vrad_channel_edges(nc, 4.0, 200.0)).to(engine.device)
    for form in (N.MG_FORM_FP32, N.MG_FORM_F16X3, N.MG_FORM_BF16X6):
        eng = InsertionEngine("cuda:0")
        cube = torch.empty((nx, ny, nc), dtype=torch.float32, device=eng.device)
        flux = torch.empty(nc + 1, dtype=torch.float64, device=eng.device)
        prob = eng.problem(parts, native_kernel_table(kernels), N.MG_SPECTRUM_GAUSSIAN, 0.0, nx,
                           ny, nc, 0, 0, edges, cube, flux, form)
        info = eng.plan(prob)
        assert info.n_partial_items > 0  # split-K in play
        eng.run(prob)
        eng.check()
        ref = cube.clone()
        graph = eng.capture(prob)
        cube.fill_(-1.0)
        graph.replay()
        graph.replay()
        torch.cuda.synchronize()
        eng.check()
        assert torch.equal(cube, ref)
