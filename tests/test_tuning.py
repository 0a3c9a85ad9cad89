"""The launch-shape autotuner: candidate sets, the per-class cache (CPU,
no GPU access) and a tuned insertion (GPU) against the oracle."""

import ctypes as C

import numpy as np
import pytest

from oracle import martini_oracle as orc


def _problem(n=1000, nx=64, ny=64, nc=32, form=2, ngal=1):
    from martini_gb300 import _native as N
    probs = (N.Problem * ngal)()
    for p in probs:
        p.n, p.nx, p.ny, p.nc, p.form = n, nx, ny, nc, form
        p.n_kernels = 1
        p.kernels[0].type = N.MG_KERNEL_WENDLAND_C2
    return probs


def test_candidates_per_form():
    from martini_gb300 import _native as N
    lib = N.load()
    for form, count, kcs in ((N.MG_FORM_FP32, 6, {0}), (N.MG_FORM_BF16X6, 12, {0, 32}),
                             (N.MG_FORM_F16X3, 12, {0, 32}), (N.MG_FORM_BF16X3, 12, {0, 32})):
        out = (N.Tuning * 16)()
        n = lib.mg_tuning_candidates(form, out, 16)
        assert n == count
        shapes = {(t.kc, t.items_per_sm, t.cost_order) for t in out[:n]}
        assert len(shapes) == n and {s[0] for s in shapes} == kcs
        assert {s[1] for s in shapes} == {24, 12, 6} and {s[2] for s in shapes} == {0, 1}
        d = N.Tuning()
        lib.mg_tuning_default(C.byref(d))
        assert (d.kc, d.items_per_sm, d.cost_order) in shapes


def test_cache_keys_store_lookup_reset():
    from martini_gb300 import _native as N
    lib = N.load()
    lib.mg_tuning_reset()
    p = _problem()
    got = N.Tuning()
    assert lib.mg_tuning_lookup(p, 1, 200_000, C.byref(got)) == 0
    assert (got.kc, got.items_per_sm, got.cost_order) == (0, 6, 1)  # the default
    t = N.Tuning(32, 12, 0, 0)
    assert lib.mg_tuning_store(p, 1, 200_000, C.byref(t)) == N.MG_OK
    assert lib.mg_tuning_lookup(p, 1, 200_000, C.byref(got)) == 1
    assert (got.kc, got.items_per_sm, got.cost_order) == (32, 12, 0)
    # the same class: pairs per tile within the half octave, particles in the octave
    assert lib.mg_tuning_lookup(_problem(n=1020), 1, 210_000, C.byref(got)) == 1
    # other classes: form, band, particle octave, pairs-per-tile bucket, cube count
    for q, pairs in ((_problem(form=3), 200_000), (_problem(nc=64), 200_000),
                     (_problem(n=5000), 200_000), (_problem(), 800_000),
                     (_problem(ngal=4), 200_000)):
        assert lib.mg_tuning_lookup(q, len(q), pairs, C.byref(got)) == 0
    # a shape the form cannot run is refused
    bad = N.Tuning(48, 24, 1, 0)
    assert lib.mg_tuning_store(_problem(form=3), 1, 200_000, C.byref(bad)) == \
        N.MG_ERR_INVALID_ARGUMENT
    assert lib.mg_tuning_store(_problem(form=0), 1, 200_000, C.byref(N.Tuning(32, 24, 1, 0))) \
        == N.MG_ERR_INVALID_ARGUMENT
    assert lib.mg_tuning_store(p, 1, 200_000, C.byref(N.Tuning(0, 99, 1, 0))) == \
        N.MG_ERR_INVALID_ARGUMENT
    lib.mg_tuning_reset()
    assert lib.mg_tuning_lookup(p, 1, 200_000, C.byref(got)) == 0


@pytest.mark.gpu
@pytest.mark.parametrize("form", [2, 3], ids=["f16x3", "bf16x6"])
def test_tuned_insertion_matches_oracle(form):
    """mg_tune picks a candidate and caches it for the class; the insertion
    with the cached shape stays within 1e-5 of peak and 1e-6 of flux."""
    from martini_gb300 import _native as N
    from martini_gb300.engine import DeviceParticles, InsertionEngine
    import torch
    lib = N.load()
    lib.mg_tuning_reset()
    rng = np.random.default_rng(21)
    n, nx, ny, nc = 20000, 64, 48, 64
    kernels = orc.adaptive_tuple("WendlandC2Kernel")
    h = 10 ** rng.uniform(-0.3, 0.9, n)
    kidx, size, resc = orc.select_kernels(kernels, h)
    x, y = rng.normal(32, 9, n), rng.normal(24, 7, n)
    ranges = orc.sm_ranges(h, size)
    v, sig = rng.normal(200, 40, n), rng.uniform(4, 12, n)
    mhi = 10 ** rng.uniform(4, 5, n)
    amp = mhi / 9.0 / orc.MHI_TO_JY
    edges = orc.vrad_channel_edges(nc, 4.0, 200.0)
    spectra = orc.init_spectra("gaussian", mhi, np.full(n, 3.0), v, edges, sig)
    ref = orc.insert_scatter(nx, ny, x, y, ranges, kernels, kidx, h * resc, spectra)
    eng = InsertionEngine("cuda:0")
    parts = DeviceParticles.from_host(eng.device, x, y, ranges, h * resc, kidx, v=v, sigma=sig,
                                      amp=amp)
    e = torch.from_numpy(edges).to(eng.device)
    table = [(N.MG_KERNEL_WENDLAND_C2, 0.0), (N.MG_KERNEL_DIRAC, 0.0), (N.MG_KERNEL_GAUSSIAN, 6.0)]
    cube = torch.empty((nx, ny, nc), dtype=torch.float32, device=eng.device)
    flux = torch.empty(nc + 1, dtype=torch.float64, device=eng.device)
    prob = eng.problem(parts, table, N.MG_SPECTRUM_GAUSSIAN, 0.0, nx, ny, nc, 0, 0, e, cube, flux,
                       form)
    info = eng.plan(prob)
    best = eng.tune(prob, reps=2)
    assert best["contract_ms"] > 0
    cands = (N.Tuning * 16)()
    k = lib.mg_tuning_candidates(form, cands, 16)
    assert (best["kc"], best["items_per_sm"], best["cost_order"]) in {
        (t.kc, t.items_per_sm, t.cost_order) for t in cands[:k]}
    got = N.Tuning()
    assert lib.mg_tuning_lookup(C.byref(prob), 1, info.n_pairs, C.byref(got)) == 1
    assert got.as_dict() == {kk: best[kk] for kk in ("kc", "items_per_sm", "cost_order")}
    eng.run(prob)
    eng.check()
    out = cube.cpu().numpy().astype(np.float64)
    assert np.abs(out - ref).max() / np.abs(ref).max() <= 1e-5
    assert abs(flux[0].item() - ref.sum()) / ref.sum() <= 1e-6
    lib.mg_tuning_reset()


@pytest.mark.gpu
@pytest.mark.parametrize("form", [2, 3], ids=["f16x3", "bf16x6"])
def test_every_candidate_shape_matches_oracle(form):
    """Each candidate launch shape of the form -- 64- and 32-particle stages
    (for bf16x6: two working accumulators, or one), 24 or 12 items per SM,
    cost-ordered or segment-ordered queue -- stored for the problem's class
    and used by the insertion, stays within 1e-5 of peak and 1e-6 of flux."""
    from martini_gb300 import _native as N
    from martini_gb300.engine import DeviceParticles, InsertionEngine
    import torch
    lib = N.load()
    lib.mg_tuning_reset()
    rng = np.random.default_rng(22)
    n, nx, ny, nc = 15000, 48, 64, 160  # two channel blocks for bf16x6
    kernels = orc.adaptive_tuple("WendlandC2Kernel")
    h = 10 ** rng.uniform(-0.3, 0.9, n)
    kidx, size, resc = orc.select_kernels(kernels, h)
    x, y = rng.normal(24, 7, n), rng.normal(32, 9, n)
    ranges = orc.sm_ranges(h, size)
    v, sig = rng.normal(0, 120, n), rng.uniform(4, 12, n)
    mhi = 10 ** rng.uniform(4, 5, n)
    amp = mhi / 9.0 / orc.MHI_TO_JY
    edges = orc.vrad_channel_edges(nc, 4.0, 0.0)
    spectra = orc.init_spectra("gaussian", mhi, np.full(n, 3.0), v, edges, sig)
    ref = orc.insert_scatter(nx, ny, x, y, ranges, kernels, kidx, h * resc, spectra)
    eng = InsertionEngine("cuda:0")
    parts = DeviceParticles.from_host(eng.device, x, y, ranges, h * resc, kidx, v=v, sigma=sig,
                                      amp=amp)
    e = torch.from_numpy(edges).to(eng.device)
    table = [(N.MG_KERNEL_WENDLAND_C2, 0.0), (N.MG_KERNEL_DIRAC, 0.0), (N.MG_KERNEL_GAUSSIAN, 6.0)]
    cube = torch.empty((nx, ny, nc), dtype=torch.float32, device=eng.device)
    flux = torch.empty(nc + 1, dtype=torch.float64, device=eng.device)
    prob = eng.problem(parts, table, N.MG_SPECTRUM_GAUSSIAN, 0.0, nx, ny, nc, 0, 0, e, cube, flux,
                       form)
    info = eng.plan(prob)
    cands = (N.Tuning * 16)()
    k = lib.mg_tuning_candidates(form, cands, 16)
    assert {t.kc for t in cands[:k]} == {0, 32}
    for t in cands[:k]:
        assert lib.mg_tuning_store(C.byref(prob), 1, info.n_pairs, C.byref(t)) == N.MG_OK
        eng.run(prob)
        eng.check()
        out = cube.cpu().numpy().astype(np.float64)
        shape = (t.kc, t.items_per_sm, t.cost_order)
        err = np.abs(out - ref).max() / np.abs(ref).max()
        assert err <= 1e-5, f"shape {shape}: max err / peak {err:.3e}"
        ferr = abs(flux[0].item() - ref.sum()) / ref.sum()
        assert ferr <= 1e-6, f"shape {shape}: flux rel err {ferr:.3e}"
    lib.mg_tuning_reset()
