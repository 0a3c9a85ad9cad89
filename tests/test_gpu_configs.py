"""Parity at the full sizes of the benchmark configurations, against the
FP64 oracle.

The oracle's whole per-pixel cube would take hours to days at these sizes
(O(N_pix * N)), so each configuration is checked two ways:

* sampled pixels: the reference's per-pixel sum (`_evaluate_pixel_spectrum`,
  martini/martini.py:243-283, restated in the oracle) at 48 pixels with
  signal and 16 uniform ones, within 1e-5 of the cube peak;
* total flux: the oracle's FP64 total over the unpadded cube
  (martini/martini.py:367-375), evaluated per particle as
  sum_p (sum_box W_p)(sum_c S_p(c)) in C (oracle/flux_total.c), within 1e-6
  relative of the GPU's FP64 flux sum.

Configurations:

* disc1m_512: 1M particles, WendlandC2 (adaptive), thermal lines,
  512 x 512 x 256;
* disc4m_1024: 4M particles, 1024 x 1024 x 512 channels of 2 km/s;
* stress16m_2048: 16M particles (disc + Plummer halo, h log-uniform
  0.05-20 kpc), thermal lines and a seeded 20 % on Dirac lines (two
  spectral groups added into one cube), 2048 x 2048 x 256.  Its sampled
  pixels use all 16M particles; its total flux is checked on a seeded
  1M-particle subset inserted into the same full-size cube (the FP64 total
  of all 16M particles is ~2.6e11 kernel evaluations, minutes of host time);
* the disc population: a seeded set of galaxies covering all four cube
  shapes, inserted as one batch, every cube checked.

Every form held to the bar is checked: bf16x6, f16x3 and fp32.
"""

import numpy as np
import pytest
import torch

from oracle import martini_oracle as orc

pytestmark = pytest.mark.gpu

TOL_PEAK = 1e-5
TOL_FLUX = 1e-6
FORMS = {"bf16x6": 3, "f16x3": 2, "fp32": 0}

_WL = {}


def workload(name):
    if name not in _WL:
        from martini_gb300 import workloads
        _WL.clear()  # one full-size workload in host memory at a time
        _WL[name] = workloads.build(name)
    return _WL[name]


def _groups(w, sel=None):
    """(particle indices, spectral model name, native model) per group."""
    from martini_gb300 import _native as N
    idx = np.arange(w["n"]) if sel is None else np.asarray(sel)
    if not w["groups"]:
        model = "dirac" if w["spectral_model"] == N.MG_SPECTRUM_DIRAC else "gaussian"
        return [(idx, model, w["spectral_model"])]
    out = []
    for g in w["groups"]:
        s = np.intersect1d(idx, g["sel"], assume_unique=True)
        model = "dirac" if g["spectral_model"] == N.MG_SPECTRUM_DIRAC else "gaussian"
        out.append((s, model, g["spectral_model"]))
    return out


def insert(w, form, sel=None):
    """GPU insertion of a workload (or a particle subset) in one form; every
    spectral group after the first adds to the cube.  Host cube and flux."""
    from martini_gb300.engine import DeviceParticles, InsertionEngine
    eng = InsertionEngine("cuda:0")
    dev = eng.device
    edges = torch.from_numpy(np.ascontiguousarray(w["edges"])).to(dev)
    cube = torch.empty((w["nx"], w["ny"], w["nc"]), dtype=torch.float32, device=dev)
    flux = None
    for gi, (s, _, model) in enumerate(_groups(w, sel)):
        kidx = w["kernel_index"][s] if w["kernel_index"] is not None else None
        sig = w["sigma"][s] if w["sigma"] is not None else None
        parts = DeviceParticles.from_host(dev, w["x"][s], w["y"][s], w["sm_range"][s],
                                          w["h_eff"][s], kidx, v=w["v"][s], sigma=sig,
                                          amp=w["amp"][s])
        _, flux = eng.insert(parts, w["kernels"], model, w["sigma_const"], w["nx"], w["ny"],
                             w["nc"], edges, form=FORMS[form], cube=cube, accumulate=gi > 0)
        del parts
    out = cube.cpu().numpy(), flux.cpu().numpy()
    del cube, eng
    torch.cuda.empty_cache()
    return out


def oracle_kernels(w):
    return orc.adaptive_tuple(w["kernel_name"])


_FLUX = {}


def oracle_flux(w, sel=None):
    """FP64 total flux of the workload (or a subset) over the cube (cached
    per workload and subset: every form is checked against the same total)."""
    key = (w["name"], None if sel is None else (len(sel), int(np.sum(sel[:1000]))))
    if key not in _FLUX:
        _FLUX[key] = _oracle_flux(w, sel)
    return _FLUX[key]


def _oracle_flux(w, sel):
    kern = oracle_kernels(w)
    tot = 0.0
    for s, model, _ in _groups(w, sel):
        sig = None
        if model == "gaussian":
            sig = w["sigma"][s] if w["sigma"] is not None else w["sigma_const"]
        ss = orc.spectrum_sums(model, w["v"][s], sig, w["amp"][s], w["edges"])
        kidx = w["kernel_index"][s] if w["kernel_index"] is not None else None
        tot += orc.flux_total(w["x"][s], w["y"][s], w["sm_range"][s], kern, kidx,
                              w["h_eff"][s].astype(np.float64), ss, w["nx"], w["ny"])
    return tot


def oracle_pixels(w, pixels):
    """The reference's per-pixel sum at each pixel (all particles, every
    group), from the oracle's mask, weights and spectra."""
    kern = oracle_kernels(w)
    acc = np.zeros((len(pixels), w["nc"]))
    for s, model, _ in _groups(w):
        kidx = w["kernel_index"][s] if w["kernel_index"] is not None else None
        sig = None
        if model == "gaussian":
            sig = w["sigma"][s] if w["sigma"] is not None else w["sigma_const"]
        acc += orc.pixel_spectra(pixels, w["x"][s], w["y"][s], w["sm_range"][s], kern, kidx,
                                 w["h_eff"][s], model, w["mHI"][s], w["dist"][s], w["v"][s],
                                 w["edges"], sig)
    return acc


def pick_pixels(cube, seed=3):
    rng = np.random.default_rng(seed)
    lit = np.argwhere(cube.max(axis=2) > 1e-3 * cube.max())
    pick = lit[rng.choice(len(lit), size=min(48, len(lit)), replace=False)]
    uni = np.stack([rng.integers(0, cube.shape[0], 16), rng.integers(0, cube.shape[1], 16)],
                   axis=1)
    return [tuple(int(v) for v in p) for p in np.concatenate([pick, uni])]


_PIX = {}


def sampled_reference(name, cube):
    """Sampled pixels (chosen from the first cube seen) and their oracle sums."""
    if name not in _PIX:
        pixels = pick_pixels(cube)
        _PIX[name] = (pixels, oracle_pixels(workload(name), pixels))
    return _PIX[name]


def check_sampled(name, cube):
    pixels, ref = sampled_reference(name, cube)
    peak = float(np.abs(cube).max())
    got = np.stack([cube[i, j] for i, j in pixels]).astype(np.float64)
    err = np.abs(got - ref).max() / peak
    assert err <= TOL_PEAK, f"{name}: sampled max err / peak = {err:.3e}"
    return err


@pytest.mark.parametrize("form", list(FORMS))
@pytest.mark.parametrize("name", ["disc1m_512", "disc4m_1024"])
def test_full_size_disc(name, form):
    """cfg2 / cfg3 at full size: sampled pixels and the FP64 total flux."""
    w = workload(name)
    cube, flux = insert(w, form)
    check_sampled(name, cube)
    ref = oracle_flux(w)
    ferr = abs(flux[0] - ref) / ref
    assert ferr <= TOL_FLUX, f"{name} {form}: flux rel err {ferr:.3e}"


@pytest.mark.parametrize("form", list(FORMS))
def test_stress_16m(form):
    """cfg5: 16M particles, two spectral groups, h over 0.05-20 kpc."""
    w = workload("stress16m_2048")
    cube, _ = insert(w, form)
    check_sampled("stress16m_2048", cube)
    del cube
    sub = np.sort(np.random.default_rng(11).choice(w["n"], 1_000_000, replace=False))
    _, flux = insert(w, form, sub)
    ref = oracle_flux(w, sub)
    ferr = abs(flux[0] - ref) / ref
    assert ferr <= TOL_FLUX, f"stress16m_2048 {form}: subset flux rel err {ferr:.3e}"


def population_subset(n=24):
    """Seeded galaxies of the population covering every cube shape."""
    from martini_gb300 import workloads
    cfgs = workloads.population_configs()
    shapes = {}
    for k, c in enumerate(cfgs):
        shapes.setdefault((c["nx"], c["nc"]), []).append(k)
    rng = np.random.default_rng(17)
    pick = []
    for key in sorted(shapes):
        pick += list(rng.choice(shapes[key], n // len(shapes), replace=False))
    return [workloads._assemble(f"pop{k}", cfgs[k], cfgs[k]["n"]) for k in sorted(pick)]


@pytest.mark.parametrize("form", list(FORMS))
def test_population_batch(form):
    """cfg4: one batched insertion of galaxies of every cube shape; each cube
    against the oracle (sampled pixels, total flux)."""
    from martini_gb300.engine import BatchInsertion, DeviceParticles, InsertionEngine
    gals = population_subset()
    assert {(g["nx"], g["nc"]) for g in gals} == {(32, 64), (64, 128), (128, 128), (256, 256)}
    eng = InsertionEngine("cuda:0")
    dev = eng.device
    items, probs = [], []
    for w in gals:
        parts = DeviceParticles.from_host(dev, w["x"], w["y"], w["sm_range"], w["h_eff"],
                                          w["kernel_index"], v=w["v"], sigma=w["sigma"],
                                          amp=w["amp"])
        edges = torch.from_numpy(np.ascontiguousarray(w["edges"])).to(dev)
        cube = torch.empty((w["nx"], w["ny"], w["nc"]), dtype=torch.float32, device=dev)
        flux = torch.empty(w["nc"] + 1, dtype=torch.float64, device=dev)
        probs.append(eng.problem(parts, w["kernels"], w["spectral_model"], w["sigma_const"],
                                 w["nx"], w["ny"], w["nc"], 0, 0, edges, cube, flux,
                                 FORMS[form]))
        items.append(dict(parts=parts, edges=edges, cube=cube, flux=flux))
    batch = BatchInsertion(eng, probs, keep=items)
    batch.plan()
    batch.run()
    batch.check()
    for w, it in zip(gals, items):
        cube = it["cube"].cpu().numpy()
        if w["n"] == 0 or cube.max() <= 0:
            continue
        pixels = pick_pixels(cube)[:24]
        ref = oracle_pixels(w, pixels)
        peak = float(np.abs(cube).max())
        got = np.stack([cube[i, j] for i, j in pixels]).astype(np.float64)
        err = np.abs(got - ref).max() / peak
        assert err <= TOL_PEAK, f"{w['name']}: sampled max err / peak = {err:.3e}"
        tot = oracle_flux(w)
        ferr = abs(it["flux"][0].item() - tot) / tot
        assert ferr <= TOL_FLUX, f"{w['name']}: flux rel err {ferr:.3e}"
