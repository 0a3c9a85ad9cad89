"""Parity at the benchmark's full size: the 1M-particle WendlandC2 disc with
thermal lines on 512 x 512 x 256 (15.9M tile-particle pairs, split-K on
every dense tile).

The oracle's full per-pixel cube would take hours here, so full-size parity
is checked in four ways:

* sampled pixels: the reference's per-pixel sum (`_evaluate_pixel_spectrum`,
  martini/martini.py:243-283, restated in the oracle) on 48 pixels with
  signal and 16 uniform ones, against every form, within the form's
  tolerance of the cube peak;
* the FP64 flux sum against the cube's own sum (every voxel counted once);
* the three forms against each other over every voxel;
* linearity: inserting two halves of the particles and adding the cubes
  gives the cube of all particles.
"""

import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest
import torch

from oracle import martini_oracle as orc

pytestmark = pytest.mark.gpu

FORM_TOL = {"fp32": 1e-5, "bf16x3": 2e-5, "f16x3": 1e-5}
FORM_CODE = {"fp32": 0, "bf16x3": 1, "f16x3": 2}


@pytest.fixture(scope="module")
def disc():
    from martini_gb300 import workloads
    return workloads.build("disc1m_512")


def _insert(w, form, sel=None):
    from martini_gb300.engine import DeviceParticles, InsertionEngine
    eng = InsertionEngine("cuda:0")
    dev = eng.device
    s = slice(None) if sel is None else sel
    kidx = w["kernel_index"][s] if w["kernel_index"] is not None else None
    sig = w["sigma"][s] if w["sigma"] is not None else None
    parts = DeviceParticles.from_host(dev, w["x"][s], w["y"][s], w["sm_range"][s],
                                      w["h_eff"][s], kidx, v=w["v"][s], sigma=sig,
                                      amp=w["amp"][s])
    edges = torch.from_numpy(np.ascontiguousarray(w["edges"])).to(dev)
    cube, flux = eng.insert(parts, w["kernels"], w["spectral_model"], w["sigma_const"], w["nx"],
                            w["ny"], w["nc"], edges, form=FORM_CODE[form])
    out = cube.cpu().numpy(), flux.cpu().numpy()
    del cube, parts
    torch.cuda.empty_cache()
    return out


@pytest.fixture(scope="module")
def cubes(disc):
    return {f: _insert(disc, f) for f in ("fp32", "bf16x3", "f16x3")}


def _spectra_weighted(w, m, sig, wgt):
    """Sum over the masked particles of weight x spectrum (oracle FP64), in
    particle chunks on a thread pool (scipy's erf releases the GIL)."""
    idx = np.flatnonzero(m)

    def part(o):
        c = idx[o:o + 8192]
        sp = orc.init_spectra("gaussian", w["mHI"][c], w["dist"][c], w["v"][c], w["edges"],
                              sig[c])
        return (sp * wgt[o:o + c.size, None]).sum(axis=0)

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        return np.sum(list(ex.map(part, range(0, idx.size, 8192))), axis=0)


def _oracle_pixels(w, pixels):
    kernels = orc.adaptive_tuple(w["kernel_name"])
    kidx = (w["kernel_index"].astype(np.int64) if w["kernel_index"] is not None
            else np.zeros(w["n"], dtype=np.int64))
    sig = w["sigma"] if w["sigma"] is not None else np.full(w["n"], w["sigma_const"])
    x, y, r = w["x"], w["y"], w["sm_range"]
    out = np.zeros((len(pixels), w["nc"]))
    for k, (i, j) in enumerate(pixels):
        m = (np.abs(i - x) <= r) & (np.abs(j - y) <= r)
        if not m.any():
            continue
        dij = np.vstack((x[m] - i, y[m] - j))
        wgt = orc.px_weight(kernels, kidx[m], dij, w["h_eff"][m])
        out[k] = _spectra_weighted(w, m, sig, wgt)
    return out


@pytest.fixture(scope="module")
def sampled(disc, cubes):
    rng = np.random.default_rng(2024)
    cube = cubes["fp32"][0]
    lit = np.argwhere(np.abs(cube).max(axis=2) > 0)
    pick = lit[rng.choice(len(lit), size=48, replace=False)]
    uni = np.stack([rng.integers(0, disc["nx"], 16), rng.integers(0, disc["ny"], 16)], axis=1)
    pixels = [tuple(int(v) for v in p) for p in np.concatenate([pick, uni])]
    return pixels, _oracle_pixels(disc, pixels)


@pytest.mark.parametrize("form", ["fp32", "bf16x3", "f16x3"])
def test_sampled_pixels_match_oracle(cubes, sampled, form):
    pixels, ref = sampled
    cube = cubes[form][0]
    peak = np.abs(cube).max()
    got = np.stack([cube[i, j] for i, j in pixels]).astype(np.float64)
    err = np.abs(got - ref).max() / peak
    assert err <= FORM_TOL[form], f"{form}: max err / peak = {err:.3e}"


@pytest.mark.parametrize("form", ["fp32", "bf16x3", "f16x3"])
def test_flux_equals_cube_sum(cubes, form):
    cube, flux = cubes[form]
    tot = cube.astype(np.float64).sum()
    assert abs(flux[0] - tot) / tot <= 1e-9
    np.testing.assert_allclose(flux[1:], cube.astype(np.float64).sum(axis=(0, 1)), rtol=1e-9,
                               atol=1e-12 * tot)


def test_forms_agree_over_every_voxel(cubes):
    ref = cubes["fp32"][0].astype(np.float64)
    peak = np.abs(ref).max()
    for form in ("bf16x3", "f16x3"):
        err = np.abs(cubes[form][0] - ref).max() / peak
        # both within their own tolerance of the oracle, so within the sum
        assert err <= FORM_TOL[form] + FORM_TOL["fp32"], f"{form}: {err:.3e}"
        ferr = abs(cubes[form][1][0] - cubes["fp32"][1][0]) / cubes["fp32"][1][0]
        assert ferr <= 2e-6, f"{form}: flux {ferr:.3e}"


def test_linearity_over_particle_halves(disc, cubes):
    n = disc["n"]
    rng = np.random.default_rng(7)
    half = np.zeros(n, dtype=bool)
    half[rng.choice(n, n // 2, replace=False)] = True
    a, fa = _insert(disc, "f16x3", np.flatnonzero(half))
    b, fb = _insert(disc, "f16x3", np.flatnonzero(~half))
    full, ff = cubes["f16x3"]
    peak = np.abs(full).max()
    err = np.abs(a.astype(np.float64) + b - full).max() / peak
    assert err <= 2 * FORM_TOL["f16x3"], f"{err:.3e}"
    assert abs(fa[0] + fb[0] - ff[0]) / ff[0] <= 2e-6
