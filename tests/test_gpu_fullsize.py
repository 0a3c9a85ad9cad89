"""Whole-cube properties at the benchmark's full size: the 1M-particle
WendlandC2 disc with thermal lines on 512 x 512 x 256 (15.9M tile-particle
pairs, split-K on every dense tile).  Sampled pixels and the FP64 total
flux against the oracle at this and the other configurations' sizes are in
test_gpu_configs.py; here:

* the three forms against each other over every voxel;
* linearity: inserting two halves of the particles and adding the cubes
  gives the cube of all particles, in the chosen form.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

FORM_TOL = {"fp32": 1e-5, "f16x3": 1e-5, "bf16x6": 1e-5}
FORM_CODE = {"fp32": 0, "f16x3": 2, "bf16x6": 3}


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
    return {f: _insert(disc, f) for f in ("fp32", "f16x3", "bf16x6")}


def test_forms_agree_over_every_voxel(cubes):
    ref = cubes["fp32"][0].astype(np.float64)
    peak = np.abs(ref).max()
    for form in ("f16x3", "bf16x6"):
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
    a, fa = _insert(disc, "bf16x6", np.flatnonzero(half))
    b, fb = _insert(disc, "bf16x6", np.flatnonzero(~half))
    full, ff = cubes["bf16x6"]
    peak = np.abs(full).max()
    err = np.abs(a.astype(np.float64) + b - full).max() / peak
    assert err <= 2 * FORM_TOL["bf16x6"], f"{err:.3e}"
    assert abs(fa[0] + fb[0] - ff[0]) / ff[0] <= 2e-6
