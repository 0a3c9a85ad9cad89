"""Shared helpers for the parity tests: golden-case inputs and the oracle
pipeline (test infrastructure; not imported by the product)."""

import os

import numpy as np

from oracle import martini_oracle as orc

GOLD = os.path.join(os.path.dirname(__file__), "golden")

NATIVE_TYPE = {orc.KT_WENDLAND_C2: 0, orc.KT_WENDLAND_C6: 1, orc.KT_CUBIC_SPLINE: 2,
               orc.KT_QUARTIC_SPLINE: 3, orc.KT_GAUSSIAN: 4, orc.KT_DIRAC: 5}


def golden_cases():
    return sorted(os.path.basename(p)[5:-4] for p in os.listdir(GOLD)
                  if p.startswith("cube_") and p.endswith(".npz"))


def load_case(name):
    return dict(np.load(os.path.join(GOLD, f"cube_{name}.npz")))


def kernels_of(d):
    kname = str(d["kernel"])
    karg = float(d["kernel_arg"])
    trunc = karg if np.isfinite(karg) else 3.0
    if kname.startswith("_") or kname == "DiracDeltaKernel":
        kt = {"_WendlandC2Kernel": orc.KT_WENDLAND_C2, "_WendlandC6Kernel": orc.KT_WENDLAND_C6,
              "_CubicSplineKernel": orc.KT_CUBIC_SPLINE,
              "_QuarticSplineKernel": orc.KT_QUARTIC_SPLINE,
              "_GaussianKernel": orc.KT_GAUSSIAN, "DiracDeltaKernel": orc.KT_DIRAC}[kname]
        return orc.simple_tuple(kt, trunc)
    return orc.adaptive_tuple(kname, trunc)


def case_inputs(d):
    """Pruned particle arrays of a golden case, as the reference inserts them."""
    kernels = kernels_of(d)
    h = d["h_px"]
    kidx, size, resc = orc.select_kernels(kernels, h)
    ranges = orc.sm_ranges(h, size)
    spectral = str(d["spectral"])
    if spectral == "gaussian":
        sig = orc.thermal_sigma_kms(d["T"]) if d["T"].size else np.broadcast_to(
            d["sigma"], h.shape).astype(float)
    else:
        sig = np.zeros_like(h)
    pad = int(d["pad"])
    nx, ny, nc = int(d["nx"]) + 2 * pad, int(d["ny"]) + 2 * pad, int(d["nc"])
    hw = sig if spectral == "gaussian" else 0.0
    keep = orc.prune_mask(d["x"], d["y"], d["vchan"], ranges, d["mHI"], nx, ny, int(d["nc"]), hw,
                          d["edges"])
    k = keep
    return dict(x=d["x"][k], y=d["y"][k], ranges=ranges[k], h_eff=(h * resc)[k],
                kidx=kidx[k], v=d["v"][k], sigma=sig[k], mHI=d["mHI"][k], dist=d["dist"][k],
                amp=d["mHI"][k] / d["dist"][k] ** 2 / orc.MHI_TO_JY, kernels=kernels,
                spectral=spectral, edges=d["edges"], nx=nx, ny=ny, nc=nc, pad=pad)


def native_kernel_table(kernels):
    return [(NATIVE_TYPE[k["ktype"]], k["truncate"]) for k in kernels]
