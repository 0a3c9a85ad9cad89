"""The generated kernel-integral tables (martini_gb300/csrc/gen_kernel_tables.py
-> mg_kernel_tables.h): the committed header is what the generator writes,
the FP32 device-form errors against the reference's closed forms stay at the
FP32 floor, and an s-table gives exactly zero past the kernel support
(CPU only)."""

import importlib.util
import os

import numpy as np
import pytest

GEN = os.path.join(os.path.dirname(__file__), os.pardir, "martini_gb300", "csrc",
                   "gen_kernel_tables.py")


@pytest.fixture(scope="module")
def gen():
    spec = importlib.util.spec_from_file_location("gen_kernel_tables", GEN)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="module")
def rendered(gen):
    return gen.render()


def test_committed_header_is_generated(gen, rendered):
    text, _ = rendered
    with open(gen.HEADER) as fh:
        assert fh.read() == text


# relative to f(0) for the kernel profiles; absolute for erf(zmax / sqrt 2)
BOUNDS = {"WENDLAND_C2": 1.5e-7, "WENDLAND_C6": 7.5e-7, "CUBIC_SPLINE": 1.2e-7,
          "QUARTIC_SPLINE": 1.0e-7, "GAUSS_TRUNC": 1.0e-7}


@pytest.mark.parametrize("name", sorted(BOUNDS))
def test_fp32_device_form_error(rendered, name):
    _, errors = rendered
    assert errors[name] <= BOUNDS[name], f"{name}: {errors[name]:.3e}"


@pytest.mark.parametrize("kidx", [0, 1, 3])  # the s-tables: WendlandC2, C6, quartic
def test_stable_is_zero_past_the_support(gen, kidx):
    name, code, f, smax, scale, regions = gen.KERNELS[kidx]
    var, lo, hi, n = regions[0]
    assert var == "S"
    coefs = np.concatenate([gen.fit_cells(gen.region_fn(f, var), lo, hi, n),
                            np.zeros((1, gen.DEG + 1), np.float32)])
    s = np.concatenate((np.full(10, smax), smax * (1 + np.logspace(-7, 3, 200))))
    assert np.all(gen.device_eval(regions, coefs, smax, s) == 0.0)
    inside = np.linspace(0.0, smax * (1 - 1e-3), 2001)
    assert np.all(gen.device_eval(regions, coefs, smax, inside) >= -1e-7 * f(np.zeros(1))[0])
