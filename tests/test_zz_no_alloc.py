"""mg_insert_noalloc: the insertion for callers that cannot allocate GPU memory.

Some callers (code inside a framework or memory pool that owns every device
allocation, or paths where allocating is not allowed) cannot hand the library
a workspace.  mg_insert_noalloc runs the same pipeline on a scratch array
built into the library.  These tests call it through the C ABI twice in a row
and compare each result with mg_insert's on a caller-provided workspace, and
check that a problem too large for the built-in scratch is refused with a
clear message.  This file is collected last, so a failure here does not stop
the other GPU tests from running first.
"""

import ctypes as C

import numpy as np
import pytest
import torch

from oracle import martini_oracle as orc

pytestmark = pytest.mark.gpu

TOL_PEAK = 1e-5   # the parity bar of every form tested here
TOL_FLUX = 1e-6


def _problem_inputs(n=3000, seed=29):
    rng = np.random.default_rng(seed)
    nx, ny, nc = 40, 36, 48
    x = rng.normal(20, 7, n)
    y = rng.normal(18, 6, n)
    h = 10 ** rng.uniform(-0.3, 0.7, n)
    kernels = orc.adaptive_tuple("WendlandC2Kernel")
    kidx, size, resc = orc.select_kernels(kernels, h)
    ranges = orc.sm_ranges(h, size)
    edges = orc.vrad_channel_edges(nc, 4.0, 250.0)
    v = rng.normal(250, 40, n)
    sig = rng.uniform(5, 12, n)
    amp = 10 ** rng.uniform(4, 5, n) / 9.0 / orc.MHI_TO_JY
    return dict(x=x, y=y, ranges=ranges, h_eff=h * resc, kidx=kidx, v=v, sigma=sig, amp=amp,
                edges=edges, nx=nx, ny=ny, nc=nc)


@pytest.mark.parametrize("form", [0, 2, 3], ids=["fp32", "f16x3", "bf16x6"])
def test_noalloc_matches_workspace_insert_twice(form):
    """Two calls in a row, each against mg_insert on a caller workspace, in
    every form held to the parity bar (the tensor-core forms also exercise
    the spectrum store's share of the built-in array)."""
    from martini_gb300 import _native as N
    from martini_gb300.engine import DeviceParticles, InsertionEngine
    c = _problem_inputs()
    eng = InsertionEngine("cuda:0")
    dev = eng.device
    parts = DeviceParticles.from_host(dev, c["x"], c["y"], c["ranges"], c["h_eff"], c["kidx"],
                                      v=c["v"], sigma=c["sigma"], amp=c["amp"])
    edges = torch.from_numpy(c["edges"]).to(dev)
    table = [(N.MG_KERNEL_WENDLAND_C2, 0.0), (N.MG_KERNEL_DIRAC, 0.0), (N.MG_KERNEL_GAUSSIAN, 6.0)]
    ref, ref_flux = eng.insert(parts, table, N.MG_SPECTRUM_GAUSSIAN, 0.0, c["nx"], c["ny"], c["nc"],
                               edges, form=form)
    ref = ref.cpu().numpy().astype(np.float64)
    ref_flux = ref_flux.cpu().numpy()
    peak = np.abs(ref).max()
    assert peak > 0
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    for call in range(2):
        cube = torch.full((c["nx"], c["ny"], c["nc"]), -1.0, dtype=torch.float32, device=dev)
        flux = torch.empty(c["nc"] + 1, dtype=torch.float64, device=dev)
        prob = eng.problem(parts, table, N.MG_SPECTRUM_GAUSSIAN, 0.0, c["nx"], c["ny"], c["nc"],
                           0, 0, edges, cube, flux, form)
        rc = eng.lib.mg_insert_noalloc(C.byref(prob), stream)
        assert rc == N.MG_OK, eng.lib.mg_last_error()
        got = cube.cpu().numpy().astype(np.float64)
        assert np.abs(got - ref).max() / peak <= TOL_PEAK, f"call {call}"
        fl = flux.cpu().numpy()
        assert abs(fl[0] - ref_flux[0]) / ref_flux[0] <= TOL_FLUX, f"call {call}"


def test_noalloc_reports_pair_overflow_of_the_builtin_scratch():
    """A dense problem whose binning needs more (tile, particle) pairs than
    the built-in array holds (200k particles of ~100-pixel footprints over a
    128 x 128 cube: ~18M pairs) is refused after the binning with a message
    that names the built-in scratch, not a caller workspace."""
    from martini_gb300 import _native as N
    from martini_gb300.engine import DeviceParticles, InsertionEngine
    rng = np.random.default_rng(3)
    n, nx, ny, nc = 200_000, 128, 128, 16
    h = np.full(n, 30.0)
    kernels = orc.adaptive_tuple("WendlandC2Kernel")
    kidx, size, resc = orc.select_kernels(kernels, h)
    eng = InsertionEngine("cuda:0")
    dev = eng.device
    parts = DeviceParticles.from_host(dev, rng.uniform(50, 78, n), rng.uniform(50, 78, n),
                                      orc.sm_ranges(h, size), h * resc, kidx,
                                      v=rng.normal(100, 5, n), sigma=np.full(n, 5.0),
                                      amp=np.full(n, 1e-6))
    edges = torch.from_numpy(orc.vrad_channel_edges(nc, 4.0, 100.0)).to(dev)
    table = [(N.MG_KERNEL_WENDLAND_C2, 0.0), (N.MG_KERNEL_DIRAC, 0.0), (N.MG_KERNEL_GAUSSIAN, 6.0)]
    cube = torch.empty((nx, ny, nc), dtype=torch.float32, device=dev)
    prob = eng.problem(parts, table, N.MG_SPECTRUM_GAUSSIAN, 0.0, nx, ny, nc, 0, 0, edges, cube,
                       None, N.MG_FORM_FP32)
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    rc = eng.lib.mg_insert_noalloc(C.byref(prob), stream)
    assert rc == N.MG_ERR_WORKSPACE
    msg = eng.lib.mg_last_error().decode()
    assert "built-in scratch" in msg and "mg_insert with a workspace" in msg, msg


def test_noalloc_rejects_problem_beyond_scratch():
    from martini_gb300 import _native as N
    lib = N.load()
    p = N.Problem()
    # 10M particle records alone exceed the built-in scratch: refused before
    # any device memory is touched
    p.n, p.nx, p.ny, p.nc = 10_000_000, 64, 64, 32
    rc = lib.mg_insert_noalloc(C.byref(p), None)
    assert rc == N.MG_ERR_WORKSPACE
    msg = lib.mg_last_error().decode()
    assert "too large" in msg and str(N.MG_NOALLOC_SCRATCH_BYTES) in msg
