"""Generate golden vectors by running the reference's own hot-path code.

The reference (kyleaoman/martini, package ``astromartini``) imports astropy at
module level; astropy is not installed here.  This script therefore loads the
reference modules ``martini/sph_kernels.py``, ``martini/spectral_models.py``
and ``martini/martini.py`` straight from the reference source tree with a
small dimensionless units shim standing in for ``astropy.units`` (every unit
is the number 1 and quantities are plain float arrays).  All inputs are given
in one consistent unit system (pixels, km/s, Msun, Mpc), so every unit
conversion on the exercised lines is the identity and the reference's own
arithmetic runs unchanged:

* kernel constants from ``find_fwhm`` / ``__init__`` (sph_kernels.py:14-48, ...),
* ``_kernel_integral`` of every simple kernel and ``_px_weight``,
* adaptive kernel selection ``_AdaptiveKernel._init_sm_lengths``
  (sph_kernels.py:1241-1274; only the FP64 angular-size step of the base
  class, sph_kernels.py:235-255, is fed precomputed pixel sizes),
* ``_init_sm_ranges``, ``_prune_particles`` (martini.py:168-241),
* ``_BaseSpectrum.init_spectra`` for GaussianSpectrum / DiracDeltaSpectrum
  (spectral_models.py:63-200),
* ``_BaseMartini._evaluate_pixel_spectrum`` for every pixel of the cube
  (martini.py:243-283).

Projection from simulation coordinates to pixel coordinates needs astropy's
WCS and is not exercised: pixel coordinates and line-of-sight velocities are
inputs of each case.  The only restated step is the final Jy/pix^2 ->
Jy/arcsec^2 division (martini.py:364-366), which the fixtures leave undone
(cubes are stored in Jy/pix^2).

Run from the repository root:  python tests/golden/make_golden.py
It writes ``tests/golden/*.npz``.  It needs the reference checkout at
/root/reference and is not used at test time.
"""

from __future__ import annotations

import importlib.util
import os
import sys
import types

import numpy as np

REF = os.environ.get("MARTINI_REFERENCE", "/root/reference")
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import martini_oracle as orc  # noqa: E402  (case generation helpers)


# ---------------------------------------------------------------------------
# dimensionless units shim
# ---------------------------------------------------------------------------


class Q(np.ndarray):
    """Float array standing in for an astropy Quantity in a fixed unit system."""

    unit = 1.0

    def __new__(cls, a):
        return np.asarray(a, dtype=np.float64).view(cls)

    def to_value(self, *args, **kwargs):
        return np.asarray(self)

    def to(self, *args, **kwargs):
        return self

    def __lshift__(self, other):
        return self

    def __ilshift__(self, other):
        return self

    def __eq__(self, other):
        # ``sigma_mode == "thermal"`` (spectral_models.py:480) on a per-particle
        # width array: a quantity never equals a mode string.
        if isinstance(other, str):
            return False
        return np.ndarray.__eq__(self, other)

    __hash__ = None

    @property
    def isscalar(self):
        return self.ndim == 0


def _install_shims():
    units = types.ModuleType("astropy.units")
    for name in ("pix", "kpc", "Mpc", "km", "s", "m", "Msun", "Jy", "arcsec", "deg",
                 "K", "Hz", "rad", "beam", "dimensionless_unscaled"):
        setattr(units, name, 1.0)
    units.Quantity = Q
    units.Unit = lambda *a, **k: 1.0
    units.pixel_scale = lambda *a, **k: None
    units.get_physical_type = lambda *a, **k: "dimensionless"
    astropy = types.ModuleType("astropy")
    astropy.units = units
    astropy.__version__ = "shim"
    consts = types.ModuleType("astropy.constants")
    # sqrt(k_B T / m_p) is evaluated by the reference in m/s and converted to
    # km/s by ``.to``; the shim folds that 1e-3 into k_B (CODATA 2018 values).
    consts.k_B = Q(orc.K_B * 1e-6)
    consts.m_p = Q(orc.M_P)
    astropy.constants = consts
    mods = {
        "astropy": astropy,
        "astropy.units": units,
        "astropy.constants": consts,
    }
    for name in ("astropy.io", "astropy.io.fits", "astropy.time", "astropy.coordinates"):
        mods[name] = types.ModuleType(name)
    mods["astropy.io"].fits = mods["astropy.io.fits"]
    mods["astropy.time"].Time = object
    mods["astropy.coordinates"].Angle = object
    # stubs of reference modules that the hot path does not execute
    pkg = types.ModuleType("martini")
    pkg.__path__ = [os.path.join(REF, "martini")]
    mods["martini"] = pkg
    ver = types.ModuleType("martini.__version__")
    ver.__version__ = "2.1.18"
    mods["martini.__version__"] = ver
    for name, attrs in (
        ("martini.sources", ("SPHSource", "CombinedSource")),
        ("martini.datacube", ("DataCube", "_GlobalProfileDataCube")),
        ("martini.beams", ("_BaseBeam",)),
        ("martini.noise", ("_BaseNoise",)),
    ):
        m = types.ModuleType(name)
        for a in attrs:
            setattr(m, a, type(a, (), {}))
        mods[name] = m
    mods["martini.datacube"].HIfreq = 1.420405751e9
    sys.modules.update(mods)


def _load(modname, relpath):
    spec = importlib.util.spec_from_file_location(modname, os.path.join(REF, relpath))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[modname] = mod
    spec.loader.exec_module(mod)
    return mod


_install_shims()
SK = _load("martini.sph_kernels", "martini/sph_kernels.py")
SM = _load("martini.spectral_models", "martini/spectral_models.py")
MM = _load("martini.martini", "martini/martini.py")


def _base_init_sm_lengths(self, source, datacube):
    # The angular size step (sph_kernels.py:235-255) needs astropy; the case
    # supplies the smoothing lengths already in pixels.
    self.sm_lengths = Q(source.h_px)


SK._BaseSPHKernel._init_sm_lengths = _base_init_sm_lengths


# ---------------------------------------------------------------------------
# fake source / datacube carrying exactly the attributes the hot path reads
# ---------------------------------------------------------------------------


class FakeSkyCoords:
    def __init__(self, v, d):
        self.radial_velocity = Q(v)
        self.distance = Q(d)

    def __getitem__(self, m):
        return FakeSkyCoords(self.radial_velocity[m], self.distance[m])


class FakeSource:
    def __init__(self, x, y, vchan, v, dist, mHI, h_px, T=None):
        self.pixcoords = Q(np.vstack((x, y, vchan)))
        self.skycoords = FakeSkyCoords(v, dist)
        self.distance = Q(dist[0] if np.ndim(dist) else dist)
        self.mHI_g = Q(mHI)
        self.h_px = np.asarray(h_px, dtype=np.float64)
        self.T_g = None if T is None else Q(T)
        self.npart = len(x)
        self.input_mass = float(np.sum(mHI))

    def apply_mask(self, mask):
        if mask.sum() == 0:
            raise RuntimeError("No non-zero mHI source particles in target region.")
        self.pixcoords = self.pixcoords[:, mask]
        self.skycoords = self.skycoords[mask]
        self.mHI_g = self.mHI_g[mask]
        self.h_px = self.h_px[mask]
        if self.T_g is not None:
            self.T_g = self.T_g[mask]
        self.npart = int(mask.sum())


class FakeCube:
    def __init__(self, nx, ny, nc, edges_kms, pad=0):
        self.n_px_x, self.n_px_y, self.n_channels = nx, ny, nc
        self.padx = self.pady = pad
        self.velocity_channel_edges = Q(edges_kms)


def make_kernel(spec):
    kind, arg = spec
    cls = getattr(SK, kind)
    return cls(arg) if arg is not None else cls()


def sigma_to_T(sigma_kms):
    """Temperature whose thermal width sqrt(k_B T / m_p) is ``sigma_kms``."""
    return (np.asarray(sigma_kms, dtype=np.float64) * 1e3) ** 2 * orc.M_P / orc.K_B


def make_spectral(spec, sigma):
    """GaussianSpectrum: a scalar width is a fixed ``sigma``; a per-particle
    width goes through the reference's thermal branch (its widths follow the
    particle mask in pruning)."""
    if spec == "gaussian":
        if np.ndim(sigma) == 0:
            return SM.GaussianSpectrum(sigma=Q(sigma))
        return SM.GaussianSpectrum(sigma="thermal")
    return SM.DiracDeltaSpectrum()


def run_case(name, x, y, vchan, v, dist, mHI, h_px, kernel_spec, spectral, sigma,
             nx, ny, nc, edges_kms, pad=0, prune=True):
    T = sigma_to_T(sigma) if (sigma is not None and np.ndim(sigma) == 1) else None
    src = FakeSource(x, y, vchan, v, np.broadcast_to(dist, x.shape).astype(float), mHI, h_px,
                     T=T)
    cube = FakeCube(nx, ny, nc, edges_kms, pad)
    k = make_kernel(kernel_spec)
    sm = make_spectral(spectral, sigma)
    self = types.SimpleNamespace(source=src, _datacube=cube, sph_kernel=k,
                                 spectral_model=sm, quiet=True)
    k._init_sm_lengths(source=src, datacube=cube)
    k._init_sm_ranges()
    n_before = src.npart
    if prune:
        MM._BaseMartini._prune_particles(self)
    kept = np.asarray(src.pixcoords)
    sm.init_spectra(src, cube)
    out = np.zeros((nx + 2 * pad, ny + 2 * pad, nc))
    for i in range(out.shape[0]):
        for j in range(out.shape[1]):
            out[i, j] = np.asarray(MM._BaseMartini._evaluate_pixel_spectrum(self, (i, j)))
    rec = dict(
        name=name,
        x=x, y=y, vchan=vchan, v=v, dist=np.broadcast_to(dist, x.shape).astype(float),
        mHI=mHI, h_px=h_px, sigma=np.broadcast_to(sigma, x.shape).astype(float)
        if sigma is not None else np.zeros(0),
        T=T if T is not None else np.zeros(0),
        edges=edges_kms, nx=nx, ny=ny, nc=nc, pad=pad,
        kernel=np.array(kernel_spec[0]), kernel_arg=np.array(
            kernel_spec[1] if kernel_spec[1] is not None else np.nan),
        spectral=np.array(spectral),
        n_before=n_before, n_after=src.npart,
        kept_x=kept[0], kept_y=kept[1],
        sm_lengths=np.asarray(k.sm_lengths), sm_ranges=np.asarray(k.sm_ranges),
        kernel_indices=np.asarray(getattr(k, "kernel_indices", np.zeros(src.npart, int))),
        rescale=np.broadcast_to(np.asarray(k._rescale, dtype=float), (src.npart,)).copy(),
        spectra=np.asarray(sm.spectra),
        cube=out,
    )
    np.savez_compressed(os.path.join(HERE, f"cube_{name}.npz"), **rec)
    print(f"{name}: N {n_before}->{src.npart}, peak {out.max():.4e}, sum {out.sum():.6e}")


# ---------------------------------------------------------------------------
# cases
# ---------------------------------------------------------------------------


def kernel_vectors():
    """_kernel_integral of every simple kernel on a grid of offsets/sizes, and
    the constants each kernel's constructor derives."""
    rng = np.random.default_rng(1234)
    n = 4000
    h = np.concatenate((np.full(200, 1.0), 10 ** rng.uniform(-1.5, 1.5, n - 200)))
    dx = rng.uniform(-1, 1, n) * (2.6 * h + 1.5)
    dy = rng.uniform(-1, 1, n) * (2.6 * h + 1.5)
    # exact special points: R = 0, half-pixel offsets, support edges
    dx[:50] = 0.0
    dy[:50] = 0.0
    dx[50:100] = 0.5
    dy[50:100] = rng.uniform(-0.49, 0.49, 50)
    dx[100:150] = -0.5
    dy[100:150] = 0.25
    dx[150:200] = rng.integers(-3, 4, 50).astype(float)
    dy[150:200] = rng.integers(-3, 4, 50).astype(float)
    dij = np.vstack((dx, dy))
    out = dict(dx=dx, dy=dy, h=h)
    specs = [("_WendlandC2Kernel", None), ("_WendlandC6Kernel", None),
             ("_CubicSplineKernel", None), ("_QuarticSplineKernel", None),
             ("_GaussianKernel", 2.0), ("_GaussianKernel", 3.0), ("_GaussianKernel", 4.0),
             ("_GaussianKernel", 5.0), ("_GaussianKernel", 6.0), ("DiracDeltaKernel", None)]
    for kind, arg in specs:
        k = make_kernel((kind, arg))
        key = kind + ("" if arg is None else f"_{arg:g}")
        out["w_" + key] = np.asarray(k._kernel_integral(Q(dij.copy()), Q(h.copy())))
        out["size_" + key] = np.array(float(k.size_in_fwhm))
        out["rescale_" + key] = np.array(float(k._rescale))
    # adaptive selection on the reference test's sizes (1 kpc pixels:
    # tests/test_sph_kernels.py:293-334) and on a dense sweep
    sweep = np.concatenate(([3.0, 1.0, 0.55, 0.1], np.linspace(0.01, 3.0, 600)))
    for name in ("WendlandC2Kernel", "WendlandC6Kernel", "CubicSplineKernel",
                 "QuarticSplineKernel", "GaussianKernel"):
        k = make_kernel((name, None))
        src = types.SimpleNamespace(h_px=sweep, mHI_g=Q(np.ones(sweep.size)))
        k._init_sm_lengths(source=src, datacube=None)
        k._init_sm_ranges()
        out["sel_idx_" + name] = np.asarray(k.kernel_indices)
        out["sel_size_" + name] = np.asarray(k.size_in_fwhm)
        out["sel_rescale_" + name] = np.asarray(k._rescale)
        out["sel_ranges_" + name] = np.asarray(k.sm_ranges)
    out["sel_h"] = sweep
    np.savez_compressed(os.path.join(HERE, "kernel_vectors.npz"), **out)
    print("kernel_vectors: ", len(specs), "kernels")


def spectra_vectors():
    """init_spectra of both spectral models on increasing and decreasing edges."""
    rng = np.random.default_rng(99)
    n = 300
    out = {}
    for tag, edges in (("vrad", orc.vrad_channel_edges(48, 4.0, 210.0)),
                       ("incr", np.linspace(150.0, 270.0, 41)),
                       ("freq", orc.freq_channel_edges(32, 20e3, 1.4194e9))):
        v = rng.uniform(edges.min() - 20, edges.max() + 20, n)
        v[:5] = edges[[3, 4, 5, 10, 20]]  # exactly on edges (Heaviside(0) = 1)
        sig = 10 ** rng.uniform(0.3, 1.3, n)
        mHI = 10 ** rng.uniform(3, 6, n)
        dist = rng.uniform(1.0, 20.0, n)
        for model in ("gaussian", "dirac"):
            src = FakeSource(np.zeros(n), np.zeros(n), np.zeros(n), v, dist, mHI, np.ones(n),
                             T=sigma_to_T(sig))
            cube = FakeCube(4, 4, edges.size - 1, edges)
            sm = make_spectral(model, sig)
            sm.init_spectra(src, cube)
            out[f"{model}_{tag}"] = np.asarray(sm.spectra)
        out[f"v_{tag}"] = v
        out[f"sigma_{tag}"] = sig
        out[f"mHI_{tag}"] = mHI
        out[f"dist_{tag}"] = dist
        out[f"edges_{tag}"] = edges
    np.savez_compressed(os.path.join(HERE, "spectra_vectors.npz"), **out)
    print("spectra_vectors")


def cubes():
    # cfg1-shaped case: 5000-particle disc, CubicSplineKernel, sigma 7 km/s,
    # 64 x 64 x 32 at 10 arcsec, 4 km/s, 3 Mpc (projected by the oracle's
    # restatement; projection itself is not what this fixture pins).
    g = orc.disc_particles(5000, seed=1)
    xyz, vxyz = orc.incline(g["xyz"], g["vxyz"], 60.0)
    D = 3.0
    ra, dec, vlos, dist = orc.project_particles(xyz, vxyz, D)
    px = 10.0 / 3600.0
    x, y = orc.tan_world2pix(ra, dec, 0.0, 0.0, 64 / 2 + 0.5, 64 / 2 + 0.5, -px, px)
    vsys = 0.7 * 100 * D
    edges = orc.vrad_channel_edges(32, 4.0, vsys)
    vchan = (32 / 2 + 0.5 - 1) + (vlos - vsys) / (-4.0)
    hpx = orc.sm_lengths_px(g["hsm"], dist, 10.0)
    run_case("cfg1_disc_cubic", x, y, vchan, vlos, dist, g["mHI"], hpx,
             ("CubicSplineKernel", None), "gaussian", 7.0, 64, 64, 32, edges)

    # every kernel x both spectral models on a 16 x 16 x 16 cube, 120 random
    # particles with sizes spanning the adaptive fallbacks, plus edge cases
    rng = np.random.default_rng(7)
    n = 120
    edges = orc.vrad_channel_edges(16, 4.0, 210.0)
    vmid = 0.5 * (edges[:-1] + edges[1:])
    for kspec in (("_WendlandC2Kernel", None), ("_WendlandC6Kernel", None),
                  ("_CubicSplineKernel", None), ("_QuarticSplineKernel", None),
                  ("_GaussianKernel", 3.0), ("DiracDeltaKernel", None),
                  ("WendlandC2Kernel", None), ("WendlandC6Kernel", None),
                  ("CubicSplineKernel", None), ("QuarticSplineKernel", None),
                  ("GaussianKernel", 3.0)):
        for spectral in ("gaussian", "dirac"):
            x = rng.uniform(-3, 19, n)
            y = rng.uniform(-3, 19, n)
            if kspec[0] == "DiracDeltaKernel":
                h = rng.uniform(0.05, 0.5, n)
            else:
                h = 10 ** rng.uniform(-1.0, 0.7, n)
            v = rng.uniform(edges.min() - 8, edges.max() + 8, n)
            # edge cases: pixel-centred, half-pixel, on channel edges
            x[:4] = [5.0, 7.5, 8.0, 0.0]
            y[:4] = [5.0, 3.0, 8.5, 0.0]
            v[4:8] = edges[[2, 5, 8, 11]]
            v[8:10] = vmid[[3, 9]]
            vchan = (16 / 2 + 0.5 - 1) + (v - 210.0) / (-4.0)
            mHI = 10 ** rng.uniform(4, 6, n)
            mHI[10] = 0.0  # pruned by mass
            sigma = 10 ** rng.uniform(0.3, 1.0, n)
            tag = (("simple_" if kspec[0].startswith("_") else "") + kspec[0].strip("_")
                   + ("" if kspec[1] is None else f"{kspec[1]:g}"))
            run_case(f"{tag}_{spectral}", x, y, vchan, v, 3.0 + 0 * x, mHI, h, kspec,
                     spectral, sigma, 16, 16, 16, edges)

    # padded cube, increasing edges, WendlandC2 + thermal-like per-particle sigma
    n = 400
    x = rng.normal(14, 5, n)
    y = rng.normal(12, 4, n)
    edges = np.linspace(180.0, 244.0, 33)
    v = rng.normal(212, 12, n)
    vchan = (v - edges[0]) / 2.0 - 0.5
    h = 10 ** rng.normal(0.4, 0.3, n)
    sigma = orc.thermal_sigma_kms(1e4 * 10 ** (0.3 * rng.normal(0, 1, n)))
    run_case("wc2_thermal_pad_incr", x, y, vchan, v, 3.0 + 0 * x, 10 ** rng.uniform(4, 5, n),
             h, ("WendlandC2Kernel", None), "gaussian", sigma, 20, 16, 32, edges, pad=3)


if __name__ == "__main__":
    kernel_vectors()
    spectra_vectors()
    cubes()
