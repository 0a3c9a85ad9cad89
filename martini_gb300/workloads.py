"""Seeded synthetic galaxies for the benchmark configurations.

No public dataset is used: each configuration is an exponential HI disc
drawn from one ``numpy.random.default_rng(seed)`` with a fixed draw order
(azimuth, radius ~ Gamma(2, R_d), height ~ N(0, z_d), isotropic velocity
dispersion, lognormal HI mass, smoothing length, temperature), placed with
the drop-in API (``SPHSource`` / ``DataCube`` / kernels / spectral model)
exactly as ``Martini.__init__`` does, so the arrays handed to the GPU are the
ones the reference's insertion would see.

Configurations (sizes of the reference workloads being accelerated):

* ``disc5k_64``: 5,000 particles, R_d 3 kpc, z 0.3 kpc, i = 60 deg, 3 Mpc,
  v_flat 200 km/s, dispersion 10 km/s, mHI 1e5 Msun (0.2 dex), h 1 kpc
  (0.3 dex); 64 x 64 px at 10 arcsec, 32 channels of 4 km/s;
  CubicSplineKernel, GaussianSpectrum(7 km/s).
* ``disc1m_512``: the same disc with 1,000,000 particles, WendlandC2Kernel,
  thermal widths from T lognormal (1e4 K, 0.3 dex); 512 x 512 x 256.
* ``disc4m_1024``: 4,000,000 particles, R_d 10 kpc at 10 Mpc, h 0.5 kpc
  (0.5 dex); 1024 x 1024 x 512 channels of 2 km/s; WendlandC2, thermal.
* ``stress16m_2048``: 16,000,000 particles (disc + 10 % of the mass in a
  Plummer sphere of scale 20 kpc), h log-uniform 0.05-20 kpc, WendlandC2;
  thermal Gaussian lines, with a seeded 20 % of the particles on Dirac
  lines (two spectral groups in one cube); 2048 x 2048 x 256.
* the disc population (``build_population``): 2000 galaxies of 1e3-1e6
  particles on cubes of 32^2 x 64 to 256^2 x 256, inserted as one batch.
"""

from __future__ import annotations

import numpy as np

from .datacube import DataCube
from .sources import SPHSource
from . import sph_kernels as K
from . import spectral_models as S

MHI_TO_JY = 2.36e5


def disc(n, seed, R_d=3.0, z_d=0.3, v_flat=200.0, v_disp=10.0, mHI_med=1e5, mHI_dex=0.2,
         h_med=1.0, h_dex=0.3, T_med=1e4, T_dex=0.3, h_loguniform=None):
    """Face-on exponential disc in the x-y plane (kpc, km/s, Msun, K)."""
    rng = np.random.default_rng(seed)
    phi = rng.uniform(0, 2 * np.pi, n)
    R = rng.gamma(2.0, R_d, n)
    z = rng.normal(0.0, z_d, n)
    disp = rng.normal(0.0, v_disp, (n, 3))
    mHI = mHI_med * 10 ** (mHI_dex * rng.normal(0, 1, n))
    if h_loguniform is None:
        hsm = h_med * 10 ** (h_dex * rng.normal(0, 1, n))
    else:
        lo, hi = h_loguniform
        hsm = 10 ** rng.uniform(np.log10(lo), np.log10(hi), n)
    T = T_med * 10 ** (T_dex * rng.normal(0, 1, n))
    vphi = v_flat * np.arctan(R / 1.0) / (np.pi / 2)
    xyz = np.stack((R * np.cos(phi), R * np.sin(phi), z), axis=1)
    vxyz = np.stack((-vphi * np.sin(phi), vphi * np.cos(phi), np.zeros(n)), axis=1) + disp
    return dict(xyz=xyz, vxyz=vxyz, mHI=mHI, hsm=hsm, T=T, rng=rng)


def incline(xyz, vxyz, incl_deg):
    """Disc normal (z) to the line of sight (x), then tilt by incl about y."""
    M0 = np.array([[0, 0, 1], [1, 0, 0], [0, 1, 0]], dtype=np.float64)
    i = np.deg2rad(incl_deg)
    Ry = np.array([[np.cos(i), 0, np.sin(i)], [0, 1, 0], [-np.sin(i), 0, np.cos(i)]])
    M = Ry @ M0
    return xyz @ M.T, vxyz @ M.T


def plummer(n, a, rng, v_disp=30.0):
    """Plummer sphere positions (kpc) with isotropic Gaussian velocities."""
    m = rng.uniform(0, 1, n)
    r = a / np.sqrt(m ** (-2.0 / 3.0) - 1.0)
    r = np.minimum(r, 20 * a)
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    return u * r[:, None], rng.normal(0, v_disp, (n, 3))


CONFIGS = {
    "disc5k_64": dict(n=5000, seed=1, D=3.0, incl=60.0, nx=64, nc=32, dv=4.0, px=10.0,
                      kernel="CubicSplineKernel", spectrum=("gaussian", 7.0), disc={}),
    "disc1m_512": dict(n=1_000_000, seed=2, D=3.0, incl=60.0, nx=512, nc=256, dv=4.0, px=10.0,
                       kernel="WendlandC2Kernel", spectrum=("thermal", None), disc={}),
    "disc4m_1024": dict(n=4_000_000, seed=3, D=10.0, incl=60.0, nx=1024, nc=512, dv=2.0, px=10.0,
                        kernel="WendlandC2Kernel", spectrum=("thermal", None),
                        disc=dict(R_d=10.0, h_med=0.5, h_dex=0.5)),
    "stress16m_2048": dict(n=16_000_000, seed=5, D=3.0, incl=60.0, nx=2048, nc=256, dv=4.0,
                           px=10.0, kernel="WendlandC2Kernel", spectrum=("thermal", None),
                           disc=dict(h_loguniform=(0.05, 20.0)), plummer=0.1,
                           dirac_fraction=0.2),
}


def build(name: str, n: int | None = None):
    """Particles of a configuration after ``Martini.__init__`` set-up.

    Returns a dict of host arrays (x, y, sm_range, h_eff, kernel_index, v,
    sigma, amp), the kernel table, the spectral model code, the channel
    edges and the cube shape.  ``n`` overrides the particle count (for
    scaled-down tests of the same configuration).
    """
    cfg = dict(CONFIGS[name])
    n = cfg["n"] if n is None else int(n)
    return _assemble(name, cfg, n)


def _assemble(name: str, cfg: dict, n: int):
    from . import _native as N
    g = disc(n, cfg["seed"], **cfg["disc"])
    xyz, vxyz = incline(g["xyz"], g["vxyz"], cfg["incl"])
    if cfg.get("plummer"):
        nh = int(round(cfg["plummer"] * n))
        hx, hv = plummer(nh, 20.0, g["rng"])
        xyz[:nh], vxyz[:nh] = hx, hv
    src = SPHSource(distance=cfg["D"], T_g=g["T"], mHI_g=g["mHI"], xyz_g=xyz, vxyz_g=vxyz,
                    hsm_g=g["hsm"])
    nx = cfg["nx"]
    dc = DataCube(n_px_x=nx, n_px_y=nx, n_channels=cfg["nc"], px_size=cfg["px"],
                  channel_width=cfg["dv"], spectral_centre=src.vsys)
    kern = getattr(K, cfg["kernel"])()
    kind, sig = cfg["spectrum"]
    sm = (S.GaussianSpectrum(sig if kind == "gaussian" else "thermal") if kind != "dirac"
          else S.DiracDeltaSpectrum())
    # Martini.__init__ set-up without a GPU (martini/martini.py:118-151)
    from .martini import _BaseMartini
    m = _BaseMartini.__new__(_BaseMartini)
    m.quiet, m.source, m._datacube, m.sph_kernel, m.spectral_model = True, src, dc, kern, sm
    src._init_skycoords()
    src._init_pixcoords(dc)
    kern._init_sm_lengths(source=src, datacube=dc)
    kern._init_sm_ranges()
    m._prune_particles()
    h_eff, kidx = kern._device_arrays()
    sigma, sig_const = sm._device_sigma(src)
    amp = src.mHI_g * np.power(src.skycoords.distance, -2.0) / MHI_TO_JY
    # two spectral groups in one cube: a seeded subset with Dirac lines, the
    # rest Gaussian (inserted by two calls, the second adding to the first)
    groups = None
    if cfg.get("dirac_fraction"):
        pick = np.random.default_rng(cfg["seed"] + 1000).random(src.npart) < cfg["dirac_fraction"]
        groups = [dict(sel=np.flatnonzero(~pick), spectral_model=sm.native_model),
                  dict(sel=np.flatnonzero(pick), spectral_model=N.MG_SPECTRUM_DIRAC)]
    return dict(
        groups=groups,
        name=name, n_input=n, n=src.npart, x=src.pixcoords[0], y=src.pixcoords[1],
        sm_range=kern.sm_ranges, h_eff=h_eff, kernel_index=kidx,
        v=src.skycoords.radial_velocity, sigma=sigma, sigma_const=sig_const, amp=amp,
        kernels=kern._device_kernels(), spectral_model=sm.native_model,
        edges=dc.velocity_channel_edges, nx=nx, ny=nx, nc=cfg["nc"], px_size=cfg["px"],
        distance=cfg["D"], mHI=src.mHI_g, dist=src.skycoords.distance,
        spectral_kind=kind if groups is None else f"{kind} + {cfg['dirac_fraction']:.0%} dirac",
        kernel_name=cfg["kernel"], native_form_default=N.MG_FORM_FP32)


# The disc population: 2000 galaxies, N log-uniform in 1e3-1e6, cos i
# uniform, v_flat uniform in 50-300 km/s, each on one cube drawn from
# {32^2 x 64, 64^2 x 128, 128^2 x 128, 256^2 x 256} at 4 km/s; distance,
# pixel size, kernel and line widths as the single-disc configurations.
POPULATION = dict(n_gal=2000, seed=4, logn=(3.0, 6.0), v_flat=(50.0, 300.0),
                  cubes=((32, 64), (64, 128), (128, 128), (256, 256)), D=3.0, dv=4.0, px=10.0,
                  kernel="WendlandC2Kernel", spectrum=("thermal", None))


def population_configs(n_gal: int | None = None, seed: int | None = None):
    """Per-galaxy configurations of the disc population (one seeded draw
    order: log N, cos i, v_flat, cube)."""
    P = POPULATION
    n_gal = P["n_gal"] if n_gal is None else int(n_gal)
    seed = P["seed"] if seed is None else int(seed)
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_gal):
        n = int(round(10 ** rng.uniform(*P["logn"])))
        incl = float(np.rad2deg(np.arccos(rng.uniform(0.0, 1.0))))
        vf = float(rng.uniform(*P["v_flat"]))
        nx, nc = P["cubes"][int(rng.integers(0, len(P["cubes"])))]
        out.append(dict(n=n, seed=seed * 100003 + k, D=P["D"], incl=incl, nx=nx, nc=nc,
                        dv=P["dv"], px=P["px"], kernel=P["kernel"], spectrum=P["spectrum"],
                        disc=dict(v_flat=vf)))
    return out


def _assemble_one(args):
    k, cfg = args
    return _assemble(f"pop{k}", cfg, cfg["n"])


def build_population(n_gal: int | None = None, seed: int | None = None, workers: int = 0):
    """The galaxies of the disc population, each as :func:`build` returns it.
    ``workers`` > 1 builds them in a spawn-started process pool."""
    cfgs = population_configs(n_gal, seed)
    jobs = list(enumerate(cfgs))
    if workers and workers > 1:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(workers) as pool:
            return pool.map(_assemble_one, jobs, chunksize=4)
    return [_assemble_one(j) for j in jobs]


def footprint_pixels(x, y, r, nx, ny):
    """Box-footprint pixel count per particle, clipped to the cube: the
    number of (pixel, particle) pairs the reference's mask selects
    (martini/martini.py:272-274)."""
    def span(c, n):
        lo = np.maximum(np.ceil(c - r), 0)
        hi = np.minimum(np.floor(c + r), n - 1)
        return np.maximum(hi - lo + 1, 0)
    return span(x, nx) * span(y, ny)
