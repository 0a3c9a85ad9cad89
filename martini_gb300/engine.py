"""Device-side insertion engine: owns the workspace and drives the C ABI.

``InsertionEngine.insert`` takes particle arrays already on the GPU (torch
tensors), runs ``mg_plan`` (footprint binning, sizes the workspace; one
host synchronisation) and ``mg_insert`` (everything else, asynchronous) on
the current CUDA stream, and returns the float32 cube and FP64 flux sums on
the device.  PyTorch supplies device memory and streams only; all compute
is in ``libmartini_gb300.so``.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as N


@dataclass
class DeviceParticles:
    """Particle inputs in device memory (one entry per particle)."""

    x: torch.Tensor                      # f64 pixel coordinate, axis 0
    y: torch.Tensor                      # f64 pixel coordinate, axis 1
    sm_range: torch.Tensor               # f64 footprint half-width, px
    h_eff: torch.Tensor                  # f32 sm_length * rescale, px
    kernel_index: torch.Tensor | None    # i8 kernel table index (-1 -> 0) or None
    v: torch.Tensor | None = None        # f64 line-of-sight velocity, km/s
    sigma: torch.Tensor | None = None    # f32 Gaussian width, km/s
    amp: torch.Tensor | None = None      # f64 mHI / D^2 / 2.36e5
    spectra: torch.Tensor | None = None  # f32 [n, nc] (table model)

    @property
    def n(self) -> int:
        return int(self.x.shape[0])

    @staticmethod
    def from_host(device, x, y, sm_range, h_eff, kernel_index=None, v=None, sigma=None, amp=None,
                  spectra=None) -> "DeviceParticles":
        def put(a, dt):
            if a is None:
                return None
            t = torch.from_numpy(np.ascontiguousarray(a, dtype=dt))
            if device.type == "cuda":
                t = t.pin_memory().to(device, non_blocking=True)
            return t
        return DeviceParticles(put(x, np.float64), put(y, np.float64), put(sm_range, np.float64),
                               put(h_eff, np.float32), put(kernel_index, np.int8),
                               put(v, np.float64), put(sigma, np.float32), put(amp, np.float64),
                               put(spectra, np.float32))


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


class InsertionEngine:
    """Owns a reusable device workspace for repeated insertions."""

    def __init__(self, device=None):
        if not torch.cuda.is_available():
            raise RuntimeError("martini_gb300 needs a CUDA GPU (no CPU fallback)")
        self.lib = N.load()
        self.device = torch.device(device) if device is not None else torch.device(
            "cuda", torch.cuda.current_device())
        self._ws = None
        self._caps = (0, 0)
        self.last_plan = None

    # ---- problem description ------------------------------------------------
    def problem(self, parts: DeviceParticles, kernels, spectral_model: int, sigma_const: float,
                nx: int, ny: int, nc: int, padx: int, pady: int, edges: torch.Tensor,
                cube: torch.Tensor, flux: torch.Tensor | None, form: int,
                accumulate: bool = False) -> N.Problem:
        p = N.Problem()
        p.n = parts.n
        p.x, p.y, p.sm_range = _ptr(parts.x), _ptr(parts.y), _ptr(parts.sm_range)
        p.h_eff, p.kernel_index = _ptr(parts.h_eff), _ptr(parts.kernel_index)
        if not 1 <= len(kernels) <= N.MG_MAX_KERNELS:
            raise ValueError("1 to 4 kernels")
        p.n_kernels = len(kernels)
        for k, (t, trunc) in enumerate(kernels):
            p.kernels[k].type = int(t)
            p.kernels[k].truncate = float(trunc)
        p.spectral_model = int(spectral_model)
        p.v, p.sigma, p.amp, p.spectra = (_ptr(parts.v), _ptr(parts.sigma), _ptr(parts.amp),
                                          _ptr(parts.spectra))
        p.sigma_const = float(sigma_const)
        p.nx, p.ny, p.nc, p.padx, p.pady = int(nx), int(ny), int(nc), int(padx), int(pady)
        p.edges = _ptr(edges)
        p.cube = _ptr(cube)
        p.flux = _ptr(flux)
        p.form = int(form)
        p.accumulate = int(bool(accumulate))
        return p

    def _workspace(self, nbytes: int) -> torch.Tensor:
        if self._ws is None or self._ws.numel() < nbytes:
            self._ws = torch.empty(max(nbytes, 1 << 16), dtype=torch.uint8, device=self.device)
        return self._ws

    def plan(self, prob: N.Problem, stream=None) -> N.PlanInfo:
        """Bin the particles and size the workspace (synchronises the stream)."""
        s = stream or torch.cuda.current_stream(self.device)
        base = C.c_size_t()
        N.check(self.lib.mg_workspace_size(C.byref(prob), 0, 0, C.byref(base)))
        ws = self._workspace(base.value)
        info = N.PlanInfo()
        N.check(self.lib.mg_plan(C.byref(prob), C.c_void_p(ws.data_ptr()), ws.numel(),
                                 C.c_void_p(s.cuda_stream), C.byref(info)))
        self._caps = (int(info.n_pairs), int(info.n_partial_items))
        # the plan's size includes the spectrum store of the tensor-core forms
        self._workspace(int(info.workspace_bytes))
        self.last_plan = info
        return info

    def tune(self, prob: N.Problem, reps: int = 3, stream=None) -> dict:
        """Autotune the launch shape of ``prob`` (after :meth:`plan`): every
        candidate is binned and its contraction timed ``reps`` times; the
        fastest is cached for the problem's class, so later runs and
        captures of this (or a like) problem use it.  Synchronises and
        overwrites the cube.  Returns the shape and its median time (ms)."""
        s = stream or torch.cuda.current_stream(self.device)
        ws = self._ws
        best = N.Tuning()
        ms = C.c_float()
        N.check(self.lib.mg_tune(C.byref(prob), C.c_void_p(ws.data_ptr()), ws.numel(),
                                 self._caps[0], self._caps[1], int(reps),
                                 C.c_void_p(s.cuda_stream), C.byref(best), C.byref(ms)))
        out = best.as_dict()
        out["contract_ms"] = float(ms.value)
        return out

    def run(self, prob: N.Problem, stream=None) -> None:
        """Full insertion with the capacities of the last plan (asynchronous)."""
        s = stream or torch.cuda.current_stream(self.device)
        ws = self._ws
        N.check(self.lib.mg_insert(C.byref(prob), C.c_void_p(ws.data_ptr()), ws.numel(),
                                   self._caps[0], self._caps[1], C.c_void_p(s.cuda_stream)))

    def capture(self, prob: N.Problem) -> "torch.cuda.CUDAGraph":
        """Capture mg_insert of ``prob`` (after :meth:`plan`) in a CUDA graph:
        ``graph.replay()`` then runs the whole insertion as one launch.  The
        problem's buffers and this engine's workspace must stay in place."""
        self.run(prob)  # first call sets the kernels' attributes outside the capture
        torch.cuda.synchronize(self.device)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            self.run(prob)
        return graph

    def run_stages(self, prob: N.Problem, stages: int, stream=None) -> None:
        """Some stages of mg_insert (N.MG_STAGE_* bits), asynchronous."""
        s = stream or torch.cuda.current_stream(self.device)
        ws = self._ws
        N.check(self.lib.mg_insert_stages(C.byref(prob), C.c_void_p(ws.data_ptr()), ws.numel(),
                                          self._caps[0], self._caps[1], int(stages),
                                          C.c_void_p(s.cuda_stream)))

    def check(self, stream=None) -> None:
        s = stream or torch.cuda.current_stream(self.device)
        N.check(self.lib.mg_check(C.c_void_p(self._ws.data_ptr()), C.c_void_p(s.cuda_stream)))

    def insert(self, parts: DeviceParticles, kernels, spectral_model: int, sigma_const: float,
               nx: int, ny: int, nc: int, edges: torch.Tensor, padx: int = 0, pady: int = 0,
               form: int = N.MG_FORM_FP32, cube: torch.Tensor | None = None, flux: bool = True,
               plan: bool = True, check: bool = True, accumulate: bool = False):
        """Insert particles into a (nx, ny, nc) float32 cube (Jy/pix^2).

        Returns (cube, flux) device tensors; flux[0] is the total flux in Jy
        over the unpadded region and flux[1:] the per-channel sums (of the
        whole cube, so in accumulate mode including what it held before).
        ``accumulate`` adds the insertion to ``cube`` instead of overwriting.
        """
        if accumulate and cube is None:
            raise ValueError("accumulate needs the cube to add into")
        if cube is None:
            cube = torch.empty((nx, ny, nc), dtype=torch.float32, device=self.device)
        fl = torch.empty(nc + 1, dtype=torch.float64, device=self.device) if flux else None
        prob = self.problem(parts, kernels, spectral_model, sigma_const, nx, ny, nc, padx, pady,
                            edges, cube, fl, form, accumulate)
        if plan or self._ws is None:
            self.plan(prob)
        self.run(prob)
        if check:
            self.check()
        return cube, fl

    def spectra(self, parts: DeviceParticles, spectral_model: int, sigma_const: float, nc: int,
                edges: torch.Tensor) -> torch.Tensor:
        """Materialised spectra [n, nc] (Jy) of a GAUSSIAN/DIRAC model."""
        out = torch.empty((parts.n, nc), dtype=torch.float32, device=self.device)
        dummy = torch.empty(1, dtype=torch.float32, device=self.device)
        prob = self.problem(parts, [(N.MG_KERNEL_DIRAC, 0.0)], spectral_model, sigma_const, 1, 1,
                            nc, 0, 0, edges, dummy, None, N.MG_FORM_FP32)
        N.check(self.lib.mg_spectra(C.byref(prob), C.c_void_p(out.data_ptr()),
                                    C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)))
        return out


class BatchInsertion:
    """Many cubes in one insertion (``mg_insert_batched``): one binning pass
    and one persistent contraction over the tiles of every cube.

    ``probs`` are Problems built with :meth:`InsertionEngine.problem`; the
    tensors they point to must outlive this object (``keep`` holds them)."""

    def __init__(self, engine: InsertionEngine, probs, keep=None):
        if not probs:
            raise ValueError("empty batch")
        self.eng = engine
        self.lib = engine.lib
        self.n = len(probs)
        self.arr = (N.Problem * self.n)(*probs)
        self.keep = keep
        self._ws = None
        self._caps = (0, 0)
        self.last_plan = None

    def _stream(self, stream):
        s = stream or torch.cuda.current_stream(self.eng.device)
        return C.c_void_p(s.cuda_stream)

    def _workspace(self, nbytes: int) -> torch.Tensor:
        if self._ws is None or self._ws.numel() < nbytes:
            self._ws = torch.empty(max(nbytes, 1 << 16), dtype=torch.uint8, device=self.eng.device)
        return self._ws

    def plan(self, stream=None) -> N.PlanInfo:
        """Bin every cube and size the workspace (synchronises the stream)."""
        base = C.c_size_t()
        N.check(self.lib.mg_workspace_size_batched(self.arr, self.n, 0, 0, C.byref(base)))
        ws = self._workspace(base.value)
        info = N.PlanInfo()
        N.check(self.lib.mg_plan_batched(self.arr, self.n, C.c_void_p(ws.data_ptr()), ws.numel(),
                                         self._stream(stream), C.byref(info)))
        self._caps = (int(info.n_pairs), int(info.n_partial_items))
        self._workspace(int(info.workspace_bytes))
        self.last_plan = info
        return info

    def tune(self, reps: int = 3, stream=None) -> dict:
        """Autotune the batch's launch shape (after :meth:`plan`; see
        :meth:`InsertionEngine.tune`): synchronises and overwrites the cubes."""
        ws = self._ws
        best = N.Tuning()
        ms = C.c_float()
        N.check(self.lib.mg_tune_batched(self.arr, self.n, C.c_void_p(ws.data_ptr()), ws.numel(),
                                         self._caps[0], self._caps[1], int(reps),
                                         self._stream(stream), C.byref(best), C.byref(ms)))
        out = best.as_dict()
        out["contract_ms"] = float(ms.value)
        return out

    def run(self, stream=None) -> None:
        ws = self._ws
        N.check(self.lib.mg_insert_batched(self.arr, self.n, C.c_void_p(ws.data_ptr()),
                                           ws.numel(), self._caps[0], self._caps[1],
                                           self._stream(stream)))

    def run_stages(self, stages: int, stream=None) -> None:
        ws = self._ws
        N.check(self.lib.mg_insert_stages_batched(self.arr, self.n, C.c_void_p(ws.data_ptr()),
                                                  ws.numel(), self._caps[0], self._caps[1],
                                                  int(stages), self._stream(stream)))

    def check(self, stream=None) -> None:
        N.check(self.lib.mg_check(C.c_void_p(self._ws.data_ptr()), self._stream(stream)))


def insert_batch(engine: InsertionEngine, items, kernels, spectral_model: int,
                 form: int = N.MG_FORM_FP32, flux: bool = True):
    """Insert several cubes in one batch.  ``items``: dicts with ``parts``
    (DeviceParticles), ``edges`` (device float64), ``nx``, ``ny``, ``nc`` and
    optionally ``padx``, ``pady``, ``sigma_const``, ``cube``.  Returns a list
    of (cube, flux) device tensors, one per item."""
    dev = engine.device
    probs, outs = [], []
    for it in items:
        nx, ny, nc = int(it["nx"]), int(it["ny"]), int(it["nc"])
        cube = it.get("cube")
        if cube is None:
            cube = torch.empty((nx, ny, nc), dtype=torch.float32, device=dev)
        fl = torch.empty(nc + 1, dtype=torch.float64, device=dev) if flux else None
        probs.append(engine.problem(it["parts"], kernels, spectral_model,
                                    float(it.get("sigma_const", 0.0)), nx, ny, nc,
                                    int(it.get("padx", 0)), int(it.get("pady", 0)), it["edges"],
                                    cube, fl, form))
        outs.append((cube, fl))
    b = BatchInsertion(engine, probs, keep=(items, outs))
    b.plan()
    b.run()
    b.check()
    return outs


def kernel_choice(sph_kernel) -> N.KernelChoice:
    """Validity rules and constants of an SPH kernel (adaptive tuple or single
    kernel) for the GPU kernel choice (sph_kernels.py:1241-1274)."""
    kc = N.KernelChoice()
    subs = getattr(sph_kernel, "kernels", None)
    kc.adaptive = 1 if subs else 0
    subs = subs or (sph_kernel,)
    kc.n_kernels = len(subs)
    for k, K in enumerate(subs):
        upper = hasattr(K, "max_valid_size")
        kc.upper[k] = 1 if upper else 0
        kc.threshold[k] = float(K.max_valid_size if upper else K.min_valid_size)
        kc.rescale[k] = float(K._rescale)
        kc.size_in_fwhm[k] = float(K.size_in_fwhm)
    return kc


def setup_on_gpu(engine: InsertionEngine, source, datacube, sph_kernel, spectral_model,
                 prune: int = N.MG_PRUNE_ALL):
    """``Martini.__init__``'s set-up on the GPU in FP64 (mg_setup): sky
    coordinates, pixel coordinates, smoothing lengths, kernel choice, ranges,
    amplitudes, thermal widths and pruning, from the source's rotated
    particle arrays.  Returns (DeviceParticles of the kept particles, kernel
    table, spectral model code, constant sigma)."""
    dev = engine.device

    def put(a, dt):
        return torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).to(dev)

    n = int(source.npart)
    xyz, vxyz = put(source.xyz_g, np.float64), put(source.vxyz_g, np.float64)
    hsm = put(source.hsm_g, np.float64)
    mhi = put(source.mHI_g, np.float64)
    model = spectral_model.native_model
    thermal = getattr(spectral_model, "sigma_mode", None) == "thermal"
    T = put(np.broadcast_to(source.T_g, (n,)), np.float64) if thermal else None
    sigma_const = 0.0
    if model == N.MG_SPECTRUM_GAUSSIAN and not thermal:
        sigma_const = float(spectral_model.sigma_mode)
    src = N.Source()
    src.n = n
    src.xyz, src.vxyz, src.hsm, src.mHI = (_ptr(t) for t in (xyz, vxyz, hsm, mhi))
    src.T = _ptr(T)
    src.ra, src.dec = float(source.ra), float(source.dec)
    src.distance, src.vpeculiar, src.h = (float(source.distance), float(source.vpeculiar),
                                          float(source.h))
    gr = N.Grid()
    for k in range(3):
        gr.crpix[k], gr.cdelt[k], gr.crval[k] = (float(datacube.crpix[k]),
                                                 float(datacube.cdelt[k]),
                                                 float(datacube.crval[k]))
    gr.freq_mode = 1 if datacube._freq_channel_mode else 0
    gr.nx, gr.ny = (int(v) for v in datacube._array.shape[:2])
    gr.nc = int(datacube.n_channels)
    gr.px_size_arcsec = float(datacube.px_size)
    gr.max_channel_width = float(np.max(np.abs(np.diff(datacube.velocity_channel_edges))))
    kc = kernel_choice(sph_kernel)
    out_t = dict(x=torch.empty(n, dtype=torch.float64, device=dev),
                 y=torch.empty(n, dtype=torch.float64, device=dev),
                 sm_range=torch.empty(n, dtype=torch.float64, device=dev),
                 h_eff=torch.empty(n, dtype=torch.float32, device=dev),
                 kernel_index=torch.empty(n, dtype=torch.int8, device=dev) if kc.adaptive
                 else None,
                 v=torch.empty(n, dtype=torch.float64, device=dev),
                 sigma=torch.empty(n, dtype=torch.float32, device=dev) if thermal else None,
                 amp=torch.empty(n, dtype=torch.float64, device=dev))
    n_kept = torch.zeros(1, dtype=torch.int64, device=dev)
    out = N.Particles()
    for k, t in out_t.items():
        setattr(out, k, _ptr(t))
    out.n_kept = _ptr(n_kept)
    ws = torch.empty(int(engine.lib.mg_setup_workspace_size(n)), dtype=torch.uint8, device=dev)
    s = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    N.check(engine.lib.mg_setup(C.byref(src), C.byref(gr), C.byref(kc), int(model),
                                float(sigma_const), int(prune), C.byref(out),
                                C.c_void_p(ws.data_ptr()), ws.numel(), s))
    m = int(n_kept.item())
    cut = {k: (None if t is None else t[:m]) for k, t in out_t.items()}
    parts = DeviceParticles(cut["x"], cut["y"], cut["sm_range"], cut["h_eff"],
                            cut["kernel_index"], v=cut["v"], sigma=cut["sigma"], amp=cut["amp"])
    return parts, sph_kernel._device_kernels(), model, sigma_const


def global_profile(engine: InsertionEngine, parts: DeviceParticles, spectral_model: int,
                   sigma_const: float, nc: int, edges: torch.Tensor) -> torch.Tensor:
    """Spatially integrated spectrum (Jy, FP64 on the device) of the
    particles' lines: mg_global_profile (martini/martini.py:1551-1596)."""
    dev = engine.device
    out = torch.empty(nc, dtype=torch.float64, device=dev)
    dummy = torch.empty(1, dtype=torch.float32, device=dev)
    prob = engine.problem(parts, [(N.MG_KERNEL_DIRAC, 0.0)], spectral_model, sigma_const, 1, 1,
                          nc, 0, 0, edges, dummy, None, N.MG_FORM_FP32)
    ws = torch.empty(int(engine.lib.mg_global_profile_workspace_size(parts.n, nc)),
                     dtype=torch.uint8, device=dev)
    s = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    N.check(engine.lib.mg_global_profile(C.byref(prob), C.c_void_p(out.data_ptr()),
                                         C.c_void_p(ws.data_ptr()), ws.numel(), s))
    N.check(engine.lib.mg_check(C.c_void_p(ws.data_ptr()), s))
    return out


def convolve_beam(engine: InsertionEngine, cube: torch.Tensor, padx: int, pady: int,
                  kernel: np.ndarray, scale: float) -> torch.Tensor:
    """Beam convolution of a padded device cube (mg_convolve_beam); returns the
    unpadded float32 cube times ``scale``."""
    dev = engine.device
    nx, ny, nc = (int(v) for v in cube.shape)
    k = torch.from_numpy(np.ascontiguousarray(kernel, dtype=np.float32)).to(dev)
    out = torch.empty((nx - 2 * padx, ny - 2 * pady, nc), dtype=torch.float32, device=dev)
    s = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    N.check(engine.lib.mg_convolve_beam(C.c_void_p(cube.data_ptr()), nx, ny, nc, int(padx),
                                        int(pady), C.c_void_p(k.data_ptr()), int(k.shape[0]),
                                        int(k.shape[1]), float(scale),
                                        C.c_void_p(out.data_ptr()), s))
    return out
