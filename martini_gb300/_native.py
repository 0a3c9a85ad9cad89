"""ctypes binding of the in-tree CUDA library ``libmartini_gb300.so``.

The library is the product: there is no CPU fallback.  Loading fails loudly
if the library has not been built (``python -m martini_gb300.build`` or
``__graft_entry__.build()``) or no CUDA device is present.
"""

from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmartini_gb300.so")

MG_OK = 0
MG_ERR_INVALID_ARGUMENT = -1
MG_ERR_CUDA = -2
MG_ERR_WORKSPACE = -3
MG_ERR_NOT_MONOTONIC = -4
MG_ERR_UNSUPPORTED = -5
MG_ERR_TIMEOUT = -6

MG_KERNEL_WENDLAND_C2 = 0
MG_KERNEL_WENDLAND_C6 = 1
MG_KERNEL_CUBIC_SPLINE = 2
MG_KERNEL_QUARTIC_SPLINE = 3
MG_KERNEL_GAUSSIAN = 4
MG_KERNEL_DIRAC = 5

MG_SPECTRUM_GAUSSIAN = 0
MG_SPECTRUM_DIRAC = 1
MG_SPECTRUM_TABLE = 2

MG_FORM_FP32 = 0
MG_FORM_BF16X3 = 1
MG_FORM_F16X3 = 2
MG_FORM_BF16X6 = 3

MG_MAX_KERNELS = 4

# every symbol include/martini_gb300.h declares
EXPORTS = ("mg_version", "mg_last_error", "mg_workspace_size", "mg_plan", "mg_insert",
           "mg_insert_stages", "mg_check", "mg_spectra", "mg_flux", "mg_insert_noalloc",
           "mg_workspace_size_batched", "mg_plan_batched", "mg_insert_batched",
           "mg_insert_stages_batched", "mg_setup_workspace_size", "mg_setup",
           "mg_global_profile_workspace_size", "mg_global_profile", "mg_convolve_beam",
           "mg_tuning_default", "mg_tuning_candidates", "mg_tune", "mg_tune_batched",
           "mg_tuning_lookup", "mg_tuning_store", "mg_tuning_reset")

MG_NOALLOC_SCRATCH_BYTES = 128 << 20

MG_STAGE_BIN = 1
MG_STAGE_CONTRACT = 2
MG_STAGE_FLUX = 4
MG_STAGE_SPEC = 8
MG_STAGE_ALL = 15


class KernelSpec(C.Structure):
    _fields_ = [("type", C.c_int32), ("truncate", C.c_float)]


class Problem(C.Structure):
    _fields_ = [
        ("n", C.c_int64),
        ("x", C.c_void_p), ("y", C.c_void_p), ("sm_range", C.c_void_p), ("h_eff", C.c_void_p),
        ("kernel_index", C.c_void_p),
        ("n_kernels", C.c_int32),
        ("kernels", KernelSpec * MG_MAX_KERNELS),
        ("spectral_model", C.c_int32),
        ("v", C.c_void_p), ("sigma", C.c_void_p), ("sigma_const", C.c_float),
        ("amp", C.c_void_p), ("spectra", C.c_void_p),
        ("nx", C.c_int32), ("ny", C.c_int32), ("nc", C.c_int32),
        ("padx", C.c_int32), ("pady", C.c_int32),
        ("edges", C.c_void_p), ("cube", C.c_void_p), ("flux", C.c_void_p),
        ("form", C.c_int32),
        ("accumulate", C.c_int32),
    ]


class Source(C.Structure):
    _fields_ = [("n", C.c_int64), ("xyz", C.c_void_p), ("vxyz", C.c_void_p), ("hsm", C.c_void_p),
                ("mHI", C.c_void_p), ("T", C.c_void_p), ("ra", C.c_double), ("dec", C.c_double),
                ("distance", C.c_double), ("vpeculiar", C.c_double), ("h", C.c_double)]


class Grid(C.Structure):
    _fields_ = [("crpix", C.c_double * 3), ("cdelt", C.c_double * 3), ("crval", C.c_double * 3),
                ("freq_mode", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32),
                ("nc", C.c_int32), ("px_size_arcsec", C.c_double),
                ("max_channel_width", C.c_double)]


class KernelChoice(C.Structure):
    _fields_ = [("n_kernels", C.c_int32), ("adaptive", C.c_int32), ("upper", C.c_int32 * 4),
                ("threshold", C.c_double * 4), ("rescale", C.c_double * 4),
                ("size_in_fwhm", C.c_double * 4)]


class Particles(C.Structure):
    _fields_ = [("x", C.c_void_p), ("y", C.c_void_p), ("sm_range", C.c_void_p),
                ("h_eff", C.c_void_p), ("kernel_index", C.c_void_p), ("v", C.c_void_p),
                ("sigma", C.c_void_p), ("amp", C.c_void_p), ("n_kept", C.c_void_p)]


MG_PRUNE_SPATIAL = 1
MG_PRUNE_SPECTRAL = 2
MG_PRUNE_MASS = 4
MG_PRUNE_ALL = 7


class Tuning(C.Structure):
    """mg_tuning: the launch shape of an insertion (its autotuner's choice)."""
    _fields_ = [("kc", C.c_int32), ("items_per_sm", C.c_int32), ("cost_order", C.c_int32),
                ("reserved", C.c_int32)]

    def as_dict(self) -> dict:
        return {"kc": int(self.kc), "items_per_sm": int(self.items_per_sm),
                "cost_order": int(self.cost_order)}


class PlanInfo(C.Structure):
    _fields_ = [("n_pairs", C.c_int64), ("n_items", C.c_int64), ("n_partial_items", C.c_int64),
                ("n_tiles", C.c_int64), ("workspace_bytes", C.c_size_t)]


class MartiniGB300Error(RuntimeError):
    """A non-zero status from the native library."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"martini_gb300 error {code}: {msg}")
        self.code = code


_lib = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load (once) and return the native library."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(
            f"{path} is missing: build it with `python -m martini_gb300.build` "
            "(the GPU path has no CPU fallback)")
    lib = C.CDLL(path)
    P = C.POINTER
    lib.mg_version.restype = C.c_char_p
    lib.mg_last_error.restype = C.c_char_p
    lib.mg_workspace_size.argtypes = [P(Problem), C.c_int64, C.c_int64, P(C.c_size_t)]
    lib.mg_plan.argtypes = [P(Problem), C.c_void_p, C.c_size_t, C.c_void_p, P(PlanInfo)]
    lib.mg_insert.argtypes = [P(Problem), C.c_void_p, C.c_size_t, C.c_int64, C.c_int64,
                              C.c_void_p]
    lib.mg_insert_stages.argtypes = [P(Problem), C.c_void_p, C.c_size_t, C.c_int64, C.c_int64,
                                     C.c_int32, C.c_void_p]
    lib.mg_check.argtypes = [C.c_void_p, C.c_void_p]
    lib.mg_workspace_size_batched.argtypes = [P(Problem), C.c_int32, C.c_int64, C.c_int64,
                                              P(C.c_size_t)]
    lib.mg_plan_batched.argtypes = [P(Problem), C.c_int32, C.c_void_p, C.c_size_t, C.c_void_p,
                                    P(PlanInfo)]
    lib.mg_insert_batched.argtypes = [P(Problem), C.c_int32, C.c_void_p, C.c_size_t, C.c_int64,
                                      C.c_int64, C.c_void_p]
    lib.mg_insert_stages_batched.argtypes = [P(Problem), C.c_int32, C.c_void_p, C.c_size_t,
                                             C.c_int64, C.c_int64, C.c_int32, C.c_void_p]
    lib.mg_insert_noalloc.argtypes = [P(Problem), C.c_void_p]
    lib.mg_global_profile_workspace_size.argtypes = [C.c_int64, C.c_int32]
    lib.mg_global_profile_workspace_size.restype = C.c_size_t
    lib.mg_global_profile.argtypes = [P(Problem), C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]
    lib.mg_convolve_beam.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                     C.c_int32, C.c_void_p, C.c_int32, C.c_int32, C.c_float,
                                     C.c_void_p, C.c_void_p]
    lib.mg_setup_workspace_size.argtypes = [C.c_int64]
    lib.mg_setup_workspace_size.restype = C.c_size_t
    lib.mg_setup.argtypes = [P(Source), P(Grid), P(KernelChoice), C.c_int32, C.c_float, C.c_int32,
                             P(Particles), C.c_void_p, C.c_size_t, C.c_void_p]
    lib.mg_spectra.argtypes = [P(Problem), C.c_void_p, C.c_void_p]
    lib.mg_flux.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                            C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]
    lib.mg_tuning_default.argtypes = [P(Tuning)]
    lib.mg_tuning_default.restype = None
    lib.mg_tuning_candidates.argtypes = [C.c_int32, P(Tuning), C.c_int32]
    lib.mg_tune.argtypes = [P(Problem), C.c_void_p, C.c_size_t, C.c_int64, C.c_int64, C.c_int32,
                            C.c_void_p, P(Tuning), P(C.c_float)]
    lib.mg_tune_batched.argtypes = [P(Problem), C.c_int32, C.c_void_p, C.c_size_t, C.c_int64,
                                    C.c_int64, C.c_int32, C.c_void_p, P(Tuning), P(C.c_float)]
    lib.mg_tuning_lookup.argtypes = [P(Problem), C.c_int32, C.c_int64, P(Tuning)]
    lib.mg_tuning_store.argtypes = [P(Problem), C.c_int32, C.c_int64, P(Tuning)]
    lib.mg_tuning_reset.argtypes = []
    lib.mg_tuning_reset.restype = None
    for f in ("mg_workspace_size", "mg_plan", "mg_insert", "mg_insert_stages", "mg_check",
              "mg_spectra", "mg_flux", "mg_insert_noalloc", "mg_workspace_size_batched",
              "mg_plan_batched", "mg_insert_batched", "mg_insert_stages_batched", "mg_setup",
              "mg_global_profile", "mg_convolve_beam", "mg_tuning_candidates", "mg_tune",
              "mg_tune_batched", "mg_tuning_lookup", "mg_tuning_store"):
        getattr(lib, f).restype = C.c_int
    _lib = lib
    return lib


def check(rc: int) -> None:
    """Raise MartiniGB300Error (ValueError for non-monotonic edges) on failure."""
    if rc == MG_OK:
        return
    msg = load().mg_last_error().decode(errors="replace")
    if rc == MG_ERR_NOT_MONOTONIC:
        raise ValueError(msg)
    raise MartiniGB300Error(rc, msg)


# SPH kernel classes (reference and mirror names, without the leading "_")
_KERNEL_TYPES = {"WendlandC2Kernel": MG_KERNEL_WENDLAND_C2,
                 "WendlandC6Kernel": MG_KERNEL_WENDLAND_C6,
                 "CubicSplineKernel": MG_KERNEL_CUBIC_SPLINE,
                 "QuarticSplineKernel": MG_KERNEL_QUARTIC_SPLINE,
                 "GaussianKernel": MG_KERNEL_GAUSSIAN,
                 "DiracDeltaKernel": MG_KERNEL_DIRAC}


def kernel_table(kernel) -> list[tuple[int, float]]:
    """(MG_KERNEL_*, truncate) rows for an SPH kernel object of the reference
    (martini/sph_kernels.py) or of martini_gb300.sph_kernels: the sub-kernels
    of an adaptive kernel in order (its ``kernels`` tuple, indexed by
    ``kernel_indices``), or the single kernel."""
    subs = getattr(kernel, "kernels", None) or (kernel,)
    rows = []
    for k in subs:
        name = type(k).__name__.lstrip("_")
        if name not in _KERNEL_TYPES:
            raise ValueError(f"unsupported SPH kernel {type(k).__name__}")
        t = _KERNEL_TYPES[name]
        rows.append((t, float(getattr(k, "truncate", 0.0)) if t == MG_KERNEL_GAUSSIAN else 0.0))
    if len(rows) > MG_MAX_KERNELS:
        raise ValueError(f"at most {MG_MAX_KERNELS} kernels in an adaptive tuple")
    return rows


def set_kernels(p: "Problem", rows) -> None:
    """Fill the kernel table of a Problem from kernel_table() rows."""
    p.n_kernels = len(rows)
    for k, (t, trunc) in enumerate(rows):
        p.kernels[k].type = int(t)
        p.kernels[k].truncate = float(trunc)
