"""martini_gb300: MARTINI's source insertion (``Martini.insert_source_in_cube``)
as hand-written sm_103a CUDA behind a C ABI, with the reference's Python API.

Importing the package does not need a GPU; inserting does (there is no CPU
fallback).
"""

from .datacube import DataCube
from .martini import GlobalProfile, Martini
from .sources import SPHSource
from . import sph_kernels, spectral_models

__version__ = "0.1.0"

__all__ = ["Martini", "GlobalProfile", "DataCube", "SPHSource", "sph_kernels", "spectral_models", "__version__"]
