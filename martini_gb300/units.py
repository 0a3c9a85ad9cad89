"""Unit handling without astropy.

The reference takes astropy Quantities everywhere.  astropy is optional
here: every argument may be an astropy Quantity (anything with
``to_value``), which is converted, or a plain number/array, which is taken
to be in the documented unit of that argument.
"""

from __future__ import annotations

import numpy as np

C_KMS = 299792.458           # speed of light, km/s
HI_FREQ_HZ = 1.420405751e9   # HI rest frequency (martini/datacube.py:21)
K_B = 1.380649e-23           # J/K (CODATA 2018, as astropy)
M_P = 1.67262192369e-27      # kg (CODATA 2018, as astropy)


def is_quantity(x) -> bool:
    return hasattr(x, "to_value") and hasattr(x, "unit")


def value(x, unit: str, equivalencies=None) -> np.ndarray | float:
    """``x`` in ``unit`` (an astropy unit string) as float / float64 array."""
    if x is None:
        return None
    if is_quantity(x):
        if equivalencies is not None:
            return np.asarray(x.to_value(unit, equivalencies=equivalencies), dtype=np.float64)
        return np.asarray(x.to_value(unit), dtype=np.float64)
    return np.asarray(x, dtype=np.float64)


def scalar(x, unit: str) -> float:
    return float(value(x, unit))


def physical_type(x) -> str | None:
    """'frequency', 'speed' or None for a plain number."""
    if not is_quantity(x):
        return None
    t = str(x.unit.physical_type)
    if "frequency" in t:
        return "frequency"
    if "speed" in t or "velocity" in t:
        return "speed"
    return t


def radio_velocity_kms(freq_hz):
    """Radio-convention Doppler velocity of a frequency (km/s)."""
    return C_KMS * (1.0 - np.asarray(freq_hz, dtype=np.float64) / HI_FREQ_HZ)


def radio_frequency_hz(v_kms):
    return HI_FREQ_HZ * (1.0 - np.asarray(v_kms, dtype=np.float64) / C_KMS)
