"""Minimal FITS writer for the cube and beam outputs (no astropy).

Implements the parts of the FITS standard (version 4.0) that the reference's
``write_fits`` / ``write_beam_fits`` outputs use (martini/martini.py:939-1105):
one primary HDU, a header of 80-character keyword records in 2880-byte
blocks ending with ``END``, and the data array in big-endian IEEE floats
(BITPIX -32 or -64) with the first axis (NAXIS1) varying fastest.
"""

from __future__ import annotations

import os

import numpy as np

BLOCK = 2880


def _fmt_value(v):
    if isinstance(v, bool):
        return f"{'T' if v else 'F':>20}"
    if isinstance(v, (int, np.integer)):
        return f"{int(v):>20d}"
    if isinstance(v, (float, np.floating)):
        s = repr(float(v)).upper()
        if "E" not in s and "." not in s:
            s += ".0"
        return f"{s:>20}"
    s = str(v).replace("'", "''")
    return f"'{s:<8}'"


def card(key: str, value=None, comment: str | None = None) -> str:
    """One 80-character header record (fixed format for numbers, quoted
    strings; logical T/F)."""
    key = key.upper()
    if len(key) > 8:
        raise ValueError(f"keyword too long: {key}")
    if value is None:
        rec = f"{key:<8}"
    else:
        rec = f"{key:<8}= {_fmt_value(value)}"
        if comment:
            rec += f" / {comment}"
    if len(rec) > 80:
        rec = rec[:80]
    return f"{rec:<80}"


def write_primary(filename: str, cards, data: np.ndarray, overwrite: bool = True) -> None:
    """Write one primary HDU.  ``cards`` are (key, value[, comment]) tuples
    after SIMPLE/BITPIX/NAXISn, which are written here from ``data`` (given
    in FITS axis order reversed, i.e. numpy C order with NAXIS1 last)."""
    if os.path.exists(filename) and not overwrite:
        raise OSError(f"File {filename} already exists.")
    data = np.asarray(data)
    if data.dtype == np.float32:
        bitpix, be = -32, ">f4"
    else:
        bitpix, be = -64, ">f8"
    recs = [card("SIMPLE", True), card("BITPIX", bitpix), card("NAXIS", data.ndim)]
    for k, n in enumerate(reversed(data.shape)):
        recs.append(card(f"NAXIS{k + 1}", int(n)))
    skip = {"SIMPLE", "BITPIX", "NAXIS"} | {f"NAXIS{k + 1}" for k in range(data.ndim)}
    for c in cards:
        if c[0].upper() in skip:
            continue
        recs.append(card(*c))
    recs.append(card("END"))
    head = "".join(recs)
    head += " " * ((-len(head)) % BLOCK)
    raw = np.ascontiguousarray(data, dtype=be).tobytes()
    raw += b"\0" * ((-len(raw)) % BLOCK)
    with open(filename, "wb") as f:
        f.write(head.encode("ascii"))
        f.write(raw)


def read_primary(filename: str):
    """(header dict, data) of a file written by write_primary (for tests and
    quick looks)."""
    with open(filename, "rb") as f:
        buf = f.read()
    hdr = {}
    pos = 0
    while True:
        rec = buf[pos:pos + 80].decode("ascii")
        pos += 80
        key = rec[:8].strip()
        if key == "END":
            break
        if rec[8:10] == "= ":
            val = rec[10:].split(" / ")[0].strip()
            if val.startswith("'"):
                val = val[1:].rsplit("'", 1)[0].rstrip().replace("''", "'")
            elif val in ("T", "F"):
                val = val == "T"
            else:
                try:
                    val = int(val)
                except ValueError:
                    val = float(val)
            hdr[key] = val
    pos += (-pos) % BLOCK
    shape = tuple(hdr[f"NAXIS{k}"] for k in range(hdr["NAXIS"], 0, -1))
    dt = ">f4" if hdr["BITPIX"] == -32 else ">f8"
    n = int(np.prod(shape))
    data = np.frombuffer(buf, dtype=dt, count=n, offset=pos).reshape(shape)
    return hdr, data
