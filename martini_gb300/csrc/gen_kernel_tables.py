"""Generate ``mg_kernel_tables.h``: piecewise polynomials for the pixel
integrals of the radial SPH kernels.

The closed forms of the reference (martini/sph_kernels.py:400-441 WendlandC2,
:544-685 WendlandC6, :791-858 cubic spline, :1486-1564 quartic spline) are
sums of large logarithmic and polynomial terms that cancel: evaluated
directly in FP32 they lose up to 2e-6 (C2), 3e-6 (cubic), 6e-6 (quartic) and
7e-4 (C6) of the peak value.  Here each profile f(s), s = R^2 (R = distance /
rescaled smoothing length; offsets doubled for the cubic spline, as the
reference does), is evaluated in FP64 from the reference formula and fitted
by Chebyshev interpolation with cubic polynomials on uniform cells: in s for
the Wendland and quartic kernels, in R (and, just inside the cubic spline's
inner shell, in A = sqrt(1 - R^2), where f has a (1 - R)^1.5 term) for the
cubic spline, whose cells are aligned with its shell radius.  The FP32
device evaluation is emulated here and its error against the FP64 formula is
written into the header.  The device computes the cell index directly (no
search), loads the cell's four coefficients as one float4 and runs a
three-FMA Horner sweep.  The pieces reach the FP32 floor (~1e-7 of f(0)); the
Wendland C6 closed form itself carries rounded constants, and its table
stays within that formula's own ~7e-7.

Run:  python martini_gb300/csrc/gen_kernel_tables.py   (writes the header
next to this file; the header is committed).
"""

from __future__ import annotations

import math
import os

import numpy as np

DEG = 3  # polynomial degree per cell (4 coefficients = one float4 load)

# ---- FP64 profiles (value of the pixel integral times h^2 / norm) -----------

def f_wendland_c2(s):
    s = np.asarray(s, dtype=np.float64)
    out = np.zeros_like(s)
    out[s == 0] = 2.0 / 3.0
    m = (s > 0) & (s < 1)
    r = s[m]
    A = np.sqrt(1 - r)
    out[m] = 5 * r * r * (0.5 * r + 3) * np.log((1 + A) / np.sqrt(r)) + A * (
        -13.5 * r * r - 14.0 / 3.0 * r + 2.0 / 3.0)
    return out


def _c6_indef(R, z):
    q = np.sqrt(R**2 + z**2)
    L = np.log(q + z)
    return (-231 * R**10 * z - 385 * R**8 * z**3 - 1155 * R**8 * z - 462 * R**6 * z**5
            - 1540 * R**6 * z**3 - 462 * R**6 * z - 330 * R**4 * z**7 - 1386 * R**4 * z**5
            - 462 * R**4 * z**3 + 66 * R**4 * z - (128 + 1 / 3) * R**2 * z**9
            - 660 * R**2 * z**7 - 277.2 * R**2 * z**5 + 44 * R**2 * z**3
            + 8 / 3 * z**11 * q + (16 + 4 / 15) * R**2 * z**9 * q + 70.4 * z**9 * q
            + 360.8 * R**2 * z**7 * q + 132 * z**7 * q + 550 * R**2 * z**5 * q - 11 * R**2 * z
            + 7.21875 * R**12 * L + 24.7813 * R**10 * z * q + 173.25 * R**10 * L
            + 530.75 * R**8 * z * q + 288.75 * R**8 * L + 47.4792 * R**8 * z**3 * q
            + 767.25 * R**6 * z * q + 58.0167 * R**6 * z**5 * q + 819.5 * R**6 * z**3 * q
            + 41.7 * R**4 * z**7 * q + 752.4 * R**4 * z**5 * q + 896.5 * R**4 * z**3 * q
            - 21 * z**11 - (128 + 1 / 3) * z**9 - 66 * z**7 + 13.2 * z**5 - 11 / 3 * z**3 + z)


def f_wendland_c6(s):
    s = np.asarray(s, dtype=np.float64)
    out = np.zeros_like(s)
    out[s == 0] = 2 * 4 / 15
    m = (s > 0) & (s < 1)
    R = np.sqrt(s[m])
    out[m] = 2 * (_c6_indef(R, np.sqrt(1 - R**2)) - _c6_indef(R, 0.0))
    return out


def f_cubic_spline(s):
    s = np.asarray(s, dtype=np.float64)
    out = np.zeros_like(s)
    out[s == 0] = 11.0 / 16.0 + 0.25 * 0.25
    c1 = (s > 0) & (s <= 1)
    c2 = (s > 1) & (s <= 4)
    r1, r2 = s[c1], s[c2]
    A1, B1, B2 = np.sqrt(1 - r1), np.sqrt(4 - r1), np.sqrt(4 - r2)
    I1 = (A1 - 0.5 * A1**3 - 1.5 * r1 * A1 + 3.0 / 32.0 * A1 * (3 * r1 + 2)
          + 9.0 / 32.0 * r1 * r1 * (np.log(1 + A1) - np.log(np.sqrt(r1))))
    I2 = (-B2 * (3 * r2 + 56) / 4.0 - 3.0 / 8.0 * r2 * (r2 + 16) * np.log((2 + B2) / np.sqrt(r2))
          + 2 * (3 * r2 + 4) * B2 + 2 * B2**3)
    I3 = (-B1 * (3 * r1 + 56) / 4.0 + A1 * (4 * r1 + 50) / 8.0
          - 3.0 / 8.0 * r1 * (r1 + 16) * np.log((2 + B1) / (1 + A1))
          + 2 * (3 * r1 + 4) * (B1 - A1) + 2 * (B1**3 - A1**3))
    out[c1] = I1 + 0.25 * I3
    out[c2] = 0.25 * I2
    return out


def _quartic_IA(R, z, A):
    q = np.sqrt(z**2 + R**2)
    R2 = R**2
    return (A**4 * z - 2 * A**3 * z * q + 2 * A**2 * z * (3 * R2 + z**2)
            - A * R2 * (4 * A**2 + 3 * R2) * np.arcsinh(z / R) / 2
            - A * z * q * (5 * R2 + 2 * z**2) / 2 + R2 * R2 * z + 2 * R2 * z**3 / 3 + z**5 / 5)


def f_quartic_spline(s):
    s = np.asarray(s, dtype=np.float64)
    out = np.zeros_like(s)
    R = np.sqrt(s)
    m1 = (R > 0) & (R < 0.2)
    out[m1] += 10 * _quartic_IA(R[m1], np.sqrt(0.04 - R[m1] ** 2), 0.2)
    m2 = (R > 0) & (R < 0.6)
    out[m2] -= 5 * _quartic_IA(R[m2], np.sqrt(0.36 - R[m2] ** 2), 0.6)
    m3 = (R > 0) & (R < 1.0)
    out[m3] += _quartic_IA(R[m3], np.sqrt(1 - R[m3] ** 2), 1.0)
    out[R == 0] = 384 / 3125
    return out


# Regions of each profile, each a uniform grid of cells in one variable:
#   ("S", 0, s_max, ncell) v = s = R^2, followed by one all-zero cell: the
#                          device clamps the cell coordinate u = s * ncell /
#                          s_max to ncell, so every s >= s_max lands on the
#                          zero cell and needs no support test
#   ("R", lo, hi, ncell)   v = R
#   ("A", lo, hi, ncell)   v = sqrt(1 - R^2), used just inside a shell at R = 1
# The Wendland and quartic profiles are smooth enough in s (the s^2 log s
# term of WendlandC2 at s = 0 sets its cell count), so the device needs no
# square root.  The cubic spline keeps cells in R aligned with its shell at
# R = 1 (doubled offsets), with the half-integer power of the inner shell,
# (1 - R)^1.5, resolved by the A grid.
KERNELS = [
    # name, code, profile, support s_max = R_max^2, device scale, regions
    ("WENDLAND_C2", 0, f_wendland_c2, 1.0, "21.0 / (2.0 * 3.14159265358979323846)",
     [("S", 0.0, 1.0, 1024)]),
    ("WENDLAND_C6", 1, f_wendland_c6, 1.0, "1365.0 / (64.0 * 3.14159265358979323846)",
     [("S", 0.0, 1.0, 1024)]),
    ("CUBIC_SPLINE", 2, f_cubic_spline, 4.0, "4.0 / 1.59689476201133",
     [("R", 0.0, 0.75, 192), ("A", 0.0, float(np.sqrt(1 - 0.75**2)), 128), ("R", 1.0, 2.0, 256)]),
    ("QUARTIC_SPLINE", 3, f_quartic_spline, 1.0, "2.0 * 15625.0 / (512.0 * 3.14159265358979323846)",
     [("S", 0.0, 1.0, 512)]),
]


def region_fn(f, var):
    if var == "S":
        return f
    if var == "R":
        return lambda v: f(v**2)
    return lambda v: f(1 - v**2)


def fit_cells(fv, lo, hi, ncell):
    """Monomial coefficients in t in [0, 1) per cell (Chebyshev interpolant)."""
    out = []
    k = np.arange(DEG + 1)
    x = np.cos(np.pi * (k + 0.5) / (DEG + 1))
    for c in range(ncell):
        a = lo + (hi - lo) * c / ncell
        b = lo + (hi - lo) * (c + 1) / ncell
        v = 0.5 * (a + b) + 0.5 * (b - a) * x
        ch = np.polynomial.chebyshev.chebfit(x, fv(v), DEG)
        P = np.polynomial.Polynomial(np.polynomial.chebyshev.cheb2poly(ch))
        out.append(P(np.polynomial.Polynomial([-1.0, 2.0])).coef.astype(np.float32))
    return np.array(out, dtype=np.float32)


def region_cells(regions):
    """Table entries (float4 cells) of each region: S regions carry one zero
    cell after their ncell fitted ones."""
    return [n + (1 if var == "S" else 0) for var, lo, hi, n in regions]


def device_eval(regions, coefs, smax, s):
    """FP32 emulation of kt_eval in mg_internal.cuh."""
    s32 = s.astype(np.float32)
    if regions[0][0] == "S":
        var, lo, hi, ncell = regions[0]
        u = np.minimum(s32 * np.float32(ncell / (hi - lo)), np.float32(ncell)).astype(np.float32)
        c = np.floor(u).astype(np.int64)
        t = (u - c.astype(np.float32)).astype(np.float32)
        cf = coefs[c]
        acc = cf[:, -1].copy()
        for k in range(DEG - 1, -1, -1):
            acc = (acc * t + cf[:, k]).astype(np.float32)
        return acc.astype(np.float64)
    R = np.sqrt(s32)
    out = np.zeros(s.shape)
    reg_idx = np.zeros(s.shape, dtype=int)
    if len(regions) == 3:
        reg_idx[R >= np.float32(regions[0][2])] = 1
        reg_idx[s32 > np.float32(1.0)] = 2
    first = np.cumsum([0] + region_cells(regions))
    for ri, (var, lo, hi, ncell) in enumerate(regions):
        m = (reg_idx == ri) & (s32 < np.float32(smax))
        if var == "R":
            v = R[m]
        else:
            v = np.sqrt(np.maximum(np.float32(1.0) - s32[m], np.float32(0))).astype(np.float32)
        u = (v - np.float32(lo)) * np.float32(ncell / (hi - lo))
        c = np.clip(u.astype(np.int32), 0, ncell - 1)
        t = (u - c.astype(np.float32)).astype(np.float32)
        cf = coefs[first[ri] + c]
        acc = cf[:, -1].copy()
        for k in range(DEG - 1, -1, -1):
            acc = acc * t + cf[:, k]
        out[m] = acc
    return out


# Truncation factor of the Gaussian kernel's pixel integral (sph_kernels.py
# :1024-1031): erf(zmax / sqrt 2), zmax = sqrt(truncate^2 - q^2) in units of
# sigma, on GT_NCELL cells over [0, GT_VMAX) and one cell holding 1 past it
# (erf(8 / sqrt 2) is 1 in FP32).
GT_VMAX = 8.0
GT_NCELL = 256


def f_trunc(v):
    return np.array([math.erf(x / math.sqrt(2.0)) for x in np.atleast_1d(v)])


def gauss_trunc_table():
    co = np.vstack([fit_cells(f_trunc, 0.0, GT_VMAX, GT_NCELL),
                    np.array([[1.0, 0.0, 0.0, 0.0]])]).astype(np.float32)
    v = np.concatenate((np.linspace(0, 10, 200001), np.random.default_rng(1).uniform(0, 9, 100000)))
    v32 = v.astype(np.float32)
    u = np.minimum(v32 * np.float32(GT_NCELL / GT_VMAX), np.float32(GT_NCELL)).astype(np.float32)
    c = np.floor(u).astype(np.int64)
    t = (u - c.astype(np.float32)).astype(np.float32)
    cf = co[c]
    acc = cf[:, 3].copy()
    for k in (2, 1, 0):
        acc = (acc * t + cf[:, k]).astype(np.float32)
    err = np.abs(acc - f_trunc(v32.astype(np.float64))).max()
    return co, err


def c_float(v):
    """A float literal of C: nine significant digits and a point or exponent."""
    t = f"{float(v):.9g}"
    if "." not in t and "e" not in t:
        t += ".0"
    return t + "f"


def render(verbose: bool = False):
    """The header text and the emulated FP32 error of each table (relative
    to f(0) for the kernel profiles, absolute for the truncation factor)."""
    errors = {}
    rng = np.random.default_rng(0)
    hdr = [
        "// Generated by gen_kernel_tables.py -- do not edit.",
        "// Degree-%d polynomials on uniform cells of the radial kernels' pixel" % DEG,
        "// integrals f(s), s = R^2, fitted in FP64 to the reference closed forms",
        "// (martini/sph_kernels.py:400-441, :544-685, :791-858, :1486-1564).",
    ]
    body = []
    infos = []
    all_coefs = []
    ncoef_cells = 0
    for name, code, f, smax, scale, regions in KERNELS:
        f0 = float(f(np.array([0.0]))[0])
        parts = []
        for var, lo, hi, n in regions:
            parts.append(fit_cells(region_fn(f, var), lo, hi, n))
            if var == "S":
                parts.append(np.zeros((1, DEG + 1), dtype=np.float32))
        coefs = np.concatenate(parts)
        s = np.concatenate((rng.uniform(0, smax, 400000), smax * 10 ** rng.uniform(-12, 0, 100000),
                            np.clip(1 + rng.uniform(-1e-3, 1e-3, 50000), 0, smax),
                            rng.uniform(smax, 4 * smax, 20000)))
        err = np.abs(device_eval(regions, coefs, smax, s)
                     - f(np.minimum(s.astype(np.float32).astype(np.float64), 2 * smax))).max() / f0
        hdr.append(f"//   {name}: {len(coefs)} cells, FP32 device-form max error {err:.2e} of f(0)")
        errors[name] = err
        if verbose:
            print(name, len(coefs), f"{err:.2e}")
        regs = []
        first = ncoef_cells
        for (var, lo, hi, n), cells in zip(regions, region_cells(regions)):
            regs.append(({"R": 0, "A": 1, "S": 2}[var], lo, n / (hi - lo), n, first))
            first += cells
        while len(regs) < 3:
            regs.append((0, 0.0, 0.0, 1, first - 1))
        split_r = regions[0][2] if len(regions) == 3 else 1e30
        infos.append((smax, scale, len(regions), split_r, len(coefs), regs))
        all_coefs.append(coefs)
        ncoef_cells += len(coefs)
    body += [
        "#pragma once",
        "",
        "namespace mg {",
        "",
        f"constexpr int KT_DEG = {DEG};",
        "",
        "struct KRegion {",
        "  int var;         // 0: v = R, 1: v = sqrt(1 - R^2), 2: v = s (zero cell after the last)",
        "  float lo;        // cell grid origin in v",
        "  float cells_per_unit;",
        "  int ncell;",
        "  int first;       // first cell in kt_coef",
        "};",
        "",
        "struct KTableInfo {",
        "  float smax;      // support: f(s) = 0 for s >= smax",
        "  float scale;     // norm multiplying f / h^2",
        "  int nreg;        // 1, or 3 for the cubic spline (R < split_r, s <= 1, s > 1)",
        "  float split_r;",
        "  int ncoef;       // float4 cells of the table, zero cells included",
        "  KRegion reg[3];",
        "};",
        "",
        "__device__ __constant__ KTableInfo kt_info[4] = {",
    ]
    for smax, scale, nreg, split_r, ncoef, regs in infos:
        rs = ", ".join(f"{{{v}, {lo!r}f, {cpu!r}f, {n}, {fi}}}" for v, lo, cpu, n, fi in regs)
        body.append(f"    {{{smax!r}f, (float)({scale}), {nreg}, {split_r!r}f, {ncoef}, {{{rs}}}}},")
    body.append("};")
    body.append("")
    flat = np.concatenate(all_coefs).ravel()
    body.append(f"// {ncoef_cells} cells x {DEG + 1} coefficients (t^0 .. t^{DEG}), t in [0, 1)")
    body.append(f"__device__ __align__(16) const float kt_coef[{len(flat)}] = {{")
    for i in range(0, len(flat), DEG + 1):
        body.append("    " + ", ".join(c_float(v) for v in flat[i:i + DEG + 1]) + ",")
    body.append("};")
    body.append("")
    gt, gt_err = gauss_trunc_table()
    errors["GAUSS_TRUNC"] = gt_err
    if verbose:
        print("GAUSS_TRUNC", len(gt), f"{gt_err:.2e}")
    hdr.append(f"//   Gaussian truncation factor erf(zmax / sqrt 2): {len(gt)} cells, "
               f"FP32 max error {gt_err:.2e}")
    body.append(f"constexpr int GT_NCELL = {GT_NCELL};  // cells of gt_coef before the cell of 1")
    body.append(f"constexpr float GT_CELLS_PER_UNIT = {GT_NCELL / GT_VMAX!r}f;  // per unit zmax")
    body.append(f"__device__ __align__(16) const float gt_coef[{gt.size}] = {{")
    for row in gt:
        body.append("    " + ", ".join(c_float(v) for v in row) + ",")
    body.append("};")
    body.append("")
    body.append("}  // namespace mg")
    body.append("")
    return "\n".join(hdr + body), errors


HEADER = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mg_kernel_tables.h")


def main():
    text, _ = render(verbose=True)
    with open(HEADER, "w") as fh:
        fh.write(text)


if __name__ == "__main__":
    main()
