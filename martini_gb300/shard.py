"""Sharding the insertion over GPUs with no exchange step.

Cube pixels are independent outputs of the insertion (each pixel's
spectrum is a sum over the particles whose footprint box contains it,
martini/martini.py:243-283), and the cubes of a batch are independent of
each other.  Two ways to spread the work over ranks, one GPU per rank:

* one large cube: contiguous bands of pixel rows (axis 0), in whole tiles
  of 8 rows, balanced by the estimated pair cost.  Each rank inserts the
  particles whose footprint box reaches its band (a halo by duplication),
  with coordinates shifted into the band, into its own sub-cube.  No
  reduction is needed: the bands are disjoint and every voxel has exactly
  one owner.
* a batch of cubes: whole cubes per rank, largest first to the least
  loaded rank (LPT).

The only communication is the assembly of the final cube (a gather to the
writing rank), which is output, not part of the insertion.

Shifting a coordinate by an integer band origin (x - i0) is exact in
FP64 whenever |x - i0| <= |x|, true for every particle at or right of the
origin; for particles left of it, whose boxes only reach in, the shift can
round in the last bit of x, far below the insertion's tolerance.
"""

from __future__ import annotations

import numpy as np

TILE_I = 8  # pixel rows (axis 0) per tile of the CUDA library


def footprint_rows(x, r, nx):
    """Clipped box rows [lo, hi] per particle (|i - x| <= r, martini.py:262-271);
    hi < lo when the box misses the cube."""
    x = np.asarray(x, dtype=np.float64)
    r = np.asarray(r, dtype=np.float64)
    lo = np.maximum(np.ceil(x - r), 0)
    hi = np.minimum(np.floor(x + r), nx - 1)
    bad = ~np.isfinite(x)
    lo = np.where(bad, 1, lo).astype(np.int64)
    hi = np.where(bad, 0, hi).astype(np.int64)
    return lo, hi


def row_costs(x, y, r, nx, ny):
    """Estimated work per tile row band: for each particle, its clipped box
    columns times one, added to every tile row its box touches (a pair count
    proxy weighted by footprint width)."""
    ilo, ihi = footprint_rows(x, r, nx)
    jlo, jhi = footprint_rows(y, r, ny)
    ok = (ilo <= ihi) & (jlo <= jhi)
    ntr = (nx + TILE_I - 1) // TILE_I
    w = (jhi - jlo + 1)[ok].astype(np.float64)
    a, b = ilo[ok] // TILE_I, ihi[ok] // TILE_I
    diff = np.zeros(ntr + 1)
    np.add.at(diff, a, w)
    np.add.at(diff, b + 1, -w)
    return np.cumsum(diff[:-1])


def partition_rows(costs, world):
    """Contiguous tile-row bands [(i0, i1)) in pixels, one per rank, whose
    cumulative cost is split as evenly as the tile rows allow; every band is
    non-empty when there are at least `world` tile rows."""
    costs = np.asarray(costs, dtype=np.float64)
    ntr = costs.size
    if world < 1:
        raise ValueError("world must be >= 1")
    cum = np.concatenate([[0.0], np.cumsum(costs)])
    total = cum[-1]
    cuts = [0]
    for k in range(1, world):
        target = total * k / world
        c = int(np.searchsorted(cum, target, side="left"))
        c = min(max(c, cuts[-1] + 1), ntr - (world - k))
        cuts.append(max(c, cuts[-1]))
    cuts.append(ntr)
    return [(cuts[k] * TILE_I, cuts[k + 1] * TILE_I) for k in range(world)]


def band_particles(x, r, nx, i0, i1):
    """Indices of the particles whose clipped box reaches rows [i0, i1)."""
    lo, hi = footprint_rows(x, r, nx)
    return np.flatnonzero((lo <= hi) & (hi >= i0) & (lo < i1))


def shard(x, y, r, nx, ny, rank, world):
    """(i0, i1, particle indices, shifted x) of this rank's band."""
    bands = partition_rows(row_costs(x, y, r, nx, ny), world)
    i0, i1 = bands[rank]
    i1 = min(i1, nx)
    idx = band_particles(x, r, nx, i0, i1)
    return i0, i1, idx, np.asarray(x, dtype=np.float64)[idx] - i0


def assign_galaxies(costs, world):
    """Whole cubes per rank: longest-processing-time-first (largest cost to
    the least loaded rank, ties to the lower rank).  Deterministic."""
    costs = np.asarray(costs, dtype=np.float64)
    order = np.argsort(-costs, kind="stable")
    load = np.zeros(world)
    out = [[] for _ in range(world)]
    for g in order:
        k = int(np.argmin(load))
        out[k].append(int(g))
        load[k] += costs[g]
    return [sorted(v) for v in out]


def insert_band(engine, parts_host, kernels, spectral_model, sigma_const, nx, ny, nc, edges,
                rank, world, form=0):
    """Insert this rank's band of the cube on the rank's GPU.

    ``parts_host`` holds host arrays x, y, sm_range, h_eff, kernel_index, v,
    sigma, amp of all particles.  Returns (i0, i1, device sub-cube of shape
    (i1 - i0, ny, nc), device flux of the band)."""
    import torch

    from .engine import DeviceParticles
    x = parts_host["x"]
    i0, i1, idx, xs = shard(x, parts_host["y"], parts_host["sm_range"], nx, ny, rank, world)
    if i1 <= i0:
        return i0, i1, None, None

    def sub(k):
        v = parts_host.get(k)
        return None if v is None else np.asarray(v)[idx]

    parts = DeviceParticles.from_host(engine.device, xs, sub("y"), sub("sm_range"), sub("h_eff"),
                                      sub("kernel_index"), v=sub("v"), sigma=sub("sigma"),
                                      amp=sub("amp"))
    e = edges if isinstance(edges, torch.Tensor) else torch.from_numpy(
        np.ascontiguousarray(edges, dtype=np.float64)).to(engine.device)
    cube, flux = engine.insert(parts, kernels, spectral_model, sigma_const, i1 - i0, ny, nc, e,
                               form=form)
    return i0, i1, cube, flux
