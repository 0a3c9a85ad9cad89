"""Sharding the insertion over ranks (martini_gb300.shard): host logic on
CPU, the band decomposition checked end to end with gloo ranks (each rank
inserts its band with the oracle; rank 0 assembles and compares with the
full cube), and on one GPU by inserting every band in turn."""

import os
import socket
import tempfile

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from martini_gb300 import shard
from oracle import martini_oracle as orc


def _case(n=1500, nx=72, ny=40, nc=16, seed=3):
    rng = np.random.default_rng(seed)
    kernels = orc.adaptive_tuple("WendlandC2Kernel")
    h = 10 ** rng.uniform(-0.5, 0.9, n)
    kidx, size, resc = orc.select_kernels(kernels, h)
    x = np.concatenate([rng.normal(30, 10, n - 20), rng.uniform(-15, nx + 15, 20)])
    y = rng.normal(20, 8, n)
    v = rng.normal(100, 20, n)
    sig = rng.uniform(3, 8, n)
    mhi = 10 ** rng.uniform(4, 5, n)
    edges = orc.vrad_channel_edges(nc, 4.0, 100.0)
    spectra = orc.init_spectra("gaussian", mhi, np.full(n, 3.0), v, edges, sig)
    return dict(x=x, y=y, r=orc.sm_ranges(h, size), h_eff=h * resc, kidx=kidx, kernels=kernels,
                spectra=spectra, nx=nx, ny=ny, nc=nc, v=v, sig=sig, amp=mhi / 9.0 / orc.MHI_TO_JY,
                edges=edges)


def test_partition_rows_covers_in_order_and_balances():
    rng = np.random.default_rng(0)
    costs = rng.exponential(1.0, 40)
    for world in (1, 2, 3, 5, 8):
        bands = shard.partition_rows(costs, world)
        assert len(bands) == world
        assert bands[0][0] == 0 and bands[-1][1] == 40 * shard.TILE_I
        for (a0, a1), (b0, _) in zip(bands, bands[1:]):
            assert a1 == b0 and a0 < a1
        per = [costs[a // shard.TILE_I:b // shard.TILE_I].sum() for a, b in bands]
        # a greedy cut misses the ideal share by at most one tile row
        assert max(per) - costs.sum() / world <= costs.max() + 1e-9


def test_band_particles_are_exactly_the_boxes_reaching_the_band():
    c = _case()
    i0, i1 = 24, 48
    idx = shard.band_particles(c["x"], c["r"], c["nx"], i0, i1)
    keep = np.zeros(c["x"].size, bool)
    for p in range(c["x"].size):
        lo, hi = orc.footprint_bounds(c["x"][p], c["r"][p], c["nx"])
        keep[p] = lo <= hi and hi >= i0 and lo < i1
    np.testing.assert_array_equal(idx, np.flatnonzero(keep))


def test_assign_galaxies_lpt():
    out = shard.assign_galaxies([5, 1, 4, 2, 3, 3], 2)
    loads = [sum([5, 1, 4, 2, 3, 3][g] for g in part) for part in out]
    assert sorted(g for part in out for g in part) == list(range(6))
    assert abs(loads[0] - loads[1]) <= 1


def _rank_main(rank, world, port, path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        c = _case()
        i0, i1, idx, xs = shard.shard(c["x"], c["y"], c["r"], c["nx"], c["ny"], rank, world)
        band = orc.insert_scatter(i1 - i0, c["ny"], xs, c["y"][idx], c["r"][idx], c["kernels"],
                                  c["kidx"][idx], c["h_eff"][idx], c["spectra"][idx])
        parts = [None] * world if rank == 0 else None
        dist.gather_object((i0, i1, band), parts, dst=0)
        if rank == 0:
            full = np.zeros((c["nx"], c["ny"], c["nc"]))
            for a, b, sub in parts:
                full[a:b] = sub
            ref = orc.insert_scatter(c["nx"], c["ny"], c["x"], c["y"], c["r"], c["kernels"],
                                     c["kidx"], c["h_eff"], c["spectra"])
            err = np.abs(full - ref).max() / np.abs(ref).max()
            np.save(path, np.array([err, len(parts)]))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_band_shards_assemble_to_the_full_cube_gloo(world):
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "err.npy")
        mp.start_processes(_rank_main, args=(world, port, path), nprocs=world, join=True,
                           start_method="spawn")
        err, nparts = np.load(path)
    assert nparts == world
    assert err <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("world", [2, 3])
def test_band_shards_on_one_gpu(world):
    """Every band inserted in turn through the CUDA library, assembled: the
    same cube as one full insertion."""
    from martini_gb300 import _native as N
    from martini_gb300.engine import DeviceParticles, InsertionEngine
    c = _case(n=4000, nx=96, ny=48, nc=24)
    eng = InsertionEngine("cuda:0")
    table = [(N.MG_KERNEL_WENDLAND_C2, 0.0), (N.MG_KERNEL_DIRAC, 0.0), (N.MG_KERNEL_GAUSSIAN, 6.0)]
    host = dict(x=c["x"], y=c["y"], sm_range=c["r"], h_eff=c["h_eff"], kernel_index=c["kidx"],
                v=c["v"], sigma=c["sig"], amp=c["amp"])
    full = np.zeros((c["nx"], c["ny"], c["nc"]), np.float32)
    tot = 0.0
    for rank in range(world):
        i0, i1, cube, flux = shard.insert_band(eng, host, table, N.MG_SPECTRUM_GAUSSIAN, 0.0,
                                               c["nx"], c["ny"], c["nc"], c["edges"], rank, world)
        if cube is not None:
            full[i0:i1] = cube.cpu().numpy()
            tot += float(flux[0].item())
    parts = DeviceParticles.from_host(eng.device, c["x"], c["y"], c["r"], c["h_eff"], c["kidx"],
                                      v=c["v"], sigma=c["sig"], amp=c["amp"])
    ref, rflux = eng.insert(parts, table, N.MG_SPECTRUM_GAUSSIAN, 0.0, c["nx"], c["ny"], c["nc"],
                            torch.from_numpy(c["edges"]).to(eng.device))
    ref = ref.cpu().numpy()
    assert np.abs(full - ref).max() / np.abs(ref).max() <= 1e-6
    assert abs(tot - float(rflux[0].item())) / float(rflux[0].item()) <= 1e-6
