"""Benchmark of the GPU source insertion (one JSON line on stdout).

A step is one complete ``insert_source_in_cube`` equivalent on the GPU for
the 1M-particle WendlandC2 disc on a 512 x 512 x 256 cube (thermal Gaussian
lines): footprint binning, spectra, kernel weights, contraction, cube write
and FP64 flux sums, from particle arrays resident in HBM.  The metric is
cubes/s (higher is better); the line also carries particle-channel
updates/s, the roofline of the dominant kernel (the contraction), the CPU
baseline (the reference algorithm's per-pixel loop, restated in numpy and
run on the host cores on a bounded pixel sample) and an end-to-end number
through the C ABI with host buffers.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--form fp32|bf16x3]
    python bench.py --impl reference ...   # the CPU reference arm

Under torchrun (N > 1) every rank inserts its own cube (independent
replicas, weak scaling); rank 0 prints the line.
"""

from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "disc1m_512"
METRIC = "cubes/s & particle-channel updates/s: FP32 vs BF16-split TC, <=1e-5 err vs FP64"
L2_BYTES = 129 * 1024 * 1024
# DRAM bytes (read + write) of one launch of the contraction kernel, from
# ncu (dram__bytes_read.sum + dram__bytes_write.sum) on the full workload;
# profiles/k_contract_tc_disc1m_512_f16x3.md gives the command and figures
TRAFFIC_BYTES = {("disc1m_512", "f16x3"): 2_895_373_312}


def launches_per_step(form: str, gaussian: bool, nx: int, ny: int, nc: int, ngal: int = 1,
                      ntiles: int | None = None) -> int:
    """Kernels one mg_insert(_batched) launches: cube table (one per 16
    cubes), tile init, edges, prep, pair scan (3), difference-array prefix,
    tile scan (3), plan, emit, radix passes x (histogram, scan (3), scatter),
    segments, item and partial scans (2 x 3), partial check, [spectrum store:
    row lengths, scan (3), rows], [cube clear for batches], contraction,
    split-K reduction, flux (3)."""
    if ntiles is None:
        ntiles = ((nx + 7) // 8) * ((ny + 15) // 16)  # 8 x 16-pixel tiles
    bits = max(ntiles - 1, 0).bit_length() + max(nc - 1, 0).bit_length()
    passes = (bits + 7) // 8
    n = (ngal + 15) // 16 + 1 + 1 + 1 + 3 + 1 + 3 + 1 + 1 + 5 * passes + 1 + 6 + 1
    if form != "fp32" and gaussian:
        n += 1 + 3 + 1
    if ngal > 1:
        n += 1
    return n + 1 + 1 + 3


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--form", default="f16x3", choices=["fp32", "bf16x3", "f16x3"])
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--n", type=int, default=None, help="override particle count")
    ap.add_argument("--cpu-sample-s", type=float, default=15.0,
                    help="seconds of host work for the CPU baseline sample (the reference "
                         "arm takes at most 4x this a step)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--n-gal", type=int, default=200,
                    help="galaxies of the disc population (workload disc_population)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---------------------------------------------------------------------------
# CPU baseline: the reference's per-pixel algorithm (oracle port), bounded
# ---------------------------------------------------------------------------


def cpu_baseline(w, budget_s, threads=None):
    """Time the reference algorithm on the host cores on a sample and scale.

    Spectra: ``init_spectra`` over a random particle subset (scaled by N /
    subset).  Insertion: ``_evaluate_pixel_spectrum`` over random pixels of
    the cube with a thread pool (scaled by N_pix / sample).  Returns
    (cubes/s, threads, sample description).
    """
    from oracle import martini_oracle as orc
    threads = threads or os.cpu_count() or 1
    rng = np.random.default_rng(0)
    n = w["n"]
    kernels = ([orc.kernel_constants(orc.KT_WENDLAND_C2), orc.kernel_constants(orc.KT_DIRAC),
                orc.kernel_constants(orc.KT_GAUSSIAN, 6.0)]
               if w["kernel_name"] == "WendlandC2Kernel" else orc.adaptive_tuple(w["kernel_name"]))
    sig = (w["sigma"].astype(np.float64) if w["sigma"] is not None
           else np.full(n, w["sigma_const"]))
    model = "dirac" if w["spectral_kind"] == "dirac" else "gaussian"
    # spectra on a subset
    sub = min(n, 50_000)
    idx = rng.choice(n, sub, replace=False)
    t0 = time.perf_counter()
    orc.init_spectra(model, w["mHI"][idx], w["dist"][idx], w["v"][idx], w["edges"], sig[idx])
    t_spec = (time.perf_counter() - t0) * n / sub
    spectra = orc.init_spectra(model, w["mHI"], w["dist"], w["v"], w["edges"], sig)
    kidx = (w["kernel_index"].astype(np.int64) if w["kernel_index"] is not None
            else np.zeros(n, np.int64))
    npix = w["nx"] * w["ny"]
    args = (w["x"], w["y"], w["sm_range"], kernels, kidx, w["h_eff"].astype(np.float64), spectra)
    # grow the pixel sample until the budget is used
    done = 0
    t_pix = 0.0
    batch = 64
    while t_pix < budget_s and done < npix:
        pix = [(int(i), int(j)) for i, j in zip(rng.integers(0, w["nx"], batch),
                                                rng.integers(0, w["ny"], batch))]
        t0 = time.perf_counter()
        orc.insert_perpixel(w["nx"], w["ny"], *args, ncpu=threads, pixels=pix)
        t_pix += time.perf_counter() - t0
        done += batch
        batch = min(batch * 2, 4096)
    t_cube = t_spec + t_pix * npix / done
    desc = (f"reference per-pixel loop (numpy restatement) on {done} random pixels of "
            f"{npix} and spectra of {sub} of {n} particles, scaled to one cube; "
            f"{threads} threads")
    return 1.0 / t_cube, threads, desc


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        # raw samples (the line carries their summary); MG_CLOCKS_DIR keeps them
        self.path = os.path.join(os.environ.get("MG_CLOCKS_DIR", tempfile.gettempdir()),
                                 f"martini_gb300_clocks_{index}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        for line in open(self.path):
            p = [s.strip() for s in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for name, val in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                                  "sw_power_cap"), p[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def main():
    a = parse()
    rank, world, local = dist_env()
    if a.impl == "reference":
        return reference_arm(a, rank, world)

    import torch
    import torch.distributed as dist
    from martini_gb300 import _native as N
    from martini_gb300 import workloads
    from martini_gb300.engine import DeviceParticles, InsertionEngine

    if world > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)
    if a.workload == "disc_population":
        run_population(a, rank, world, local, dev)
        if world > 1:
            dist.destroy_process_group()
        return
    w = workloads.build(a.workload, n=a.n)
    form = {"fp32": N.MG_FORM_FP32, "bf16x3": N.MG_FORM_BF16X3, "f16x3": N.MG_FORM_F16X3}[a.form]
    edges = torch.from_numpy(np.ascontiguousarray(w["edges"])).to(dev)
    nx, ny, nc = w["nx"], w["ny"], w["nc"]
    cube = torch.empty((nx, ny, nc), dtype=torch.float32, device=dev)
    flux = torch.empty(nc + 1, dtype=torch.float64, device=dev)
    # one insertion per spectral group; later groups add to the cube
    groups = w["groups"] or [dict(sel=None, spectral_model=w["spectral_model"])]
    ins = []
    for gi, grp in enumerate(groups):
        s = slice(None) if grp["sel"] is None else grp["sel"]
        kidx = w["kernel_index"][s] if w["kernel_index"] is not None else None
        sig = w["sigma"][s] if w["sigma"] is not None else None
        eng = InsertionEngine(dev)
        parts = DeviceParticles.from_host(dev, w["x"][s], w["y"][s], w["sm_range"][s],
                                          w["h_eff"][s], kidx, v=w["v"][s], sigma=sig,
                                          amp=w["amp"][s])
        prob = eng.problem(parts, w["kernels"], grp["spectral_model"], w["sigma_const"], nx, ny,
                           nc, 0, 0, edges, cube, flux, form, accumulate=gi > 0)
        info = eng.plan(prob)
        ins.append(dict(eng=eng, parts=parts, prob=prob, info=info, s=s))
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)

    # one CUDA graph for the whole step (every group's insertion): the 45-odd
    # launches of an insertion replay as one
    for g in ins:
        g["eng"].run(g["prob"])
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        for g in ins:
            g["eng"].run(g["prob"])

    def step():
        graph.replay()

    # the clock sampler starts before the warm-up: nvidia-smi's start-up
    # stalls the GPU for a moment and must not fall into the timed region
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(1.5)
    for _ in range(a.warmup):
        flush.zero_()
        step()
    torch.cuda.synchronize()
    for g in ins:
        g["eng"].check()

    # --- timed region: K full insertions, L2 flushed between steps ----------
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(a.steps)]
    for k in range(a.steps):
        flush.zero_()
        ev[k][0].record(stream)
        step()
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    t_steps = sum(s.elapsed_time(e) for s, e in ev) / 1e3  # s
    for g in ins:
        g["eng"].check()

    # --- dominant kernel: the contraction stage alone ------------------------
    for g in ins:
        g["eng"].run_stages(g["prob"], N.MG_STAGE_BIN | N.MG_STAGE_SPEC)
    cev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(3)]
    for s0, e0 in cev:
        flush.zero_()
        s0.record(stream)
        for g in ins:
            g["eng"].run_stages(g["prob"], N.MG_STAGE_CONTRACT)
        e0.record(stream)
    torch.cuda.synchronize()
    t_contract = float(np.mean([s0.elapsed_time(e0) for s0, e0 in cev])) / 1e3

    # --- end to end through the C ABI with host buffers -------------------------
    for g in ins:
        s = g["s"]
        host = {k: torch.from_numpy(np.ascontiguousarray(w[k][s], dtype=dt)).pin_memory()
                for k, dt in (("x", np.float64), ("y", np.float64), ("sm_range", np.float64),
                              ("h_eff", np.float32), ("v", np.float64), ("amp", np.float64))}
        if w["kernel_index"] is not None:
            host["kernel_index"] = torch.from_numpy(
                w["kernel_index"][s].astype(np.int8)).pin_memory()
        if w["sigma"] is not None:
            host["sigma"] = torch.from_numpy(w["sigma"][s].astype(np.float32)).pin_memory()
        g["host"] = host
        g["dev"] = {k: getattr(g["parts"], k) for k in host}
    # two buffer sets (device particles, cube, flux; pinned host results) so
    # that the copies of one step overlap the insertion of the next: inputs
    # go up and results come back on a copy stream, insertions run in order
    # on the compute stream (one workspace per engine)
    import dataclasses
    sets = [dict(cube=cube, flux=flux, probs=[g["prob"] for g in ins],
                 dev=[g["dev"] for g in ins])]
    cube1, flux1 = torch.empty_like(cube), torch.empty_like(flux)
    probs1, dev1 = [], []
    for gi, g in enumerate(ins):
        p1 = dataclasses.replace(g["parts"], **{k: torch.empty_like(getattr(g["parts"], k))
                                               for k in g["host"]})
        probs1.append(g["eng"].problem(p1, w["kernels"], g["prob"].spectral_model,
                                       w["sigma_const"], nx, ny, nc, 0, 0, edges, cube1, flux1,
                                       form, accumulate=gi > 0))
        dev1.append({k: getattr(p1, k) for k in g["host"]})
        g["parts1"] = p1
    sets.append(dict(cube=cube1, flux=flux1, probs=probs1, dev=dev1))
    for st in sets:
        st["host_cube"] = torch.empty((nx, ny, nc), dtype=torch.float32).pin_memory()
        st["host_flux"] = torch.empty(nc + 1, dtype=torch.float64).pin_memory()
    h2d = sum(t.numel() * t.element_size() for g in ins for t in g["host"].values())
    d2h = sets[0]["host_cube"].numel() * 4 + sets[0]["host_flux"].numel() * 8
    up, down = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    comp_ev, down_ev = {}, {}

    def e2e_step(k):
        st = sets[k % 2]
        # inputs of step k: after the insertion that last read this set
        if k - 2 in comp_ev:
            up.wait_event(comp_ev[k - 2])
        with torch.cuda.stream(up):
            for gi, g in enumerate(ins):
                for key, t in g["host"].items():
                    st["dev"][gi][key].copy_(t, non_blocking=True)
        stream.wait_event(up.record_event())
        # the insertion overwrites this set's cube: after its read-back
        if k - 2 in down_ev:
            stream.wait_event(down_ev[k - 2])
        for gi, g in enumerate(ins):
            g["eng"].run(st["probs"][gi], stream=stream)
        comp_ev[k] = stream.record_event()
        down.wait_event(comp_ev[k])
        with torch.cuda.stream(down):
            st["host_cube"].copy_(st["cube"], non_blocking=True)
            st["host_flux"].copy_(st["flux"], non_blocking=True)
        down_ev[k] = down.record_event()

    e2e_step(0)
    e2e_step(1)
    torch.cuda.synchronize()
    comp_ev.clear()
    down_ev.clear()
    ke = max(2, min(a.steps, 6))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    up.wait_event(e0)
    down.wait_event(e0)
    for k in range(ke):
        e2e_step(k)
    stream.wait_event(down_ev[ke - 1])
    stream.wait_event(down_ev[ke - 2])
    e1.record(stream)
    torch.cuda.synchronize()
    t_e2e = e0.elapsed_time(e1) / 1e3 / ke

    # --- aggregate over ranks ---------------------------------------------------
    if world > 1:
        tt = torch.tensor([t_steps, t_e2e], dtype=torch.float64, device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_steps, t_e2e = float(tt[0]), float(tt[1])
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return

    # algorithmic work: box-footprint pixels x channels (the reference's
    # per-pixel mask selects exactly these pairs)
    F = workloads.footprint_pixels(w["x"], w["y"], w["sm_range"], nx, ny)
    updates = float(F.sum()) * nc
    flops = 2.0 * updates
    cubes_per_s = world * a.steps / t_steps
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak_tf = peaks.get("bf16_tflops", 1900.0)
    achieved_tf = flops / t_contract / 1e12
    # measured on the full workload only: no figure for a reduced particle count
    traffic = TRAFFIC_BYTES.get((a.workload, a.form)) if a.n is None else None
    line = {
        "metric": METRIC,
        "value": cubes_per_s,
        "unit": "cubes/s",
        "n_gpus": world,
        "steps": a.steps,
        "warmup": a.warmup,
        "ms_per_step": t_steps / a.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": a.form,
        "data": "synthetic (seeded exponential disc, no dataset)",
        "config": {"workload": a.workload, "particles": w["n"], "particles_generated":
                   w["n_input"], "cube": [nx, ny, nc], "kernel": w["kernel_name"],
                   "spectrum": w["spectral_kind"], "form": a.form,
                   "l2": "flushed between steps (256 MiB write)", "parallelism":
                   f"replicas{world}", "pairs": int(sum(g["info"].n_pairs for g in ins)),
                   "groups": len(ins)},
        "particle_channel_updates_per_s": world * updates * a.steps / t_steps,
        "roofline": {"bound": "tensor", "achieved": achieved_tf, "peak": peak_tf,
                     "unit": "TFLOP/s", "frac": achieved_tf / peak_tf, "traffic": traffic,
                     "kernel": ("k_contract_tc" if a.form != "fp32" else "k_contract_fp32")
                     + " (stage timed: cube clear, contraction, split-K reduction)",
                     "contract_ms": t_contract * 1e3,
                     "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)" if peaks
                     else "fallback 1.9 PFLOP/s"},
        "e2e": {"value": world / t_e2e, "unit": "cubes/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": a.steps * sum(launches_per_step(
            a.form, g["prob"].spectral_model == N.MG_SPECTRUM_GAUSSIAN, nx, ny, nc) for g in ins),
        "step_ms": [round(s.elapsed_time(e), 3) for s, e in ev],
        "clocks": clk,
    }
    if not a.no_cpu_baseline:
        v, cores, desc = cpu_baseline(w, a.cpu_sample_s)
        line["cpu_baseline"] = {"value": v, "unit": "cubes/s", "cores": cores, "kind": "port",
                                "sample": desc}
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_population(a, rank, world, local, dev):
    """The disc population as one batch (mg_insert_batched) against the same
    cubes inserted one call at a time (the looped plain form)."""
    import torch
    import torch.distributed as dist
    from martini_gb300 import _native as N
    from martini_gb300 import workloads
    from martini_gb300.engine import BatchInsertion, DeviceParticles, InsertionEngine

    form = {"fp32": N.MG_FORM_FP32, "bf16x3": N.MG_FORM_BF16X3, "f16x3": N.MG_FORM_F16X3}[a.form]
    gals = workloads.build_population(a.n_gal, workers=0)
    eng = InsertionEngine(dev)
    items, probs = [], []
    for w in gals:
        parts = DeviceParticles.from_host(dev, w["x"], w["y"], w["sm_range"], w["h_eff"],
                                          w["kernel_index"], v=w["v"], sigma=w["sigma"],
                                          amp=w["amp"])
        edges = torch.from_numpy(np.ascontiguousarray(w["edges"])).to(dev)
        cube = torch.empty((w["nx"], w["ny"], w["nc"]), dtype=torch.float32, device=dev)
        flux = torch.empty(w["nc"] + 1, dtype=torch.float64, device=dev)
        prob = eng.problem(parts, w["kernels"], w["spectral_model"], w["sigma_const"], w["nx"],
                           w["ny"], w["nc"], 0, 0, edges, cube, flux, form)
        items.append(dict(parts=parts, edges=edges, cube=cube, flux=flux, w=w))
        probs.append(prob)
    batch = BatchInsertion(eng, probs, keep=items)
    info = batch.plan()
    # looped plain form: one mg_insert per cube on one shared workspace
    loop_eng = InsertionEngine(dev)
    caps = []
    for prob in probs:
        loop_eng.plan(prob)
        caps.append(loop_eng._caps)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)

    def looped():
        ws = loop_eng._ws
        for prob, cp in zip(probs, caps):
            N.check(loop_eng.lib.mg_insert(C.byref(prob), C.c_void_p(ws.data_ptr()), ws.numel(),
                                           cp[0], cp[1], C.c_void_p(stream.cuda_stream)))

    def timed(fn, k):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(k)]
        for s0, e0 in ev:
            flush.zero_()
            s0.record(stream)
            fn()
            e0.record(stream)
        torch.cuda.synchronize()
        return [s0.elapsed_time(e0) / 1e3 for s0, e0 in ev]

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(1.5)
    for _ in range(a.warmup):
        flush.zero_()
        batch.run()
        looped()
    torch.cuda.synchronize()
    batch.check()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    t_batch = timed(batch.run, a.steps)
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    batch.check()
    t_loop = timed(looped, a.steps)
    batch.run_stages(N.MG_STAGE_BIN | N.MG_STAGE_SPEC)
    t_contract = float(np.mean(timed(lambda: batch.run_stages(N.MG_STAGE_CONTRACT), 3)))
    # end to end: particles from pinned host memory, every cube back.  Two
    # buffer sets (device particles and cubes, each with its batched problem;
    # pinned host cubes) so that the copies of one batch overlap the
    # insertion of the other: uploads and read-backs run on their own
    # streams, insertions in order on the compute stream
    import dataclasses
    host = []
    for it in items:
        w = it["w"]
        hp = {k: torch.from_numpy(np.ascontiguousarray(w[k], dtype=dt)).pin_memory()
              for k, dt in (("x", np.float64), ("y", np.float64), ("sm_range", np.float64),
                            ("h_eff", np.float32), ("v", np.float64), ("amp", np.float64))}
        if w["kernel_index"] is not None:
            hp["kernel_index"] = torch.from_numpy(w["kernel_index"].astype(np.int8)).pin_memory()
        if w["sigma"] is not None:
            hp["sigma"] = torch.from_numpy(w["sigma"].astype(np.float32)).pin_memory()
        host.append(hp)
    h2d = sum(t.numel() * t.element_size() for hp in host for t in hp.values())
    d2h = sum(it["cube"].numel() * 4 for it in items)
    sets = [dict(batch=batch, dev=[{k: getattr(it["parts"], k) for k in hp}
                                   for it, hp in zip(items, host)],
                 cubes=[it["cube"] for it in items])]
    items1, probs1 = [], []
    for it, hp in zip(items, host):
        w = it["w"]
        # the second set starts as a copy of the first (the plan sizes its
        # workspace from the particles it bins)
        p1 = dataclasses.replace(it["parts"], **{k: getattr(it["parts"], k).clone()
                                                for k in hp})
        cube1, flux1 = torch.empty_like(it["cube"]), torch.empty_like(it["flux"])
        probs1.append(eng.problem(p1, w["kernels"], w["spectral_model"], w["sigma_const"],
                                  w["nx"], w["ny"], w["nc"], 0, 0, it["edges"], cube1, flux1,
                                  form))
        items1.append(dict(parts=p1, cube=cube1, flux=flux1))
    batch1 = BatchInsertion(eng, probs1, keep=items1)
    batch1.plan()
    sets.append(dict(batch=batch1, dev=[{k: getattr(it1["parts"], k) for k in hp}
                                        for it1, hp in zip(items1, host)],
                     cubes=[it1["cube"] for it1 in items1]))
    for st in sets:
        st["host_cubes"] = [torch.empty(tuple(c.shape), dtype=torch.float32).pin_memory()
                            for c in st["cubes"]]
    up, down = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    comp_ev, down_ev = {}, {}

    def e2e_step(k):
        st = sets[k % 2]
        # inputs of batch k: after the insertion that last read this set
        if k - 2 in comp_ev:
            up.wait_event(comp_ev[k - 2])
        with torch.cuda.stream(up):
            for hp, dp in zip(host, st["dev"]):
                for key, t in hp.items():
                    dp[key].copy_(t, non_blocking=True)
        stream.wait_event(up.record_event())
        # the insertion overwrites this set's cubes: after their read-back
        if k - 2 in down_ev:
            stream.wait_event(down_ev[k - 2])
        st["batch"].run(stream=stream)
        comp_ev[k] = stream.record_event()
        down.wait_event(comp_ev[k])
        with torch.cuda.stream(down):
            for hc, c in zip(st["host_cubes"], st["cubes"]):
                hc.copy_(c, non_blocking=True)
        down_ev[k] = down.record_event()

    e2e_step(0)
    e2e_step(1)
    torch.cuda.synchronize()
    comp_ev.clear()
    down_ev.clear()
    ke = max(2, min(a.steps, 4))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    up.wait_event(e0)
    down.wait_event(e0)
    for k in range(ke):
        e2e_step(k)
    stream.wait_event(down_ev[ke - 1])
    stream.wait_event(down_ev[ke - 2])
    e1.record(stream)
    torch.cuda.synchronize()
    t_e2e = e0.elapsed_time(e1) / 1e3 / ke
    batch1.check()
    tb, tl = float(np.sum(t_batch)), float(np.sum(t_loop))
    if world > 1:
        tt = torch.tensor([tb, tl, t_e2e], dtype=torch.float64, device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        tb, tl, t_e2e = (float(v) for v in tt)
    if rank != 0:
        return
    ng = len(gals)
    updates = float(sum(workloads.footprint_pixels(w["x"], w["y"], w["sm_range"], w["nx"],
                                                   w["ny"]).sum() * w["nc"] for w in gals))
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak_tf = peaks.get("bf16_tflops", 1900.0)
    achieved = 2.0 * updates / t_contract / 1e12
    ntiles = sum(((w["nx"] + 7) // 8) * ((w["ny"] + 15) // 16) for w in gals)
    line = {
        "metric": METRIC, "value": world * ng * a.steps / tb, "unit": "cubes/s", "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": tb / a.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": a.form,
        "data": "synthetic (seeded disc population, no dataset)",
        "config": {"workload": "disc_population", "galaxies": ng,
                   "particles": int(sum(w["n"] for w in gals)),
                   "cubes": "32^2x64 | 64^2x128 | 128^2x128 | 256^2x256 at 4 km/s",
                   "kernel": "WendlandC2Kernel", "spectrum": "thermal", "form": a.form,
                   "l2": "flushed between steps (256 MiB write)",
                   "parallelism": f"replicas{world}", "pairs": int(info.n_pairs),
                   "form_batched": True},
        "looped": {"value": world * ng * a.steps / tl, "unit": "cubes/s",
                   "ms_per_step": tl / a.steps * 1e3,
                   "note": "same cubes, one mg_insert per cube"},
        "particle_channel_updates_per_s": world * updates * a.steps / tb,
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak_tf,
                     "unit": "TFLOP/s", "frac": achieved / peak_tf, "traffic": None,
                     "kernel": "k_contract_tc (stage timed: cube clear, contraction, split-K "
                               "reduction, all cubes)", "contract_ms": t_contract * 1e3,
                     "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)" if peaks
                     else "fallback 1.9 PFLOP/s"},
        "e2e": {"value": world * ng / t_e2e, "unit": "cubes/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": a.steps * launches_per_step(a.form, True, 0, 0,
                                                    max(w["nc"] for w in gals), ng, ntiles),
        "step_ms": [round(t * 1e3, 3) for t in t_batch],
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def reference_arm(a, rank, world):
    """The reference algorithm (per-pixel numpy restatement) on the host cores."""
    if rank != 0:
        return
    from martini_gb300 import workloads
    # about a minute of host work in all (at most 4 x --cpu-sample-s a step)
    budget = min(max(2.0, 60.0 / max(1, a.steps + a.warmup)), 4.0 * a.cpu_sample_s)
    if a.workload == "disc_population":
        # a seeded sample of the population's galaxies; cubes/s from the mean
        # time per cube over the sample
        gals = workloads.build_population(a.n_gal)
        pick = np.random.default_rng(1).choice(len(gals), min(4, len(gals)), replace=False)
        sample = [gals[k] for k in pick]
        w = dict(n=int(sum(g["n"] for g in gals)), nx="32-256", ny="32-256", nc="64-256",
                 kernel_name="WendlandC2Kernel", spectral_kind="thermal")

        def one(b):
            tsum = 0.0
            for g in sample:
                v, cores, _ = cpu_baseline(g, b / len(sample))
                tsum += 1.0 / v
            return len(sample) / tsum, cores, (f"reference per-pixel loop (numpy restatement) on "
                                               f"{len(sample)} sampled galaxies of {len(gals)}, "
                                               f"each on a pixel sample, scaled to whole cubes")
    else:
        w = workloads.build(a.workload, n=a.n)

        def one(b):
            return cpu_baseline(w, b)
    for _ in range(a.warmup):
        one(budget / 4)
    vals = []
    t0 = time.perf_counter()
    for _ in range(a.steps):
        v, cores, desc = one(budget)
        vals.append(v)
    wall = time.perf_counter() - t0
    value = float(np.mean(vals))
    line = {
        "impl": "reference",
        "metric": METRIC, "value": value, "unit": "cubes/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": 1e3 / value, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded exponential disc, no dataset)",
        "config": {"workload": a.workload, "particles": w["n"], "cube": [w["nx"], w["ny"], w["nc"]],
                   "kernel": w["kernel_name"], "spectrum": w["spectral_kind"]},
        "cpu_baseline": {"value": value, "unit": "cubes/s", "cores": cores, "kind": "port",
                         "sample": desc},
        "e2e": {"value": value, "unit": "cubes/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "wall_s": wall,
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
