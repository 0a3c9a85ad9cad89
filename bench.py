"""Benchmark of the GPU source insertion (one JSON line on stdout).

A step is one complete ``insert_source_in_cube`` equivalent on the GPU:
footprint binning, spectra, kernel weights, contraction, cube write and
FP64 flux sums, from particle arrays resident in HBM.  The default workload
is the precision-form configuration: the 4M-particle WendlandC2 disc on a
1024 x 1024 x 512 cube of 2 km/s channels (thermal Gaussian lines), in the
chosen tensor-core form (bf16x6, the exact three-piece BF16 split).  The
metric is cubes/s (higher is better); the line also carries:

* particle-channel updates/s and spectrum evaluations/s;
* ``fp32``: the plain FP32 CUDA-core form on the same workload;
* ``errors``: max error / cube peak at 64 sampled pixels and the relative
  error of the total flux, both against the FP64 CPU oracle;
* the roofline of the dominant kernel (the contraction);
* the CPU baseline (the reference algorithm's per-pixel loop, restated in
  numpy, on a bounded pixel sample and extrapolated: ``timed_fraction``);
* an end-to-end number through the C ABI with host buffers.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--form bf16x6|f16x3|fp32|bf16x3]
                    [--workload disc4m_1024|disc1m_512|stress16m_2048|disc_population]
    python bench.py --impl reference ...   # the CPU reference arm

Under torchrun (N > 1) the cube is split into bands of tile rows balanced by
estimated cost, one per rank with a halo of duplicated particles
(strong scaling; no collective on the data path); the disc population is
split into whole cubes per rank, largest first.  Rank 0 prints the line.
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

WORKLOAD = "disc4m_1024"
METRIC = "cubes/s & particle-channel updates/s: FP32 vs BF16-split TC, <=1e-5 err vs FP64"
L2_BYTES = 129 * 1024 * 1024
# contraction forms (the MG_FORM_* codes)
FORMS = {"fp32": 0, "bf16x3": 1, "f16x3": 2, "bf16x6": 3}
# DRAM bytes (read + write) of one launch of the contraction kernel, from
# one ncu pass (dram__bytes_read.sum + dram__bytes_write.sum) on the full
# workload, for the kernel as it stands
TRAFFIC_BYTES = {("disc4m_1024", "bf16x6"): 5_896_006_400}


def launches_per_step(form: str, gaussian: bool, nx: int, ny: int, nc: int, ngal: int = 1,
                      ntiles: int | None = None) -> int:
    """Kernels one mg_insert(_batched) launches: cube table (one per 16
    cubes), tile init, edges, prep, pair scan (3), difference-array prefix,
    tile scan (3), plan, emit, radix passes x (histogram, scan (3), scatter),
    segments, item and partial scans (2 x 3), work-queue keys and their two
    radix passes (2 x 5), partial check, [spectrum store: row lengths, scan
    (3), rows], [cube clear for batches], [tensor-core parameters],
    contraction, split-K reduction, flux (3)."""
    if ntiles is None:
        ntiles = ((nx + 7) // 8) * ((ny + 15) // 16)  # 8 x 16-pixel tiles
    bits = max(ntiles - 1, 0).bit_length() + max(nc - 1, 0).bit_length()
    passes = (bits + 7) // 8
    n = (ngal + 15) // 16 + 1 + 1 + 1 + 3 + 1 + 3 + 1 + 1 + 5 * passes + 1 + 6 + 1 + 10 + 1
    if form != "fp32" and gaussian:
        n += 1 + 3 + 1
    if form != "fp32":
        n += 1
    if ngal > 1:
        n += 1
    return n + 1 + 1 + 3


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--form", default="bf16x6", choices=sorted(FORMS))
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--n", type=int, default=None, help="override particle count")
    ap.add_argument("--cpu-sample-s", type=float, default=15.0,
                    help="seconds of host work for the CPU baseline sample (the reference "
                         "arm takes at most 4x this a step)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp32", action="store_true",
                    help="skip timing the plain FP32 form beside the chosen form")
    ap.add_argument("--no-errors", action="store_true",
                    help="skip the error fields against the FP64 oracle")
    ap.add_argument("--no-tune", action="store_true",
                    help="use the default launch shape instead of autotuning it")
    ap.add_argument("--no-e2e", action="store_true",
                    help="skip the end-to-end leg (its second buffer set): for profiling")
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
            f"{npix} and spectra of {sub} of {n} particles, extrapolated linearly to one "
            f"cube; {threads} threads")
    return 1.0 / t_cube, threads, desc, done / npix


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


def peaks_of():
    """Roofline denominators: the measured peaks when present, else the
    fallback figures (and which was used)."""
    try:
        pk = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return (float(pk.get("bf16_tflops", 1900.0)), float(pk.get("hbm_gbs", 6800.0)),
                "MEASURED_PEAKS.json (bf16_tflops burst, hbm_gbs)")
    except (OSError, ValueError):
        return 1900.0, 6800.0, "fallback (1.9 PFLOP/s bf16, 6.8 TB/s)"


def roofline(flops, nbytes, t_kernel):
    """Roofline of one launch: the bound is whichever of the tensor peak and
    the HBM peak takes longer for the algorithmic work; achieved and frac are
    in that resource's unit."""
    peak_tf, peak_gbs, src = peaks_of()
    t_tensor = flops / (peak_tf * 1e12)
    t_hbm = nbytes / (peak_gbs * 1e9)
    if t_tensor >= t_hbm:
        out = {"bound": "tensor", "achieved": flops / t_kernel / 1e12, "peak": peak_tf,
               "unit": "TFLOP/s"}
    else:
        out = {"bound": "hbm", "achieved": nbytes / t_kernel / 1e9, "peak": peak_gbs,
               "unit": "GB/s"}
    out["frac"] = out["achieved"] / out["peak"]
    out["peak_source"] = src
    out["algorithmic"] = {"flops": flops, "bytes": nbytes,
                          "tensor_ms_at_peak": t_tensor * 1e3, "hbm_ms_at_peak": t_hbm * 1e3}
    return out


def band_workload(w, rank, world):
    """This rank's band of a single-cube workload: contiguous tile rows
    balanced by estimated pair cost, the particles whose box reaches them
    (a halo by duplication) with x shifted into the band (shard.shard)."""
    from martini_gb300 import shard
    i0, i1, idx, xs = shard.shard(w["x"], w["y"], w["sm_range"], w["nx"], w["ny"], rank, world)
    sub = dict(w)
    for k in ("y", "sm_range", "h_eff", "kernel_index", "v", "sigma", "amp", "mHI", "dist"):
        if isinstance(w.get(k), np.ndarray) and w[k].shape[:1] == (w["n"],):
            sub[k] = w[k][idx]
    sub["x"] = xs
    sub["n"] = int(idx.size)
    sub["nx"] = int(i1 - i0)
    sub["band"] = (int(i0), int(i1))
    if w["groups"]:
        sub["groups"] = [dict(g, sel=np.flatnonzero(np.isin(idx, g["sel"])))
                         for g in w["groups"]]
    return sub


def build_insertions(w, form, dev, edges, cube, flux, tune=False):
    """One planned insertion per spectral group of the workload; groups after
    the first add to the cube.  With ``tune`` each insertion's launch shape is
    autotuned (mg_tune) and cached before any timed or captured run."""
    from martini_gb300.engine import DeviceParticles, InsertionEngine
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
        prob = eng.problem(parts, w["kernels"], grp["spectral_model"], w["sigma_const"], w["nx"],
                           w["ny"], w["nc"], 0, 0, edges, cube, flux, form,
                           accumulate=gi > 0)
        info = eng.plan(prob)
        shape = eng.tune(prob, reps=2) if tune else None
        ins.append(dict(eng=eng, parts=parts, prob=prob, info=info, s=s, shape=shape))
    return ins


def graph_of(ins):
    """One CUDA graph for a whole step (every group's insertion): the 45-odd
    launches of an insertion replay as one."""
    import torch
    for g in ins:
        g["eng"].run(g["prob"])
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        for g in ins:
            g["eng"].run(g["prob"])
    return graph


def timed_steps(fn, k, flush, stream):
    """K calls of fn, each after an L2 flush, timed with CUDA events on the
    launching stream (seconds per call)."""
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(k)]
    for s0, e0 in ev:
        flush.zero_()
        s0.record(stream)
        fn()
        e0.record(stream)
    torch.cuda.synchronize()
    return [s0.elapsed_time(e0) / 1e3 for s0, e0 in ev]


def errors_vs_oracle(w, cube, flux0, max_box_px=6e10):
    """Max |cube - oracle| / cube peak over 64 sampled pixels (48 with signal,
    16 uniform; the reference's per-pixel sum in the FP64 oracle) and the
    relative error of the FP64 flux against the oracle's FP64 total (per
    particle, in C; skipped when the workload's box pixels exceed
    max_box_px)."""
    from martini_gb300 import workloads
    from oracle import martini_oracle as orc
    t0 = time.perf_counter()
    rng = np.random.default_rng(3)
    lit = np.argwhere(cube.max(axis=2) > 1e-3 * cube.max())
    pick = lit[rng.choice(len(lit), size=min(48, len(lit)), replace=False)]
    uni = np.stack([rng.integers(0, cube.shape[0], 16), rng.integers(0, cube.shape[1], 16)], 1)
    pixels = [tuple(int(v) for v in p) for p in np.concatenate([pick, uni])]
    kern = orc.adaptive_tuple(w["kernel_name"])
    groups = w["groups"] or [dict(sel=None, spectral_model=w["spectral_model"])]
    ref = np.zeros((len(pixels), w["nc"]))
    total = 0.0
    box_px = float(workloads.footprint_pixels(w["x"], w["y"], w["sm_range"], w["nx"],
                                              w["ny"]).sum())
    do_flux = box_px <= max_box_px
    for grp in groups:
        s = np.arange(w["n"]) if grp["sel"] is None else grp["sel"]
        model = "dirac" if grp["spectral_model"] == FORMS_SPECTRUM_DIRAC else "gaussian"
        kidx = w["kernel_index"][s] if w["kernel_index"] is not None else None
        sig = None
        if model == "gaussian":
            sig = w["sigma"][s] if w["sigma"] is not None else w["sigma_const"]
        ref += orc.pixel_spectra(pixels, w["x"][s], w["y"][s], w["sm_range"][s], kern, kidx,
                                 w["h_eff"][s], model, w["mHI"][s], w["dist"][s], w["v"][s],
                                 w["edges"], sig)
        if do_flux:
            ss = orc.spectrum_sums(model, w["v"][s], sig, w["amp"][s], w["edges"])
            total += orc.flux_total(w["x"][s], w["y"][s], w["sm_range"][s], kern, kidx,
                                    w["h_eff"][s].astype(np.float64), ss, w["nx"], w["ny"])
    got = np.stack([cube[i, j] for i, j in pixels]).astype(np.float64)
    out = {"max_err_over_peak": float(np.abs(got - ref).max() / np.abs(cube).max()),
           "pixels_sampled": len(pixels),
           "flux_rel_err": float(abs(flux0 - total) / total) if do_flux else None,
           "oracle": "FP64 CPU oracle: per-pixel sums at the sampled pixels; total flux as "
                     "sum_p (sum_box W_p)(sum_c S_p) over every particle" +
                     ("" if do_flux else " (skipped: too many box pixels for the host)"),
           "oracle_s": round(time.perf_counter() - t0, 2)}
    return out


FORMS_SPECTRUM_DIRAC = 1  # MG_SPECTRUM_DIRAC


def main():
    a = parse()
    rank, world, local = dist_env()
    if a.impl == "reference":
        return reference_arm(a, rank, world)

    import torch
    import torch.distributed as dist
    from martini_gb300 import _native as N
    from martini_gb300 import workloads

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
    w_full = workloads.build(a.workload, n=a.n)
    # one cube per step: with N ranks each inserts its own band of it
    w = band_workload(w_full, rank, world) if world > 1 else w_full
    form = FORMS[a.form]
    edges = torch.from_numpy(np.ascontiguousarray(w["edges"])).to(dev)
    nx, ny, nc = w["nx"], w["ny"], w["nc"]
    cube = torch.empty((nx, ny, nc), dtype=torch.float32, device=dev)
    flux = torch.empty(nc + 1, dtype=torch.float64, device=dev)
    ins = build_insertions(w, form, dev, edges, cube, flux, tune=not a.no_tune)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)
    graph = graph_of(ins)

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
    t_step = timed_steps(step, a.steps, flush, stream)
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    t_steps = float(np.sum(t_step))
    for g in ins:
        g["eng"].check()
    cube_host = cube.cpu().numpy() if rank == 0 else None
    flux0 = float(flux[0].item())

    # --- dominant kernel: the contraction stage alone ------------------------
    for g in ins:
        g["eng"].run_stages(g["prob"], N.MG_STAGE_BIN | N.MG_STAGE_SPEC)
    t_contract = float(np.mean(timed_steps(
        lambda: [g["eng"].run_stages(g["prob"], N.MG_STAGE_CONTRACT) for g in ins], 3, flush,
        stream)))

    # --- the plain FP32 form on the same workload -----------------------------
    fp32 = None
    if form != FORMS["fp32"] and not a.no_fp32 and world == 1:
        cube32 = torch.empty_like(cube)
        flux32 = torch.empty_like(flux)
        ins32 = build_insertions(w, FORMS["fp32"], dev, edges, cube32, flux32,
                                 tune=not a.no_tune)
        g32 = graph_of(ins32)
        flush.zero_()
        g32.replay()
        t32 = timed_steps(g32.replay, max(3, min(a.steps, 5)), flush, stream)
        for g in ins32:
            g["eng"].check()
        fp32 = {"value": len(t32) / float(np.sum(t32)), "unit": "cubes/s",
                "ms_per_step": float(np.mean(t32)) * 1e3}
        del ins32, g32, cube32, flux32
        torch.cuda.empty_cache()

    # --- end to end through the C ABI with host buffers -------------------------
    t_e2e, h2d, d2h = (float("nan"), 0, 0) if a.no_e2e else e2e_time(a, w, ins, cube, flux,
                                                                      form, edges, dev, stream)

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
    # per-pixel mask selects exactly these pairs), of the whole cube
    F = workloads.footprint_pixels(w_full["x"], w_full["y"], w_full["sm_range"], w_full["nx"],
                                   w_full["ny"])
    updates = float(F.sum()) * w_full["nc"]
    cubes_per_s = a.steps / t_steps
    # roofline of this rank's contraction launch: its own band's work
    Fr = workloads.footprint_pixels(w["x"], w["y"], w["sm_range"], nx, ny)
    flops_r = 2.0 * float(Fr.sum()) * nc
    bytes_r = float(nx) * ny * nc * 4 + 72.0 * w["n"]
    rl = roofline(flops_r, bytes_r, t_contract)
    rl["kernel"] = (("k_contract_tc" if a.form != "fp32" else "k_contract_fp32") +
                    " (stage timed: cube clear, contraction, split-K reduction)")
    rl["contract_ms"] = t_contract * 1e3
    # measured on the full workload only: no figure for a reduced particle count
    rl["traffic"] = (TRAFFIC_BYTES.get((a.workload, a.form))
                     if a.n is None and world == 1 else None)
    err = errors_vs_oracle(w, cube_host, flux0) if not a.no_errors else None
    line = {
        "metric": METRIC,
        "value": cubes_per_s,
        "unit": "cubes/s",
        "n_gpus": world,
        "steps": a.steps,
        "warmup": a.warmup,
        "ms_per_step": t_steps / a.steps * 1e3,
        "higher_is_better": True,
        "scaling": "strong" if world > 1 else "weak",
        "vs_baseline": None,
        "dtype": a.form,
        "data": "synthetic (seeded exponential disc, no dataset)",
        "config": {"workload": a.workload, "particles": w_full["n"], "particles_generated":
                   w_full["n_input"], "cube": [w_full["nx"], w_full["ny"], w_full["nc"]],
                   "kernel": w_full["kernel_name"], "spectrum": w_full["spectral_kind"],
                   "form": a.form, "l2": "flushed between steps (256 MiB write)",
                   "parallelism": f"bands{world}" if world > 1 else "single",
                   "pairs": int(sum(g["info"].n_pairs for g in ins)), "groups": len(ins),
                   "launch_shape": [g["shape"] for g in ins] if not a.no_tune
                   else "default (not tuned)"},
        "particle_channel_updates_per_s": updates * a.steps / t_steps,
        "spectrum_evaluations_per_s": float(w_full["n"]) * w_full["nc"] * a.steps / t_steps,
        "errors": err,
        "fp32": fp32,
        "roofline": rl,
        "e2e": {"value": 1.0 / t_e2e, "unit": "cubes/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": a.steps * sum(launches_per_step(
            a.form, g["prob"].spectral_model == N.MG_SPECTRUM_GAUSSIAN, nx, ny, nc) for g in ins),
        "step_ms": [round(t * 1e3, 3) for t in t_step],
        "clocks": clk,
    }
    if world > 1:
        line["config"]["band_rows_rank0"] = w["band"]
    if not a.no_cpu_baseline:
        v, cores, desc, frac = cpu_baseline(w_full, a.cpu_sample_s)
        line["cpu_baseline"] = {"value": v, "unit": "cubes/s", "cores": cores, "kind": "port",
                                "sample": desc, "extrapolated": True, "timed_fraction": frac}
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def e2e_time(a, w, ins, cube, flux, form, edges, dev, stream):
    """Seconds per cube end to end through the C ABI: every step copies its
    particles from pinned host memory and reads the cube and flux back.  Two
    buffer sets (device particles, cube, flux; pinned host results) so that
    the copies of one step overlap the insertion of the next: inputs go up
    and results come back on copy streams, insertions run in order on the
    compute stream (one workspace per engine).  Returns (s, h2d, d2h bytes)."""
    import dataclasses
    import torch
    nx, ny, nc = w["nx"], w["ny"], w["nc"]
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
    for g in ins:
        g["eng"].check()
    return e0.elapsed_time(e1) / 1e3 / ke, h2d, d2h


def run_population(a, rank, world, local, dev):
    """The disc population as one batch (mg_insert_batched) against the same
    cubes inserted one call at a time (the looped plain form)."""
    import torch
    import torch.distributed as dist
    from martini_gb300 import _native as N
    from martini_gb300 import workloads
    from martini_gb300.engine import BatchInsertion, DeviceParticles, InsertionEngine

    form = FORMS[a.form]
    # large populations are set up in a spawn-started process pool (numpy
    # host set-up of up to 2000 galaxies; no GPU work in the workers)
    nw = min(8, os.cpu_count() or 1) if a.n_gal > 200 else 0
    gals_all = workloads.build_population(a.n_gal, workers=nw)
    gals = gals_all
    imbalance = None
    if world > 1:
        # whole cubes per rank, largest estimated cost first to the least
        # loaded rank (shard.assign_galaxies); no exchange step
        from martini_gb300 import shard
        cost = [float(workloads.footprint_pixels(g["x"], g["y"], g["sm_range"], g["nx"],
                                                 g["ny"]).sum()) * g["nc"] for g in gals_all]
        parts_of = shard.assign_galaxies(cost, world)
        loads = [sum(cost[k] for k in ks) for ks in parts_of]
        imbalance = max(loads) / (sum(loads) / world) if sum(loads) > 0 else 1.0
        gals = [gals_all[k] for k in parts_of[rank]]
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
    shape = batch.tune(reps=2) if not a.no_tune else None
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

    # the plain FP32 form looped over the same cubes
    probs32, caps32 = [], []
    loop32 = InsertionEngine(dev)
    for prob in probs:
        q = N.Problem.from_buffer_copy(prob)
        q.form = FORMS["fp32"]
        loop32.plan(q)
        probs32.append(q)
        caps32.append(loop32._caps)

    def looped_fp32():
        ws = loop32._ws
        for prob, cp in zip(probs32, caps32):
            N.check(loop32.lib.mg_insert(C.byref(prob), C.c_void_p(ws.data_ptr()), ws.numel(),
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
    looped_fp32()
    t_loop32 = timed(looped_fp32, max(1, min(a.steps, 3)))
    batch.run_stages(N.MG_STAGE_BIN | N.MG_STAGE_SPEC)
    t_contract = float(np.mean(timed(lambda: batch.run_stages(N.MG_STAGE_CONTRACT), 3)))
    def pop_e2e():
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
        return t_e2e, h2d, d2h

    # (skipped with --no-e2e: it holds a second set of particles, cubes and
    # workspace, which the full 2000-galaxy population cannot spare)
    t_e2e, h2d, d2h = (float("nan"), 0, 0) if a.no_e2e else pop_e2e()
    tb, tl = float(np.sum(t_batch)), float(np.sum(t_loop))
    if world > 1:
        tt = torch.tensor([tb, tl, t_e2e], dtype=torch.float64, device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        tb, tl, t_e2e = (float(v) for v in tt)
    if rank != 0:
        return
    ng = len(gals_all)
    updates = float(sum(workloads.footprint_pixels(w["x"], w["y"], w["sm_range"], w["nx"],
                                                   w["ny"]).sum() * w["nc"] for w in gals_all))
    updates_r = float(sum(workloads.footprint_pixels(w["x"], w["y"], w["sm_range"], w["nx"],
                                                     w["ny"]).sum() * w["nc"] for w in gals))
    bytes_r = float(sum(w["nx"] * w["ny"] * w["nc"] * 4 + 72 * w["n"] for w in gals))
    rl = roofline(2.0 * updates_r, bytes_r, t_contract)
    rl.update({"traffic": None, "contract_ms": t_contract * 1e3,
               "kernel": "k_contract_tc (stage timed: cube clear, contraction, split-K "
                         "reduction, all cubes)"})
    ntiles = sum(((w["nx"] + 7) // 8) * ((w["ny"] + 15) // 16) for w in gals)
    line = {
        "metric": METRIC, "value": ng * a.steps / tb, "unit": "cubes/s", "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": tb / a.steps * 1e3,
        "higher_is_better": True, "scaling": "strong" if world > 1 else "weak",
        "vs_baseline": None, "dtype": a.form,
        "data": "synthetic (seeded disc population, no dataset)",
        "config": {"workload": "disc_population", "galaxies": ng,
                   "particles": int(sum(w["n"] for w in gals)),
                   "cubes": "32^2x64 | 64^2x128 | 128^2x128 | 256^2x256 at 4 km/s",
                   "kernel": "WendlandC2Kernel", "spectrum": "thermal", "form": a.form,
                   "l2": "flushed between steps (256 MiB write)",
                   "parallelism": f"lpt{world}" if world > 1 else "single",
                   "pairs_rank0": int(info.n_pairs), "form_batched": True,
                   "lpt_imbalance": imbalance,
                   "launch_shape": shape if shape else "default (not tuned)"},
        "looped": {"value": ng * a.steps / tl, "unit": "cubes/s",
                   "ms_per_step": tl / a.steps * 1e3,
                   "note": f"same cubes, one mg_insert per cube, {a.form}"},
        "looped_fp32": {"value": ng * len(t_loop32) / float(np.sum(t_loop32)),
                        "unit": "cubes/s", "ms_per_step": float(np.mean(t_loop32)) * 1e3,
                        "note": "same cubes, one mg_insert per cube, plain FP32 form"},
        "particle_channel_updates_per_s": updates * a.steps / tb,
        "spectrum_evaluations_per_s": float(sum(w["n"] * w["nc"] for w in gals_all)) * a.steps
                                      / tb,
        "roofline": rl,
        "e2e": {"value": ng / t_e2e, "unit": "cubes/s", "h2d_bytes_per_step": int(h2d),
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
            tsum, fr = 0.0, []
            for g in sample:
                v, cores, _, f = cpu_baseline(g, b / len(sample))
                tsum += 1.0 / v
                fr.append(f)
            return (len(sample) / tsum, cores,
                    f"reference per-pixel loop (numpy restatement) on {len(sample)} sampled "
                    f"galaxies of {len(gals)}, each on a pixel sample, extrapolated linearly to "
                    f"whole cubes", float(np.mean(fr)) * len(sample) / len(gals))
    else:
        w = workloads.build(a.workload, n=a.n)

        def one(b):
            return cpu_baseline(w, b)
    for _ in range(a.warmup):
        one(budget / 4)
    vals, fracs = [], []
    t0 = time.perf_counter()
    for _ in range(a.steps):
        v, cores, desc, frac = one(budget)
        vals.append(v)
        fracs.append(frac)
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
                         "sample": desc, "extrapolated": True,
                         "timed_fraction": float(np.mean(fracs))},
        "e2e": {"value": value, "unit": "cubes/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "wall_s": wall,
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
