"""E-step throughput benchmark (particles/s) on the box-256 configuration.

Workload: relion_refine's expectation step (coarse search, significance,
fine search, weighted sums, backprojection) on synthetic particles of the
"plain GPU vs reference CPU at production size" configuration: box 256 px,
1.0 A/px, 5,000-Gaussian volume in a 90 px radius, defocus 0.8-2.5 um,
SNR 0.03, initial reference low-passed to 20 A (first iteration: current
size 46 px), HEALPix order 3 (768 directions x 48 psi), offsets +/-6 px
step 1 (113 translations), oversampling 1, one class, C1.

A step is one E-step call on a batch of --batch particles (default 768:
the per-call fixed work -- two host synchronisations, the host
finalisation, the small launches -- is ~4 % of a call there; particles/s
rises by 1 % more from 768 to 1024).  `value` uses
inputs already resident in HBM; `e2e` calls the same C-ABI entry point with
pinned host buffers (host->device copies inside the timed region).  The L2
cache is flushed (a 512 MB write) before every timed step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--batch B] [--impl reference]

With torchrun (N > 1) each rank runs an independent replica on its own GPU
("replicas only": particles are independent; no collective on the data
path); rank 0 prints the aggregate.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "E-step particles/s @box256, 1 GB300: learned+batched vs plain GPU at equal FSC"
CONFIG = "cfg1_box256"
# reference arm: particles of the batch per step (the oracle takes ~1 s per
# box-256 particle on 16 host threads)
REF_PARTICLES_PER_STEP = 2

# DRAM bytes of one coarse cross-term GEMM launch (plain FP32 path) from an
# ncu capture of a 16-particle batch: the projection-table read is independent
# of the batch, the diff2 write grows with it.
NCU_CROSS_B16 = {"read": 262.75e6, "write": 222.41e6, "batch": 16}
# dram__bytes_read.sum / dram__bytes_write.sum of one k_tc_diff2<0> launch at
# the bench's batch of 768 (ncu, one-pass metrics, full-size capture)
NCU_TC = {"read": 3.326e9, "write": 0.755e9, "batch": 768}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=768)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mstep", action="store_true", help="skip the reconstruction-side section (profiling runs)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP32 path leg (profiling runs)")
    ap.add_argument("--no-late", action="store_true", help="skip the late-iteration section (profiling runs)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="skip the autotuner; the worker keeps its defaults and --options (profiling runs)")
    ap.add_argument("--options", default="{}",
                    help="worker options as JSON (e.g. '{\"bp_direct\": 1}'), set before the autotuner")
    ap.add_argument("--workload", default=CONFIG,
                    choices=["cfg1_box256", "cfg1_box256_late", "cfg1_box128_late", "cfg4_box256_K4", "cfg3_box128_2d",
                             "cfg0_box64"],
                    help="dataset shape (the headline line is cfg1_box256; the others for reference figures; "
                         "cfg1_box256_late: the same refinement in a late iteration, current size 256; "
                         "cfg1_box128_late: the late shape at box 128, small enough for profiler captures)")
    ap.add_argument("--precision", default="bf16", choices=["fp32", "bf16"],
                    help="coarse cross term: plain FP32 SIMT or tcgen05 BF16 (precision form)")
    return ap.parse_args()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def run_ours(args, world, rank, local):
    import torch
    from relion_gb300 import datagen
    from relion_gb300.estep import MlDeviceBundle, MlOptimiserCuda, STAGES, measure_fp32_peak

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    B = args.batch
    ds = datagen.Dataset(args.workload, seed=args.seed + rank, n_particles=B, device=str(dev))
    model = ds.model(precision=1 if args.precision == "bf16" else 0)
    batch = ds.particles(0, B)
    bundle = MlDeviceBundle(model, device=local)
    for k, r in enumerate(ds.refs):
        bundle.setup_projector(k, r["data"], r["yinit"], r["zinit"], r["r_max"], r["pad"])
    bundle.reserve(64 << 30)
    worker = MlOptimiserCuda(bundle, **json.loads(args.options))

    # device-resident copy of the batch (for `value`) and pinned host copy (for `e2e`)
    keys = ("fimg", "fimg_nomask", "fctf", "power_img", "old_offset", "prior", "highres_Xi2",
            "norm_correction", "scale")
    dtypes = dict(fimg=torch.complex64, fimg_nomask=torch.complex64, fctf=torch.float32)
    dev_t, pin = {}, {}
    for k in keys:
        t = torch.from_numpy(np.ascontiguousarray(batch[k])).to(dtypes.get(k, torch.float64))
        pin[k] = t.pin_memory()
        dev_t[k] = t.to(dev)
    dev_batch = {"n": B, "device_resident": 1}
    dev_batch.update({k: v.data_ptr() for k, v in dev_t.items()})
    host_batch = {"n": B}
    host_batch.update({k: v.numpy() for k, v in pin.items()})
    h2d = sum(pin[k].numel() * pin[k].element_size() for k in keys)

    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)

    # tile order, coarse-kernel form and fine-pass form picked on this batch
    # (the autotuner clears the sums its own runs added)
    from relion_gb300 import autotune
    if args.no_autotune:
        tuned = {"options": json.loads(args.options), "coarse": [], "fine": [], "cached": False}
    else:
        tuned = autotune.tune(bundle, worker, dev_batch, repeats=2)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    for _ in range(args.warmup):
        worker.do_expectation_some_particles(dev_batch)
    torch.cuda.synchronize()

    # ---- value: device-resident inputs; each step is the whole library call
    # bracketed by CUDA events (host gaps inside the call included) ----
    stage0 = worker.stage_times().copy()
    launches0 = worker.launch_count()
    barrier()
    torch.cuda.synchronize()
    step_ms, stage_sum_ms = [], []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            before = worker.stage_times().sum()
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record()
            res = worker.do_expectation_some_particles(dev_batch)
            ev1.record()
            ev1.synchronize()
            step_ms.append(ev0.elapsed_time(ev1))
            stage_sum_ms.append(worker.stage_times().sum() - before)
        torch.cuda.synchronize()
    barrier()
    stage = (worker.stage_times() - stage0) / args.steps
    launches = (worker.launch_count() - launches0) // args.steps
    total_ms = float(sum(step_ms))

    # ---- e2e: host (pinned) buffers through the same C-ABI call ----
    e2e_ms = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        worker.do_expectation_some_particles(host_batch)
        ev1.record()
        ev1.synchronize()
        e2e_ms.append(ev0.elapsed_time(ev1))
    e2e_total = float(sum(e2e_ms))

    # ---- e2e from raw images: image preparation on the device + E-step per
    # call (gbr_expect_images), real-space images in pinned host memory ----
    bundle.set_optics(kV=300.0, Cs=2.7, Q0=0.1, particle_diameter=ds.cfg["diameter"], width_mask_edge=5.0)
    ib = ds.particle_images(0, B)
    img_batch = {}
    for k in ("images", "old_offset", "prior", "norm_correction", "scale", "ctf"):
        t = torch.from_numpy(np.ascontiguousarray(ib[k])).pin_memory()
        img_batch[k] = t.numpy()
    h2d_img = sum(v.nbytes for v in img_batch.values())
    worker.do_expectation_images(img_batch)  # plan creation outside the timed steps
    img_stage0 = worker.stage_times().copy()
    img_ms = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        worker.do_expectation_images(img_batch)
        ev1.record()
        ev1.synchronize()
        img_ms.append(ev0.elapsed_time(ev1))
    img_total = float(sum(img_ms))
    img_stage = (worker.stage_times() - img_stage0) / args.steps

    # ---- the same, streaming: each step's images are staged (copied on the
    # worker's copy stream) while the previous step computes ----
    worker.stage_images(img_batch)
    worker.do_expectation_images(img_batch)
    torch.cuda.synchronize()
    flush.zero_()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    worker.stage_images(img_batch)
    for i in range(args.steps):
        if i + 1 < args.steps:
            # the next step's batch (the same host arrays: a full copy each step)
            worker.stage_images(img_batch)
        worker.do_expectation_images(img_batch)
    ev1.record()
    ev1.synchronize()
    stream_total = float(ev0.elapsed_time(ev1))

    if world > 1:
        from relion_gb300.replicas import max_over_ranks
        total_ms, e2e_total, img_total, stream_total = max_over_ranks([total_ms, e2e_total, img_total, stream_total],
                                                                      device=dev)

    # ---- the plain FP32 path on the same batch (the metric's denominator) ----
    plain = None
    if args.precision == "bf16" and not args.no_plain:
        plain = plain_section(args, ds, model, dev_batch, host_batch, h2d, flush, local)
        if world > 1:
            from relion_gb300.replicas import max_over_ranks
            plain["total_ms"], plain["e2e_total_ms"] = max_over_ranks([plain["total_ms"], plain["e2e_total_ms"]],
                                                                      device=dev)

    extra = rank == 0 and not args.no_mstep and args.workload == CONFIG  # sections of the headline workload
    mstep = mstep_section(args, ds, model, bundle, worker, dev_batch, local) if extra else None
    io = io_section(ds, ib, model) if extra else None
    learned = (learned_section(args, ds, model, bundle, worker, batch, dev_batch, res, flush, local,
                               world * B * args.steps / (total_ms * 1e-3))
               if extra and args.precision == "bf16" else None)

    # ---- roofline of the dominant kernel: the coarse cross-term GEMM ----
    R = bundle.nr_classes * bundle.ndir * bundle.npsi
    T = bundle.ntrans
    nc = active_coarse_pixels(model)
    flops = 2.0 * R * (B * T) * (2 * nc)
    cross_ms = float(stage[STAGES.index("cross_gemm")])
    achieved = flops / (cross_ms * 1e-3) / 1e12
    if args.precision == "bf16":
        peak, bound = measured_peaks().get("bf16_tflops"), "tensor"
        peak_src = "MEASURED_PEAKS.json bf16_tflops (burst, cuBLAS bf16)"
        kname = "coarse cross-term GEMM, tcgen05 BF16 (k_tc_diff2)"
        if not peak:
            peak, peak_src = 1900.0, "fallback 1.9 PFLOP/s bf16 burst"
    else:
        peak, bound = measure_fp32_peak(local), "fp32"
        peak_src = "measured live (gbr_measure_fp32_peak: FMA chains on all SMs)"
        kname = "coarse cross-term GEMM, FP32 SIMT (k_gemm<RowsK,CrossY,Diff2Epi>)"
    d2h = B * (96 + (model["ori_size"] // 2 + 1) * 8 + 64) + (R + 2) * 8
    out = {
        "metric": METRIC,
        "value": world * B * args.steps / (total_ms * 1e-3),
        "unit": "particles/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "bf16 (coarse cross term) / fp32 (fine pass) / f64 (sums, volumes)"
                 if args.precision == "bf16" else "fp32 / f64 (sums, volumes)",
        "data": "synthetic (seeded Gaussian-blob volume, analytic Fourier slices, CTF, white noise)",
        "config": {"workload": workload_text(args.workload, model, bundle.nr_classes, bundle.ndir, bundle.npsi,
                                             bundle.ntrans)},
        "run": {"batch_particles": B,
                "precision": "precision form: tcgen05 BF16 coarse pass, FP32 fine pass"
                             if args.precision == "bf16" else "plain FP32 path",
                "l2": "flushed (512 MB write) before every timed step",
                "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": world * B * args.steps / (e2e_total * 1e-3), "unit": "particles/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "e2e_from_images": {"value": world * B * args.steps / (img_total * 1e-3), "unit": "particles/s",
                            "h2d_bytes_per_step": int(h2d_img), "d2h_bytes_per_step": int(d2h),
                            "note": "raw real-space images (pinned host): image preparation on the device "
                                    "(cuFFT, mask, spectra, CTF) + E-step per call, as the reference's "
                                    "doThreadExpectationSomeParticles does",
                            "stage_ms": {k: round(float(v), 4) for k, v in zip(STAGES, img_stage)
                                         if k in ("image_upload", "image_prep", "cross_gemm")}},
        "e2e_from_images_streaming": {"value": world * B * args.steps / (stream_total * 1e-3), "unit": "particles/s",
                                      "h2d_bytes_per_step": int(h2d_img), "d2h_bytes_per_step": int(d2h),
                                      "note": "as e2e_from_images, with each step's upload staged on the "
                                              "worker's copy stream during the previous step (gbr_stage_images); "
                                              "one timed region over all steps"},
        "gpu_launches": int(launches),
        "autotune": {"options": tuned["options"],
                     "cross_term_ms": [[o, round(float(v), 4)] for o, v in tuned["coarse"]],
                     "fine_stages_ms": [[o, round(float(v), 4)] for o, v in tuned["fine"]],
                     "note": "measured on the bench batch before the warm-up steps; each candidate on the "
                             "stages it changes"},
        "roofline": {"bound": bound, "kernel": kname,
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                     "peak_source": peak_src,
                     "traffic": (NCU_CROSS_B16["read"] + NCU_CROSS_B16["write"] * B / NCU_CROSS_B16["batch"])
                     if args.precision == "fp32" else
                     ((NCU_TC["read"] + NCU_TC["write"])
                      if B == NCU_TC["batch"] and args.workload == CONFIG else None),
                     "traffic_note": "ncu dram read+write of a 16-particle launch, write scaled to the batch"
                     if args.precision == "fp32" else
                     "ncu dram read+write of one full-size launch at batch 768 (one-pass metrics); "
                     "algorithmic: 0.13 GB orientation tiles + 0.31 GB particle columns read once, diff2 "
                     "written only near each particle's running minimum; the particle columns are read "
                     "once per group of 32 orientation tiles (9 groups, 2.8 GB), the kernel is bound by "
                     "the tensor pipe's operand feed, not by HBM (0.6 TB/s)"},
        "stage_ms": {k: round(float(v), 4) for k, v in zip(STAGES, stage)},
        "stage_sum_ms_per_step": float(sum(stage_sum_ms)) / args.steps,
        "mean_nr_sign": float(np.mean(res["nr_sign"])),
        "mean_fine_poses": float(np.mean(res["n_fine"])),
    }
    if plain is not None:
        pv = world * B * args.steps / (plain.pop("total_ms") * 1e-3)
        pe = world * B * args.steps / (plain.pop("e2e_total_ms") * 1e-3)
        plain["value"], plain["e2e"]["value"] = pv, pe
        out["plain"] = plain
        out["vs_plain"] = {"value": out["value"] / pv, "e2e": out["e2e"]["value"] / pe,
                           "note": "this line's value / the plain FP32 path's, same batch and timing"}
    if rank == 0:
        out["clocks"] = clk.summary()
        out["mstep"] = mstep
        out["io"] = io
        out["learned"] = learned
    return out, ds, batch, model


def plain_section(args, ds, model, dev_batch, host_batch, h2d, flush, local):
    """The plain FP32 path (FP32 SIMT cross term and norms, every coarse row
    read, full diff2 stores) on the same batch, timed like the headline:
    device-resident steps, then host-buffer (e2e) steps, L2 flushed before
    each.  Its roofline: the FP32 cross-term GEMM against the live-measured
    FP32 FMA peak (the bound of this path), next to the HBM byte model of the
    reference's unfused plain path (bytes per particle below)."""
    import torch
    from relion_gb300.estep import MlDeviceBundle, MlOptimiserCuda, STAGES, measure_fp32_peak
    B = dev_batch["n"]
    b = MlDeviceBundle(dict(model, precision=0), device=local)
    for k, r in enumerate(ds.refs):
        b.setup_projector(k, r["data"], r["yinit"], r["zinit"], r["r_max"], r["pad"])
    b.reserve(64 << 30)
    w = MlOptimiserCuda(b)
    for _ in range(max(1, min(args.warmup, 2))):
        w.do_expectation_some_particles(dev_batch)
    torch.cuda.synchronize()

    def timed(batch):
        ms = []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record()
            w.do_expectation_some_particles(batch)
            ev1.record()
            ev1.synchronize()
            ms.append(ev0.elapsed_time(ev1))
        return float(sum(ms))
    st0 = w.stage_times().copy()
    total = timed(dev_batch)
    stage = (w.stage_times() - st0) / args.steps
    e2e_total = timed(host_batch)
    R = b.nr_classes * b.ndir * b.npsi
    T = b.ntrans
    nc = active_coarse_pixels(model)
    cross_ms = float(stage[STAGES.index("cross_gemm")])
    achieved = 2.0 * R * (B * T) * (2 * nc) / (cross_ms * 1e-3) / 1e12
    peak = measure_fp32_peak(local)
    # HBM byte model of the reference's plain path per particle (unfused):
    # image, CTF and noise weights; the coarse diff2 / weight array written and
    # read ~8 times (min, exp, max, filter, sort, scan, threshold); the coarse
    # projections shared by the batch
    npix_f = model["current_size"] * (model["current_size"] // 2 + 1)
    per_part = npix_f * 16 + 8 * R * T * 4 + R * nc * 8 / B
    step_s = total * 1e-3 / args.steps
    hbm = measured_peaks().get("hbm_gbs")
    w.close()
    b.close()
    return {"total_ms": total, "e2e_total_ms": e2e_total,
            "ms_per_step": total / args.steps,
            "unit": "particles/s", "dtype": "fp32 (cross term, norms, fine pass) / f64 (weight sums, volumes)",
            "e2e": {"unit": "particles/s", "h2d_bytes_per_step": int(h2d)},
            "stage_ms": {k: round(float(v), 4) for k, v in zip(STAGES, stage) if v > 0},
            "roofline": {"bound": "fp32", "kernel": "coarse cross-term GEMM, FP32 SIMT (k_gemm<RowsK,CrossY,Diff2Epi>)",
                         "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                         "peak_source": "measured live (gbr_measure_fp32_peak: FMA chains on all SMs)"},
            "hbm_model": {"bytes_per_particle": per_part,
                          "achieved_GBps": per_part * B / step_s / 1e9,
                          "peak_GBps": hbm, "frac": (per_part * B / step_s / 1e9 / hbm) if hbm else None,
                          "note": "the reference's unfused plain-path byte model (image + CTF + noise weights, "
                                  "coarse diff2 array written and read 8 times, projections shared by the batch) "
                                  "over this path's step time; this path stores the diff2 array once and reads it "
                                  "once, and its time goes to the FP32 contraction"}}


def _slice_batch(batch, sl, n):
    out = {k: (v[sl] if isinstance(v, np.ndarray) and v.ndim >= 1 and v.shape[0] == n else v)
           for k, v in batch.items()}
    out["n"] = len(range(n)[sl])
    return out


def _half_set_maps(model, ds, batch, local, blocks=None):
    """Gold-standard check of one path: the batch split into two halves, each
    half's E-step (optionally restricted to `blocks`) and reconstruction
    (updateSSNRarrays, MAP) in its own bundle; returns the half maps and
    their FSC."""
    from relion_gb300.estep import MlDeviceBundle, MlOptimiserCuda
    n = batch["n"]
    ns = model["ori_size"] // 2 + 1
    maps = []
    for h in range(2):
        sl = slice(h * n // 2, (h + 1) * n // 2)
        b = MlDeviceBundle(model, device=local)
        r = ds.ref
        b.setup_projector(0, r["data"], r["yinit"], r["zinit"], r["r_max"], r["pad"])
        w = MlOptimiserCuda(b)
        w.do_expectation_some_particles(_slice_batch(batch, sl, n), blocks=None if blocks is None else blocks[sl])
        ws = b.get_wsum()
        b.symmetrise(0)
        s = b.update_ssnr_arrays(0, 1.0, np.full(ns, 1.0))
        maps.append(b.reconstruct(0, do_map=True, tau2=s["tau2"], normalise=ws["pdf_class"][0]))
        w.close()
        b.close()
    b = MlDeviceBundle(model, device=local)
    fsc = b.fsc(maps[0], maps[1])
    b.close()
    return maps, fsc


def _angles_between(ra, rb):
    """Angle (degrees) between rotation matrices [n, 3, 3]."""
    tr = np.einsum("nij,nij->n", ra, rb)
    return np.degrees(np.arccos(np.clip((tr - 1.0) / 2.0, -1.0, 1.0)))


def learned_section(args, ds, model, bundle, worker, batch, dev_batch, res_ex, flush, local, value_ex,
                    train_steps=2000, posterior_steps=400, blocks_per_particle=24, mass_threshold=0.9):
    """Learned pose proposal on this workload, judged by the exhaustive search.

    The network is trained on the device on views of the current reference
    (CTFs of this batch, the model's noise), then on the E-step's own
    posteriors (the exhaustive E-step's best directions) of a second batch
    of the workload.  For the timed batch it proposes orientation blocks
    (four sibling directions x every psi): each particle scores its
    `blocks_per_particle` most probable blocks, or everything when they hold
    less than `mass_threshold` of its probability.  A timed learned step is
    the proposal (features, network, top blocks) plus the restricted E-step
    (gbr_expect_batch_blocks), L2 flushed before each.  Judged against the
    exhaustive precision form on the same batch: best-pose agreement and
    angular error, the fine-posterior mass the restriction leaves out on a
    seeded subset (its total-variation distance to the exhaustive
    posterior), and the FSC and gold-standard FSC-0.143 resolution of
    half-set maps reconstructed from each path."""
    import torch
    from relion_gb300 import datagen
    from relion_gb300.estep import MlDeviceBundle, MlOptimiserCuda
    from relion_gb300.iteration import resolution_at
    from relion_gb300.posenet import BlockProposer, PoseProposer, best_directions, direction_targets
    B = dev_batch["n"]
    out = {}
    net = PoseProposer(bundle, nangle=24, max_batch=256, seed=1)
    t0 = time.perf_counter()
    loss = net.train(batch["fctf"], steps=train_steps, batch=256, lr=2e-3)
    out["train_views_s"] = round(time.perf_counter() - t0, 2)
    out["train_views_steps"] = train_steps
    out["loss_views"] = round(float(loss), 4)
    # the E-step's own posteriors of a second batch of the workload (untimed
    # exhaustive E-step): the first half trains the network, the second half
    # (held out) calibrates its softmax temperature
    b2 = ds.particles(B, B)
    w2 = MlOptimiserCuda(bundle)
    r2 = w2.do_expectation_some_particles(b2)
    w2.close()
    h = B // 2
    t0 = time.perf_counter()
    loss2 = net.train_targets(b2["fimg"][:h], direction_targets(bundle, r2[:h], smoothing=0.1),
                              steps=posterior_steps, batch=min(256, h), lr=5e-4)
    out["train_posteriors_s"] = round(time.perf_counter() - t0, 2)
    out["train_posteriors_steps"] = posterior_steps
    out["train_posteriors_particles"] = h
    out["loss_posteriors"] = round(float(loss2), 4)
    best = best_directions(bundle, res_ex)
    recall = {}
    for k in (16, 8, 4):
        M = net.ndir // k
        idx, _ = net.propose(batch["fimg"], M)
        recall["ndir/%d" % k] = {"M": int(M), "recall": round(float(np.mean([best[i] in idx[i] for i in range(B)])), 4),
                                 "uniform": round(M / net.ndir, 4)}
    out["recall_exhaustive_best_direction"] = recall
    prop = BlockProposer(net, bundle, blocks_per_particle, mass_threshold)
    out["temperature"] = prop.calibrate(b2["fimg"][h:], best_directions(bundle, r2[h:]))
    out["calibration_particles"] = B - h
    nblk, dpb, rows = bundle.orientation_blocks()
    blocks = prop(batch["fimg"])
    fallback = prop.last["fallback"]
    scored = np.where(fallback, nblk, np.minimum(blocks_per_particle, nblk) * bundle.nr_classes)
    out.update(blocks_per_particle=int(blocks_per_particle), mass_threshold=mass_threshold,
               blocks_total=int(nblk), fallback_fraction=round(float(np.mean(fallback)), 4),
               scored_orientation_fraction=round(float(np.sum(scored)) / (B * nblk), 4),
               proposal_mass_median=round(float(np.median(prop.last["mass"])), 4))
    # ---- timed learned steps: proposal + restricted E-step, both on the
    # device-resident batch (the proposer reads the images in place) ----
    fimg_dev = torch.from_numpy(np.ascontiguousarray(batch["fimg"])).to(torch.complex64).to(
        torch.device("cuda", local))
    for _ in range(max(1, min(args.warmup, 3))):
        worker.do_expectation_some_particles(dev_batch, blocks=prop(fimg_dev))
    torch.cuda.synchronize()
    ms, prop_ms = [], []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        t0 = time.perf_counter()
        blk = prop(fimg_dev)
        prop_ms.append(1e3 * (time.perf_counter() - t0))
        res_l = worker.do_expectation_some_particles(dev_batch, blocks=blk)
        ev1.record()
        ev1.synchronize()
        ms.append(ev0.elapsed_time(ev1))
    v_learned = B * args.steps / (sum(ms) * 1e-3)
    out["value"] = v_learned
    out["unit"] = "particles/s"
    out["ms_per_step"] = sum(ms) / args.steps
    out["propose_ms"] = round(float(np.mean(prop_ms)), 3)
    out["vs_exhaustive"] = v_learned / value_ex
    # training per iteration amortised over the configuration's particle count
    n_cfg = int(datagen.CONFIGS[args.workload]["n_particles"])
    t_tr = out["train_views_s"] + out["train_posteriors_s"]
    out["amortised"] = {"particles_per_iteration": n_cfg, "training_s": round(t_tr, 2),
                        "value": n_cfg / (n_cfg / v_learned + t_tr),
                        "note": "particles/s of one iteration over the configuration's particle set with the "
                                "network trained once in it"}
    # ---- judged by the exhaustive search ----
    eq = res_l["best_ihidden_over"] == res_ex["best_ihidden_over"]
    ra = datagen.euler_matrices(res_l["rot"], res_l["tilt"], res_l["psi"]).numpy()
    rb = datagen.euler_matrices(res_ex["rot"], res_ex["tilt"], res_ex["psi"]).numpy()
    ang = _angles_between(ra, rb)
    rt = np.asarray(batch["true_rot"])
    out["pose"] = {"best_pose_agreement": round(float(np.mean(eq)), 4),
                   "angle_to_exhaustive_deg_mean": round(float(np.mean(ang)), 3),
                   "angle_to_exhaustive_deg_p99": round(float(np.percentile(ang, 99)), 3),
                   "angle_to_truth_deg_median_learned": round(float(np.median(_angles_between(ra, rt))), 3),
                   "angle_to_truth_deg_median_exhaustive": round(float(np.median(_angles_between(rb, rt))), 3),
                   "pmax_abs_diff_mean": round(float(np.mean(np.abs(res_l["pmax"] - res_ex["pmax"]))), 6)}
    # weight divergence on a seeded subset: exhaustive fine posterior mass in unscored blocks
    nsub = min(24, B)
    sub = _slice_batch(batch, slice(0, nsub), B)
    bd = MlDeviceBundle(model, device=local)
    r = ds.ref
    bd.setup_projector(0, r["data"], r["yinit"], r["zinit"], r["r_max"], r["pad"])
    wd = MlOptimiserCuda(bd, debug=True)
    wd.do_expectation_some_particles(sub)
    tv = []
    per = bd.nover_rot * bd.nover_trans * bd.ntrans
    for i in range(nsub):
        idx = wd.debug_fetch(2, i)
        wf = wd.debug_fetch(4, i)
        fblk = (idx // per // bd.npsi) // dpb
        if fallback[i]:
            tv.append(0.0)
            continue
        keep = np.isin(fblk, blocks[i][blocks[i] >= 0])
        tv.append(float(np.sum(wf[~keep]) / max(np.sum(wf), 1e-300)))
    wd.close()
    bd.close()
    out["weight_divergence"] = {"particles": nsub, "tv_mean": float(np.mean(tv)), "tv_max": float(np.max(tv)),
                                "note": "exhaustive fine-posterior mass outside the scored blocks (total-variation "
                                        "distance of the restricted posterior to the exhaustive one)"}
    # FSC: half-set maps of each path, same particles
    m_l, f_l = _half_set_maps(model, ds, batch, local, blocks=blk)
    m_e, f_e = _half_set_maps(model, ds, batch, local)
    m_p, f_p = _half_set_maps(dict(model, precision=0), ds, batch, local)
    cur = model["current_size"]
    rmax = cur // 2
    # resolution over the shells inside the current size (beyond it the maps
    # hold no data)
    f_l, f_e, f_p = f_l[:rmax + 1], f_e[:rmax + 1], f_p[:rmax + 1]
    b = MlDeviceBundle(model, device=local)
    f_le = b.fsc(m_l[0], m_e[0])
    b.close()
    ori, pix = model["ori_size"], model["pixel_size"]
    out["fsc"] = {"resolution_A_learned": resolution_at(f_l, ori, pix),
                  "resolution_A_exhaustive": resolution_at(f_e, ori, pix),
                  "resolution_A_plain": resolution_at(f_p, ori, pix),
                  "half_map_fsc_max_abs_diff_learned_vs_plain": round(float(np.max(np.abs(f_l[1:rmax] - f_p[1:rmax]))), 5),
                  "min_fsc_learned_vs_exhaustive_map": round(float(np.min(f_le[1:rmax])), 6),
                  "shells": "1..%d (inside the current size)" % (rmax - 1),
                  "note": "gold-standard FSC-0.143 of two half-set maps (%d particles each) per path; first "
                          "iteration, so the current size bounds the resolution" % (B // 2)}
    net.close()
    return out


def io_section(ds, ib, model):
    """Data formats: the batch's raw images written as an MRC stack with a
    RELION 3.1 STAR file, then read back through the native reader (page
    cache warm: the second of two reads is timed)."""
    import shutil
    import tempfile
    import time
    from relion_gb300 import io as gio
    d = tempfile.mkdtemp()
    try:
        n, box, pix = ib["images"].shape[0], model["ori_size"], model["pixel_size"]
        stack = os.path.join(d, "parts.mrcs")
        gio.write_mrc_stack(stack, ib["images"], pix)
        star = os.path.join(d, "parts.star")
        gio.write_star(star, {"optics": {"rlnOpticsGroup": [1], "rlnVoltage": [300.0],
                                         "rlnSphericalAberration": [2.7], "rlnAmplitudeContrast": [0.1],
                                         "rlnImagePixelSize": [pix], "rlnImageSize": [box]},
                              "particles": {"rlnImageName": ["%06d@parts.mrcs" % (i + 1) for i in range(n)],
                                            "rlnDefocusU": list(ib["ctf"][:, 0]), "rlnDefocusV": list(ib["ctf"][:, 1]),
                                            "rlnDefocusAngle": list(ib["ctf"][:, 2]),
                                            "rlnOriginXAngst": [0.0] * n, "rlnOriginYAngst": [0.0] * n,
                                            "rlnOpticsGroup": [1] * n}})
        out = np.empty((n, box, box), np.float32)
        threads = min(16, os.cpu_count() or 1)
        for _ in range(2):
            t0 = time.perf_counter()
            gio.read_mrc_images(stack, out=out, nthreads=threads)
            t_mrc = time.perf_counter() - t0
        for _ in range(2):
            t0 = time.perf_counter()
            lb = gio.load_particles(star, nthreads=threads)
            t_load = time.perf_counter() - t0
        assert np.array_equal(lb["images"], ib["images"])
        return {"mrc_read_GBps": round(out.nbytes / t_mrc / 1e9, 2), "load_particles_per_s": round(n / t_load),
                "threads": threads, "note": "%d images of %d^2 float32 (%.0f MB), page cache warm; "
                "load_particles = STAR parse + MRC read into the image batch" % (n, box, out.nbytes / 1e6)}
    finally:
        shutil.rmtree(d, ignore_errors=True)


def mstep_section(args, ds, model, bundle, worker, dev_batch, local):
    """Reconstruction side of the iteration on the device, timed once per
    call (host wall clock around each synchronous C-ABI call, map copies
    included): symmetrise, updateSSNRarrays, reconstruct and
    computeFourierTransformMap of this batch's volumes at the workload's
    sizes, and reconstruct at the Nyquist-limited size (current 256).  Also
    the equal-FSC check of the precision form: the same batch through the
    plain FP32 path, both volumes reconstructed, FSC between the two maps."""
    import time
    from relion_gb300.estep import MlDeviceBundle, MlOptimiserCuda

    ori, cur = model["ori_size"], model["current_size"]
    ns = ori // 2 + 1
    out = {}

    def timed(name, fn):
        t0 = time.perf_counter()
        r = fn()
        out[name] = round((time.perf_counter() - t0) * 1e3, 3)
        return r

    def chain(b, prefix, sym):
        if sym:
            b.symmetrise(0)
        ws = b.get_wsum()
        s = timed(prefix + "update_ssnr_ms", lambda: b.update_ssnr_arrays(0, 1.0, np.full(ns, 1.0)))
        vol = timed(prefix + "reconstruct_ms", lambda: b.reconstruct(0, do_map=True, tau2=s["tau2"],
                                                                    normalise=ws["pdf_class"][0]))
        return vol

    bundle.reset_wsum()
    worker.do_expectation_some_particles(dev_batch)
    timed("symmetrise_ms", lambda: bundle.symmetrise(0))
    bundle.set_fourier_transform_map(0, bundle.reconstruct(0), cur)  # FFT plans outside the timed calls
    vol = chain(bundle, "", False)  # symmetrised above
    timed("projector_from_map_ms", lambda: bundle.set_fourier_transform_map(0, vol, cur))
    out["sizes"] = "current %d: padded Fourier grid %d^3, real-space transform %d^3" % (
        cur, bundle.backprojector_dims()[1], 2 * ori)
    # FP32 transforms, map kept on the device between the two calls
    ws0 = bundle.get_wsum()
    s0 = bundle.update_ssnr_arrays(0, 1.0, np.full(ns, 1.0))
    kw = dict(do_map=True, tau2=s0["tau2"], normalise=ws0["pdf_class"][0])
    bundle.set_recon_precision(True)
    bundle.set_fourier_transform_map(0, bundle.reconstruct(0, **kw), cur)  # FP32 plans
    vol_f = timed("fp32_reconstruct_ms", lambda: bundle.reconstruct(0, **kw))
    timed("fp32_reconstruct_on_device_ms", lambda: bundle.reconstruct(0, to_host=False, **kw))
    timed("fp32_projector_from_device_map_ms", lambda: bundle.set_fourier_transform_map(0, None, cur))
    bundle.set_recon_precision(False)
    out["fp32_map_rel_l2_vs_fp64"] = float(np.linalg.norm(vol_f - vol) / np.linalg.norm(vol))
    out["transforms"] = "*_ms: FP64 cuFFT (the reference's precision); fp32_*: FP32 cuFFT, FP64 weights and sums"
    # restore the workload's projector for anything run after this section
    r = ds.ref
    bundle.setup_projector(0, r["data"], r["yinit"], r["zinit"], r["r_max"], r["pad"])

    # the same batch through the plain FP32 path; FSC between the two maps
    m32 = dict(model, precision=0)
    b32 = MlDeviceBundle(m32, device=local)
    b32.setup_projector(0, r["data"], r["yinit"], r["zinit"], r["r_max"], r["pad"])
    w32 = MlOptimiserCuda(b32)
    w32.do_expectation_some_particles(dev_batch)
    vol32 = chain(b32, "fp32_path_", True)
    f = bundle.fsc(vol, vol32)
    w32.close()
    b32.close()
    rmax = cur // 2
    out["equal_fsc"] = {"min_fsc_precision_vs_plain": round(float(np.min(f[1:rmax])), 6),
                        "shells": "1..%d (inside the current size)" % (rmax - 1),
                        "note": "maps reconstructed from the same %d particles: BF16 tensor-core coarse "
                                "pass vs plain FP32 path" % dev_batch["n"]}
    for k in ("fp32_path_update_ssnr_ms", "fp32_path_reconstruct_ms"):
        out.pop(k, None)

    # Nyquist-limited size: current 256 (padded grid 515^3, transform 512^3)
    mn = dict(model, current_size=ori, coarse_size=model["coarse_size"])
    bn = MlDeviceBundle(mn, device=local)
    xd, yd, zd = bn.backprojector_dims()[:3]
    rng = np.random.default_rng(1)
    data = (rng.standard_normal((zd, yd, xd)) + 1j * rng.standard_normal((zd, yd, xd))) * 1e-3
    bn.set_mdl_data(0, data, np.ones((zd, yd, xd)))
    del data
    bn.symmetrise(0)
    bn.set_fourier_transform_map(0, bn.reconstruct(0), ori)  # FFT plans outside the timed calls
    timed("nyquist_reconstruct_ms", lambda: bn.reconstruct(0))
    timed("nyquist_projector_from_map_ms", lambda: bn.set_fourier_transform_map(0, vol, ori))
    bn.close()
    return out


def workload_text(name, model, nr_classes, ndir, npsi, ntrans):
    """One line naming the workload with its sizes (both arms print it)."""
    box = model["ori_size"]
    grid = ("%d classes x %d psi" % (nr_classes, npsi) if int(model.get("ref_dim", 3) or 3) == 2
            else "HEALPix %d directions x %d psi, %d class%s" % (ndir, npsi, nr_classes,
                                                                 "" if nr_classes == 1 else "es"))
    stage = "late-iteration" if name.endswith("_late") else "iteration-1"
    return ("%s: box%d E-step, %s sizes (current %d px, coarse %d px), %s, %d translations, "
            "oversampling 1" % (name, box, stage, model["current_size"], model["coarse_size"], grid, ntrans))


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def active_coarse_pixels(model):
    """Coarse pixels with a non-zero noise weight (the K of the cross term / 2)."""
    s = model["coarse_size"]
    X = s // 2 + 1
    n = 0
    for i in range(s):
        y = i if i < X else i - s
        for x in range(X):
            r = int(np.sqrt(x * x + y * y) + 0.5)
            if r < s // 2 + 1 and not (x == 0 and y < 0) and 0 < r < model["sigma2_len"]:
                n += 1
    return n


def cpu_particles_per_s(ds, batch, model, n_particles, threads):
    """Oracle (CPU restatement of the reference's CPU E-step) on n particles
    with `threads` host threads; returns (particles/s, threads in effect).
    The thread count is set through the OpenMP runtime itself: torch has
    started it already, so OMP_NUM_THREADS would no longer be read."""
    from oracle import build as obuild
    obuild.build()
    from oracle import pyoracle
    used = pyoracle.set_threads(threads)
    sub = {k: (v[:n_particles] if isinstance(v, np.ndarray) else v) for k, v in batch.items()}
    sub["n"] = n_particles
    t0 = time.perf_counter()
    pyoracle.run(model, ds.refs, sub)
    return n_particles / (time.perf_counter() - t0), used


def run_reference(args, world, rank):
    """Reference arm: the reference's CPU path for this E-step, as restated
    by the oracle (the reference's relion_refine needs FFTW, MPI and TIFF
    and is not built here), on all host cores, same config and metric."""
    if rank != 0:
        return None
    from relion_gb300 import datagen
    from oracle import pyoracle
    cores = os.cpu_count() or 1
    per_step = REF_PARTICLES_PER_STEP
    # the GPU arm's workload (same generator and seed); each step is a bounded
    # sample of its batch: the first particles of it
    ds = datagen.Dataset(args.workload, seed=args.seed, n_particles=per_step)
    model = ds.model()
    batch = ds.particles(0, per_step)
    for _ in range(args.warmup if args.warmup < 1 else 1):
        cpu_particles_per_s(ds, batch, model, 1, cores)
    t_total, n_total, used = 0.0, 0, 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _, used = cpu_particles_per_s(ds, batch, model, per_step, cores)
        t_total += time.perf_counter() - t0
        n_total += per_step
    v = n_total / t_total
    ndir, npsi, ntr = pyoracle.sampling_sizes(int(model["healpix_order"]), float(model["psi_step"]),
                                             float(model["offset_range"]), float(model["offset_step"]),
                                             int(model.get("ref_dim", 3) or 3))
    return {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "particles/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Gaussian-blob volume, analytic Fourier slices, CTF, white noise)",
        "config": {"workload": workload_text(args.workload, model, int(model["nr_classes"]), ndir, npsi, ntr)},
        "particles_per_step": per_step,
        "cpu_baseline": {"value": v, "unit": "particles/s", "cores": used, "kind": "port",
                         "sample": "%d particles of the GPU arm's batch per step (its first ones), the oracle "
                                   "(FP64 restatement of the reference's CPU E-step) on %d host threads "
                                   "(OpenMP over orientations; %d cores on the host)" % (per_step, used, cores)},
        "e2e": {"value": v, "unit": "particles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def late_section(args, local, B=512, steps=3, warmup=3):
    """The same refinement in a late iteration (cfg1_box256_late: current
    size 256, coarse size 48, reference sharp to Nyquist), a reference figure
    beside the headline: device-resident particles/s and raw images through
    gbr_expect_images, per-stage times, B particles per call."""
    import torch
    from relion_gb300 import datagen
    from relion_gb300.estep import MlDeviceBundle, MlOptimiserCuda, STAGES
    dev = torch.device("cuda", local)
    name = "cfg1_box256_late"
    ds = datagen.Dataset(name, seed=args.seed, n_particles=B, device=str(dev))
    model = ds.model(precision=1)
    batch = ds.particles(0, B)
    t0 = time.time()
    bundle = MlDeviceBundle(model, device=local)
    for k, r in enumerate(ds.refs):
        bundle.setup_projector(k, r["data"], r["yinit"], r["zinit"], r["r_max"], r["pad"])
    bundle.reserve(64 << 30)
    torch.cuda.synchronize()
    setup_s = time.time() - t0
    worker = MlOptimiserCuda(bundle)
    keys = ("fimg", "fimg_nomask", "fctf", "power_img", "old_offset", "prior", "highres_Xi2",
            "norm_correction", "scale")
    dtypes = dict(fimg=torch.complex64, fimg_nomask=torch.complex64, fctf=torch.float32)
    dev_t = {k: torch.from_numpy(np.ascontiguousarray(batch[k])).to(dtypes.get(k, torch.float64)).to(dev)
             for k in keys}
    dev_batch = {"n": B, "device_resident": 1}
    dev_batch.update({k: v.data_ptr() for k, v in dev_t.items()})
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    # the first call builds the iteration's projection tables (every coarse and
    # oversampled orientation at the current size); timed on its own
    t1 = time.time()
    worker.do_expectation_some_particles(dev_batch)
    torch.cuda.synchronize()
    first_call_s = time.time() - t1
    bundle.reset_wsum()
    # the same per-shape choices as the headline worker
    from relion_gb300 import autotune
    tuned = autotune.tune(bundle, worker, dev_batch, repeats=2)

    def timed(call, arg):
        for _ in range(warmup):
            call(arg)
        torch.cuda.synchronize()
        s0 = worker.stage_times().copy()
        ms = []
        res = None
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            res = call(arg)
            e1.record()
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return float(sum(ms)), (worker.stage_times() - s0) / steps, res

    tot, stage, res = timed(worker.do_expectation_some_particles, dev_batch)
    bundle.set_optics(kV=300.0, Cs=2.7, Q0=0.1, particle_diameter=ds.cfg["diameter"], width_mask_edge=5.0)
    ib = ds.particle_images(0, B)
    img_batch = {k: torch.from_numpy(np.ascontiguousarray(ib[k])).pin_memory().numpy()
                 for k in ("images", "old_offset", "prior", "norm_correction", "scale", "ctf")}
    tot_img, stage_img, _ = timed(worker.do_expectation_images, img_batch)
    out = {
        "workload": workload_text(name, model, bundle.nr_classes, bundle.ndir, bundle.npsi, bundle.ntrans),
        "batch_particles": B,
        "value": B * steps / (tot * 1e-3),
        "unit": "particles/s",
        "ms_per_step": tot / steps,
        "e2e_from_images": {"value": B * steps / (tot_img * 1e-3), "unit": "particles/s",
                            "h2d_bytes_per_step": int(sum(v.nbytes for v in img_batch.values()))},
        "stage_ms": {k: round(float(v), 4) for k, v in zip(STAGES, stage) if v > 0},
        "image_stage_ms": {k: round(float(v), 4) for k, v in zip(STAGES, stage_img)
                           if k in ("image_upload", "image_prep")},
        "mean_nr_sign": float(np.mean(res["nr_sign"])),
        "mean_fine_poses": float(np.mean(res["n_fine"])),
        "setup_s": round(setup_s, 2),
        "first_call_s": round(first_call_s, 3),
        "autotune": tuned["options"],
        "note": "setup_s: bundle and reference upload; first_call_s: the first call, which also builds the "
                "projection tables of every coarse and oversampled orientation at current size 256 (once per "
                "iteration); the fine pass, weighted sums and backprojection grow x30 over iteration 1, the "
                "coarse pass barely",
    }
    worker.close()
    bundle.close()
    return out


def main():
    args = parse()
    world, rank, local = dist_setup()
    if world > 1:
        import torch.distributed as dist
        backend = "gloo" if args.impl == "reference" else "nccl"
        dist.init_process_group(backend=backend)
    if args.impl == "reference":
        out = run_reference(args, world, rank)
        if out is not None:
            print(json.dumps(out))
        return
    out, ds, batch, model = run_ours(args, world, rank, local)
    if rank == 0 and not args.no_late and args.workload == CONFIG:
        import gc
        import torch
        gc.collect()
        torch.cuda.empty_cache()
        out["late_iteration"] = late_section(args, local)
    if rank == 0:
        if not args.no_cpu_baseline:
            # bounded sample: one particle on one host thread (~10-30 s)
            v, used = cpu_particles_per_s(ds, batch, model, 1, 1)
            out["cpu_baseline"] = {"value": v, "unit": "particles/s", "cores": used, "kind": "port",
                                   "sample": "1 particle of the same batch, the oracle (FP64 restatement of the "
                                             "reference's CPU E-step) on %d host thread(s)" % used}
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
