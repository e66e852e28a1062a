#!/usr/bin/env python
"""Benchmark of the trace-transform sinogram + circus path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
    python bench.py --impl reference ...

The metric is sinograms per second (sinograms = images x T-functionals), the
measure of "batched vs plain" the path is quoted on.  Default workload
``batch512``: 512 synthetic blob+noise images, sides 64-512 px per axis
(half of them non-square), 180 or 360 angles each, T0-T5 x P1-P3.  A step is
one pass of the whole batch through the batched engine: one replay of its
captured graph (persistent rotate + T-functional kernel over every image,
batched P-functional kernel, batched z-score).  Prints one JSON line (rank 0):

* value        device-resident throughput: the images already in HBM, CUDA
               events around each step, L2 flushed (256 MiB write) between
               steps
* e2e          the same metric through the C ABI (tt_transform_batch) with
               pinned host buffers: images in, circus functions and
               signatures out, inside the timed region
* plain_per_image / batched_over_plain
               the same 512 images through the plain per-image device path
               (one sinogram, circus and z-score launch per image) and the
               drop-in tt_transform per image
* roofline     the persistent sinogram kernel (event-timed inside the graph):
               algorithmic bytes per launch (4 A H W image sweeps + 4 nT N A
               sinogram writes, per image) / its duration, against the
               measured HBM copy bandwidth
* single4096   the 4096^2 workload's fused sinogram kernel (N 5793, 720
               angles, T0-T7): duration and roofline fraction, and its
               backward pass (T0-T2 x P1/P3, rotations recomputed) against
               the forward
* grad64       64 images of 256^2: forward and backward of an MSE loss over
               the circus functions through tracetransform_gb300.autograd
* cpu_baseline the CPU oracle (a C restatement of the reference's float path,
               OpenMP over angles as the reference's openmp/ port) on all
               host cores, on a sample of the batch's images; ``parity``
               accounts every sinogram, circus and signature entry of those
               images against it (oracle/parity.py)

--impl reference times that CPU implementation alone as the reference arm:
every step transforms the next images of the batch, and the reported rate
is the sinograms those steps actually computed over their measured time.
Other workloads (--workload): single256, single1024, single4096 (one image
per step; the last two with the orthonormal Hermite circus beside P1-P3) and
grad64.  Multi-GPU (torchrun): every rank runs its own replica (weak scaling).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "sinograms/sec"
HERMITE = [1, 2, 3, 4, 5]
WORKLOADS = {
    # name: (rows, cols, n_blobs, sigma, seed, angle_step, T list, P list,
    #        Hermite orders of the orthonormal circus beside P1-P3)
    "single256": (256, 256, 8, (8, 40), 1, 1.0, [0, 1, 2, 3, 4, 5], [1, 2, 3], []),
    "single1024": (1024, 1024, 32, (16, 160), 2, 1.0, [0, 1, 2, 3, 4, 5, 6, 7], [1, 2, 3],
                   HERMITE),
    "single4096": (4096, 4096, 256, (32, 640), 6, 0.5, [0, 1, 2, 3, 4, 5, 6, 7], [1, 2, 3],
                   HERMITE),
}
DEFAULT_WORKLOAD = "batch512"
L2_FLUSH_BYTES = 256 << 20
BATCH_T, BATCH_P = [0, 1, 2, 3, 4, 5], [1, 2, 3]
GRAD_T, GRAD_P, GRAD_IMAGES, GRAD_SIDE = [0, 1, 2], [1, 3], 64, 256


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["engine", "reference"], default="engine")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["batch512", "grad64"],
                    default=DEFAULT_WORKLOAD)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="batch512: skip the single4096 and grad64 side measurements")
    ap.add_argument("--kernel-only", type=int, default=0, metavar="CALLS",
                    help="for profiler captures: run only the fused sinogram kernel CALLS "
                         "times on the workload and exit (prints no bench line)")
    ap.add_argument("--profile-steps", type=int, default=0, metavar="STEPS",
                    help="for profiler launch lists: run the workload's full device step "
                         "STEPS times and exit")
    ap.add_argument("--images", type=int, default=0,
                    help="with --profile-steps on batch512: only the first IMAGES images (a "
                         "small case for profiler captures)")
    ap.add_argument("--tile", default=None, metavar="LINES,CTAS_PER_SM,LINES_PER_WARP",
                    help="with --profile-steps on batch512: pin the sinogram kernel's tile "
                         "shape instead of the autotuner's choice")
    ap.add_argument("--tfuncs", default=None,
                    help="comma-separated T-functional ids overriding the workload's")
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="CPU time of the baseline sample")
    return ap.parse_args()


def make_image(name):
    from tracetransform_gb300.synthetic import blob_image
    rows, cols, nb, sigma, seed, step, tfs, pfs, _ = WORKLOADS[name]
    img = blob_image(rows, cols, nb, sigma, (40, 200), seed)
    n_ang = int(np.floor(360.0 / step))
    angles = (np.arange(n_ang, dtype=np.float64) * step).astype(np.float32)
    return img, angles, tfs, pfs


def config_dict(name, n, angles, tfs, pfs, world):
    rows, cols = WORKLOADS[name][:2]
    return {"workload": name, "image": f"{rows}x{cols}", "padded": n, "angles": len(angles),
            "angle_step_deg": WORKLOADS[name][5], "t_functionals": tfs,
            "p_functionals": pfs, "hermite_orders": WORKLOADS[name][8],
            "hermite": ("orthonormal circus on each sinogram's nearest orthonormal sinogram "
                        "(device QR + Jacobi), beside P1-P3") if WORKLOADS[name][8] else None,
            "images_per_step_per_gpu": 1,
            "l2": "flushed between timed steps (256 MiB write)",
            "parallelism": f"replicas{world}" if world > 1 else "single"}


def make_batch():
    from tracetransform_gb300.synthetic import workload
    items = workload("batch512")
    return [im for im, _ in items], [int(s) for _, s in items]


def batch_config(imgs, world):
    return {"workload": "batch512", "images": len(imgs),
            "sides": "rows, cols independently uniform in 64..512",
            "angles": "360 or 180 (step 1 or 2 degrees, p = 1/2)",
            "t_functionals": BATCH_T, "p_functionals": BATCH_P,
            "images_per_step_per_gpu": len(imgs),
            "l2": "inputs 170 MB > L2 and L2 flushed between timed steps",
            "parallelism": f"replicas{world}" if world > 1 else "single"}


def job_rate(units_per_rank, world, ms):
    """Whole-job throughput of a weak-scaling run: every rank processes
    units_per_rank per step and ms is the slowest rank's step time."""
    return world * units_per_rank / (ms / 1e3)


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64,
                     device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
# CPU side (oracle): the reference arm, the timed baseline and parity
# ---------------------------------------------------------------------------

def _oracle():
    from oracle import oracle as O
    O.build()
    return O


def cpu_batch_steps(imgs, steps, per_step, n_steps, start=0):
    """Transform per_step images per step (the batch's next images, wrapping
    around) with the oracle on all host cores -- Transformer + getTransform
    of c++/src/transform.cpp:49-112, OpenMP over angles as openmp/.  Returns
    per-step (seconds, sinograms, images) and the indices transformed."""
    O = _oracle()
    pf = [(p, 0) for p in BATCH_P]
    out, done, i = [], [], start
    for _ in range(n_steps):
        idx = [(i + k) % len(imgs) for k in range(per_step)]
        i += per_step
        t0 = time.perf_counter()
        res = [O.transform(imgs[j], steps[j], BATCH_T, pf) for j in idx]
        dt = time.perf_counter() - t0
        out.append((dt, per_step * len(BATCH_T), idx, res))
        done.extend(idx)
    return out, done


def batch_parity(imgs, steps, idx, results, gpu):
    """Accounts every sinogram, circus and signature entry of the images idx
    (oracle results `results`) against the engine's (gpu: image index ->
    (sinograms (nT, N, A), circus, signatures)), as tests/test_batch_gpu.py
    does; returns the totals and the largest unexcused error per functional."""
    from oracle import oracle as O
    from oracle.parity import account_circus, account_sinograms, zscore_mismatches
    pf = [(p, 0, 0) for p in BATCH_P]
    tot = {"images": 0, "sinogram_entries": 0, "circus_entries": 0, "median_ties": 0,
           "selection_ties": 0, "unexplained": 0, "signature_mismatches": 0}
    worst = {}
    for j, ref in zip(idx, results):
        sino, circ, sig = gpu[j]
        padded = ref["padded"]
        ang = O.angles_for_step(steps[j])
        rs = account_sinograms(padded, ang, BATCH_T, sino, ref["sino"])
        rc = account_circus(sino, pf, circ)
        re = account_circus(ref["sino"], pf, circ, ref=ref["circus"],
                            tie_columns=rs["tie_columns"], key_rtol=1e-4)
        tot["images"] += 1
        tot["sinogram_entries"] += rs["entries"]
        tot["circus_entries"] += rc["entries"]
        tot["median_ties"] += rs["median_ties"]
        tot["selection_ties"] += rs["selection_ties"] + rc["selection_ties"]
        tot["unexplained"] += rs["unexplained"] + rc["unexplained"] + re["unexplained"]
        tot["signature_mismatches"] += zscore_mismatches(circ, sig)
        for rep in (rs, rc):
            for nm, v in rep["per_functional"].items():
                worst[nm] = max(worst.get(nm, 0.0), v["max_rel_unexcused"])
    tot["max_rel_unexcused"] = worst
    tot["criterion"] = ("every entry within 1e-4 relative (column guard 1e-3 of the column "
                        "maximum) of the reference's float path, or a proven tie of its own "
                        "arithmetic; signatures bit-identical to zscore of the circus")
    return tot


def cpu_single_steps(img, angles, tfs, pfs, herm, n_steps, threads=0):
    """One sinogram per step (the T-functionals in turn): its sinogram over
    all angles, P1-P3, z-scores and -- with Hermite orders -- its nearest
    orthonormal sinogram and Hermite circus.  Returns per-step (total s,
    T+P seconds)."""
    O = _oracle()
    padded = O.pad(img)
    out = []
    for s in range(n_steps):
        t = tfs[s % len(tfs)]
        t0 = time.perf_counter()
        sino = O.sinograms(padded, angles, [t], threads)[0]
        circ = O.circus(sino, [(p, 0, 0) for p in pfs], threads)
        for v in circ:
            O.zscore(v)
        t1 = time.perf_counter()
        if herm:
            nos, c = O.nos(sino)
            for v in O.circus(nos, [(0, o, c) for o in herm], threads):
                O.zscore(v)
        out.append((time.perf_counter() - t0, t1 - t0))
    return out


def cpu_angle_sample_steps(img, angles, tfs, pfs, n_steps, per_step, threads=0):
    """Steps of per_step angles (in turn over the angle list) of every
    T-functional with P1-P3 of those columns; for images whose full sinogram
    takes the oracle minutes.  Returns per-step (seconds, sinograms done)."""
    O = _oracle()
    padded = O.pad(img)
    out = []
    for s in range(n_steps):
        sub = angles[(s * per_step + np.arange(per_step)) % len(angles)]
        t0 = time.perf_counter()
        sino = O.sinograms(padded, sub, tfs, threads)
        for t in range(sino.shape[0]):
            O.circus(sino[t], [(p, 0, 0) for p in pfs], threads)
        out.append((time.perf_counter() - t0, len(tfs) * per_step / len(angles)))
    return out


def reference_line(args, world, value, ms, config, cb, extra=None):
    line = {"metric": METRIC, "value": value, "unit": "sinograms/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded blob+noise)", "impl": "reference", "config": config,
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": "sinograms/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    line.update(extra or {})
    print(json.dumps(line), flush=True)


def run_reference(args, world):
    """The reference arm: the CPU path on the workload, every reported step
    executed in full and timed."""
    cores = os.cpu_count() or 1
    if args.workload == "batch512":
        imgs, steps = make_batch()
        per = 8
        _, _ = cpu_batch_steps(imgs, steps, per, args.warmup)
        st, _ = cpu_batch_steps(imgs, steps, per, args.steps, start=per * args.warmup)
        secs = sum(s[0] for s in st)
        sinos = sum(s[1] for s in st)
        value = sinos / secs
        cb = {"value": value, "unit": "sinograms/s", "cores": cores, "kind": "port",
              "sample": f"each step transforms {per} images of the batch in turn (T0-T5 x "
                        f"P1-P3, z-scores), {args.steps} steps = {args.steps * per} images, "
                        f"{secs:.1f} s"}
        reference_line(args, world, value, 1e3 * secs / args.steps,
                       batch_config(imgs, world), cb)
        return
    if args.workload == "grad64":
        print(json.dumps({"impl": "reference", "unavailable": "the reference computes no "
                          "gradients; grad64 has no reference arm"}), flush=True)
        return
    img, angles, tfs, pfs = make_image(args.workload)
    herm = WORKLOADS[args.workload][8]
    n = _oracle().pad_geometry(*img.shape)[0]
    if args.workload == "single4096":
        per = 12
        cpu_angle_sample_steps(img, angles, tfs, pfs, args.warmup, per)
        st = cpu_angle_sample_steps(img, angles, tfs, pfs, args.steps, per)
        secs, sinos = sum(s[0] for s in st), sum(s[1] for s in st)
        desc = (f"each step: {per} of the {len(angles)} angles (in turn) of all "
                f"{len(tfs)} T-functionals with P1-P3; the orthonormal circus is not timed "
                f"at this size (its double Jacobi takes the oracle minutes per sinogram)")
    else:
        cpu_single_steps(img, angles, tfs, pfs, herm, args.warmup)
        st = cpu_single_steps(img, angles, tfs, pfs, herm, args.steps)
        secs, sinos = sum(s[0] for s in st), float(len(st))
        desc = (f"each step: one sinogram (the {len(tfs)} T-functionals in turn) over all "
                f"{len(angles)} angles, P1-P3 and z-scores" +
                (", its nearest orthonormal sinogram and Hermite circus" if herm else ""))
    value = sinos / secs
    cb = {"value": value, "unit": "sinograms/s", "cores": cores, "kind": "port", "sample": desc}
    extra = {}
    if herm and args.workload != "single4096":
        extra["cpu_no_hermite"] = {"value": sinos / sum(s[1] for s in st),
                                   "unit": "sinograms/s",
                                   "note": "the same steps without the orthonormal circus"}
    reference_line(args, world, value, 1e3 * secs / args.steps,
                   config_dict(args.workload, n, angles, tfs, pfs, world), cb, extra)


# ---------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------

def _split_batch(rows, cols, steps, ntf, npf):
    """Per-image offsets into the batch's flat sinogram and circus buffers."""
    import tracetransform_gb300 as tt
    so, co, out = 0, 0, []
    for r, c, s in zip(rows, cols, steps):
        n = tt.pad_geometry(r, c)[0]
        a = 360 // s
        out.append((so, co, n, a))
        so += ntf * a * n
        co += ntf * npf * a
    return out


def run_batch(args, world, rank, local_rank):
    """512 uneven images per step through the batched engine (one graph
    replay), against the same images through the plain per-image path."""
    import torch
    import tracetransform_gb300 as tt
    from tracetransform_gb300.device import Engine

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    imgs, steps = make_batch()
    rows = [im.shape[0] for im in imgs]
    cols = [im.shape[1] for im in imgs]
    bufs = [np.ascontiguousarray(im.ravel(order="F")) for im in imgs]
    offsets = np.zeros(len(bufs), np.int64)
    offsets[1:] = np.cumsum([b.size for b in bufs])[:-1]
    flat_h = np.concatenate(bufs)
    flat = torch.from_numpy(flat_h).to(dev)
    eng = Engine(local_rank)
    pf = [(p, -1, -1) for p in BATCH_P]
    n_sino = len(imgs) * len(BATCH_T)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    circ = torch.empty(sum(len(BATCH_T) * len(BATCH_P) * (360 // s) for s in steps),
                       dtype=torch.float32, device=dev)
    sig = torch.empty_like(circ)

    def batched():
        return eng.transform_batch(flat, offsets, rows, cols, steps, BATCH_T, pf, circ, sig)

    def timed(fn, k, stage=None):
        ms = []
        for _ in range(k):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
            if stage is not None:
                stage.append(eng.batch_stage_ms())
        return ms

    for _ in range(args.warmup):     # the first call builds, autotunes and captures
        batched()
    torch.cuda.synchronize()
    barrier(world)
    tile = eng.batch_tile()
    clocks = ClockSampler(local_rank)
    clocks.start()
    stages = []
    ms = statistics.mean(timed(batched, args.steps, stages))
    clk = clocks.stop()
    sino_ms = statistics.mean(s[0] for s in stages)
    circ_ms = statistics.mean(s[1] for s in stages)
    z_ms = statistics.mean(s[2] for s in stages)
    gpu_sino = eng.batch_sinograms(flat)
    gpu_circ, gpu_sig = circ.cpu().numpy(), sig.cpu().numpy()

    # plain per-image device path: three launches per image, no graph
    views = [flat[int(o): int(o) + r * c].view(c, r) for o, r, c in zip(offsets, rows, cols)]
    angle_lists = {s: tt.angles_from_step(s) for s in set(steps)}

    def plain():
        for v, r, c, s in zip(views, rows, cols, steps):
            sn = eng.sinograms(v, r, c, angle_lists[s], BATCH_T)
            eng.zscore(eng.circus(sn, pf))

    plain()
    torch.cuda.synchronize()
    plain_ms = statistics.mean(timed(plain, max(1, min(3, args.steps))))

    # end to end: host buffers through the C ABI, batched and per image
    h_flat = torch.from_numpy(flat_h).pin_memory().numpy()
    tt.api.transform_batch_flat(h_flat, offsets, rows, cols, steps, BATCH_T, BATCH_P,
                                plan=eng.plan)
    e2e = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        tt.api.transform_batch_flat(h_flat, offsets, rows, cols, steps, BATCH_T, BATCH_P,
                                    plan=eng.plan)
        e2e.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(statistics.mean(e2e) * 1e3, world) / 1e3
    t0 = time.perf_counter()
    for im, s in zip(imgs, steps):
        tt.Transformer(im, "plain", s, False, plan=eng.plan).getTransform(
            [str(t) for t in BATCH_T], [str(p) for p in BATCH_P], write_data=False)
    e2e_plain_s = time.perf_counter() - t0
    ms = max_over_ranks(ms, world)
    extras = {} if args.no_extras else side_measurements(eng, dev, args)
    if rank != 0:
        return
    peak, peak_kind = measured_peak()
    alg = 0.0
    out_floats = 0
    for r, c, s in zip(rows, cols, steps):
        n = tt.pad_geometry(r, c)[0]
        a = 360 // s
        alg += 4.0 * a * r * c + 4.0 * len(BATCH_T) * n * a
        out_floats += len(BATCH_T) * len(BATCH_P) * a
    achieved = alg / (sino_ms / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": job_rate(n_sino, world, ms), "unit": "sinograms/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded blob+noise, the reference ships no images)",
        "config": batch_config(imgs, world),
        "e2e": {"value": job_rate(n_sino, world, e2e_s * 1e3), "unit": "sinograms/s",
                "h2d_bytes_per_step": int(flat_h.nbytes),
                "d2h_bytes_per_step": int(2 * 4 * out_floats),
                "call": "tt_transform_batch (host buffers)"},
        "plain_per_image": {"value": n_sino / (plain_ms / 1e3), "unit": "sinograms/s",
                            "ms_per_step": plain_ms, "e2e_value": n_sino / e2e_plain_s,
                            "note": "the same 512 images, one tt_sinograms_device + "
                                    "tt_circus_device + tt_zscore_device per image; e2e: one "
                                    "tt_transform (host buffers) per image"},
        "batched_over_plain": plain_ms / ms,
        "batched_over_plain_e2e": e2e_plain_s / e2e_s,
        "images_per_s": job_rate(len(imgs), world, ms),
        "gpu_launches": 3 * args.steps,
        "stage_ms": {"sinograms": sino_ms, "circus": circ_ms, "zscore": z_ms},
        "tile": {"lines_per_cta": tile[0], "ctas_per_sm": tile[1], "lines_per_warp": tile[2],
                 "chosen_by": "the engine's autotuner (timed on this batch)"},
        "roofline": {"bound": "hbm", "kernel": "sino_batch_kernel", "achieved": achieved,
                     "peak": peak, "peak_source": peak_kind, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "traffic_source": "not measured live: DRAM bytes of this kernel are in "
                                       "the committed ncu summary of the batch workload",
                     "algorithmic_bytes_per_launch": alg, "kernel_ms": sino_ms},
        "clocks": clk,
    }
    line.update(extras)
    if not args.no_cpu_baseline:
        line.update(batch_cpu_leg(imgs, steps, rows, cols, gpu_sino, gpu_circ, gpu_sig,
                                  args.cpu_seconds))
    print(json.dumps(line), flush=True)


def batch_cpu_leg(imgs, steps, rows, cols, gpu_sino, gpu_circ, gpu_sig, seconds):
    """The oracle on the batch's images, 8 per step until `seconds`, and the
    parity of those images' engine results against its outputs."""
    nt, npf = len(BATCH_T), len(BATCH_P)
    split = _split_batch(rows, cols, steps, nt, npf)
    done, secs, sinos, results = [], 0.0, 0, []
    while secs < seconds and len(done) < len(imgs):
        st, idx = cpu_batch_steps(imgs, steps, 8, 1, start=len(done))
        secs += st[0][0]
        sinos += st[0][1]
        done.extend(idx)
        results.extend(st[0][3])
    gpu = {}
    for j in done:
        so, co, n, a = split[j]
        s = gpu_sino[so: so + nt * a * n].cpu().numpy().reshape(nt, a, n).transpose(0, 2, 1)
        gpu[j] = (s, gpu_circ[co: co + nt * npf * a].reshape(nt, npf, a),
                  gpu_sig[co: co + nt * npf * a].reshape(nt, npf, a))
    return {"cpu_baseline": {"value": sinos / secs, "unit": "sinograms/s",
                             "cores": os.cpu_count() or 1, "kind": "port",
                             "sample": f"images 0-{len(done) - 1} of the batch transformed "
                                       f"(T0-T5 x P1-P3, z-scores), 8 per step, {secs:.1f} s"},
            "parity": batch_parity(imgs, steps, done, results, gpu)}


def side_measurements(eng, dev, args):
    """The 4096^2 workload's fused sinogram kernel and backward pass, and the
    64-image gradient step, measured in the same run as the batch."""
    import torch
    import tracetransform_gb300 as tt
    from tracetransform_gb300.device import to_colmajor
    peak, peak_kind = measured_peak()
    img, angles, tfs, _ = make_image("single4096")
    rows, cols = img.shape
    n = tt.pad_geometry(rows, cols)[0]
    img_dev = to_colmajor(torch.from_numpy(np.ascontiguousarray(img)).to(dev))
    sino = torch.empty((len(tfs), len(angles), n), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    eng.sinograms(img_dev, rows, cols, angles, tfs, out=sino)
    kms = []
    for _ in range(3):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        eng.sinograms(img_dev, rows, cols, angles, tfs, out=sino)
        b.record(stream)
        torch.cuda.synchronize()
        kms.append(a.elapsed_time(b))
    k = statistics.mean(kms)
    alg = 4.0 * len(angles) * rows * cols + 4.0 * len(tfs) * n * len(angles)
    out = {"single4096": {
        "kernel": "sino_kernel (rotate + T0-T7), N 5793, 720 angles at 0.5 degrees",
        "kernel_ms": k, "sinograms_per_s": len(tfs) / (k / 1e3),
        "roofline": {"bound": "hbm", "achieved": alg / (k / 1e3) / 1e9, "peak": peak,
                     "peak_source": peak_kind, "unit": "GB/s",
                     "frac": alg / (k / 1e3) / 1e9 / peak,
                     "algorithmic_bytes_per_launch": alg},
        "backward": backward_timing(eng, img_dev, rows, cols, angles, 3)}}
    del sino
    out["grad64"] = grad_timing(dev, 3)
    return out


def backward_timing(eng, img_dev, rows, cols, angles, steps):
    """Forward (T0-T2 sinograms with their medians, P1/P3 circus) and backward
    (P-stage adjoint, then the rotation adjoint with the rotations
    recomputed) of the differentiable functionals on one image, timed with
    CUDA events on the launching stream."""
    import torch
    tf, pf = [0, 1, 2], [(1, -1, -1), (3, -1, -1)]
    stream = torch.cuda.current_stream()

    def fwd():
        sino, med = eng.sinograms(img_dev, rows, cols, angles, tf, medians=True)
        return sino, med, eng.circus(sino, pf)

    def bwd(sino, med, g):
        gs = eng.circus_backward(sino, pf, g)
        return eng.sinograms_backward(gs, med, rows, cols, angles, tf)

    sino, med, circ = fwd()
    grad = torch.ones_like(circ)
    bwd(sino, med, grad)
    torch.cuda.synchronize()
    f_ms, b_ms = [], []
    for _ in range(steps):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record(stream)
        sino, med, circ = fwd()
        e[1].record(stream)
        bwd(sino, med, grad)
        e[2].record(stream)
        torch.cuda.synchronize()
        f_ms.append(e[0].elapsed_time(e[1]))
        b_ms.append(e[1].elapsed_time(e[2]))
    f, b = statistics.mean(f_ms), statistics.mean(b_ms)
    return {"t_functionals": tf, "p_functionals": [1, 3], "forward_ms": f, "backward_ms": b,
            "backward_over_forward": b / f, "steps": steps,
            "note": "gradient of the sum of the circus functions with respect to the image; "
                    "rotations recomputed in the adjoint, nothing stored but the medians"}


def make_grad_batch(seed0):
    from tracetransform_gb300.synthetic import blob_image
    return np.stack([np.ascontiguousarray(blob_image(GRAD_SIDE, GRAD_SIDE, 8, (8, 40),
                                                     (40, 200), seed0 + i))
                     for i in range(GRAD_IMAGES)])


def grad_setup(dev):
    import torch
    import tracetransform_gb300 as tt
    from tracetransform_gb300 import autograd as tta
    angles = tt.angles_from_step(1)
    h_imgs = torch.from_numpy(make_grad_batch(10)).pin_memory()
    with torch.no_grad():
        target = tta.circus(torch.from_numpy(make_grad_batch(5000)).to(dev), angles, GRAD_T,
                            GRAD_P)
    # each (T, P) circus function in units of its targets' mean magnitude: the
    # raw P3 values of T2 sinograms (~1e23 here) would overflow a float32 MSE
    scale = target.abs().mean(dim=(0, 3), keepdim=True)
    target = target / scale
    stream = torch.cuda.current_stream(dev)

    def train_step(x_dev, evs=None):
        x = x_dev.requires_grad_(True)
        loss = torch.nn.functional.mse_loss(tta.circus(x, angles, GRAD_T, GRAD_P) / scale,
                                            target)
        if evs:
            evs[1].record(stream)
        loss.backward()
        return loss, x.grad

    return h_imgs, train_step, stream


def grad_timing(dev, steps, flush=None):
    """Forward + backward of the 64-image MSE step, CUDA events per phase."""
    import torch
    h_imgs, train_step, stream = grad_setup(dev)
    imgs = h_imgs.to(dev)
    for _ in range(2):
        train_step(imgs.clone())
    torch.cuda.synchronize()
    fwd, bwd = [], []
    for _ in range(steps):
        x_dev = imgs.clone()
        if flush is not None:
            flush.zero_()
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        evs[0].record(stream)
        train_step(x_dev, evs)
        evs[2].record(stream)
        torch.cuda.synchronize()
        fwd.append(evs[0].elapsed_time(evs[1]))
        bwd.append(evs[1].elapsed_time(evs[2]))
    f, b = statistics.mean(fwd), statistics.mean(bwd)
    return {"images": GRAD_IMAGES, "image": f"{GRAD_SIDE}x{GRAD_SIDE}", "angles": 360,
            "t_functionals": GRAD_T, "p_functionals": GRAD_P, "forward_ms": f,
            "backward_ms": b, "backward_over_forward": b / f, "steps": steps}


def run_single(args, world, rank, local_rank):
    """One image per step: the fused sinogram kernel, P1-P3, z-scores and,
    for the 1024^2 and 4096^2 workloads, the orthonormal Hermite circus."""
    import torch
    import tracetransform_gb300 as tt
    from tracetransform_gb300.device import Engine, to_colmajor

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    img, angles, tfs, pfs = make_image(args.workload)
    rows, cols = img.shape
    n = tt.pad_geometry(rows, cols)[0]
    A = len(angles)
    eng = Engine(local_rank)
    img_dev = to_colmajor(torch.from_numpy(np.ascontiguousarray(img)).to(dev))
    sino = torch.empty((len(tfs), A, n), dtype=torch.float32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    pf = [(p, 0, -1) for p in pfs]
    herm = WORKLOADS[args.workload][8]
    herm_out = torch.empty((len(tfs), len(herm), A), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step(ev_sino=None):
        if ev_sino:
            ev_sino[0].record(stream)
        eng.sinograms(img_dev, rows, cols, angles, tfs, out=sino)
        if ev_sino:
            ev_sino[1].record(stream)
        sig = eng.zscore(eng.circus(sino, pf))
        if herm:  # the orthonormal (Hermite) circus beside P1-P3
            hc, _ = eng.circus_orthonormal(sino, herm, out=herm_out)
            return sig, eng.zscore(hc)
        return sig

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(world)
    clocks = ClockSampler(local_rank)
    clocks.start()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ks = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    torch.cuda.synchronize()
    barrier(world)
    for i in range(args.steps):
        flush.zero_()
        starts[i].record(stream)
        step(ks[i])
        ends[i].record(stream)
    torch.cuda.synchronize()
    barrier(world)
    ms = statistics.mean(s.elapsed_time(e) for s, e in zip(starts, ends))
    kern_ms = statistics.mean(a.elapsed_time(b) for a, b in ks)
    ms = max_over_ranks(ms, world)
    # sinograms, circus, z-score; with the Hermite circus: weighted-median
    # offsets, alignment, QR (qr_init, one launch per column step, R^T), the
    # sweeps (one launch per block round), assembly (6), one circus launch
    # per sinogram and a z-score
    launches = 3
    if herm:
        nb = (A + 15) // 16  # 16-column blocks, nbp - 1 block rounds per sweep
        nbp = nb + (nb & 1)
        launches += 2 + (A + 2) + eng.last_sweeps * (nbp - 1) + 6 + len(tfs) + 1

    # end to end: one C ABI call with host buffers (pinned)
    h_img = torch.from_numpy(np.ascontiguousarray(img.ravel(order="F"))).pin_memory()
    n_out = len(tfs) * len(pfs) * A
    n_herm = len(tfs) * len(herm) * A
    h_out = torch.empty(2 * (n_out + n_herm), dtype=torch.float32).pin_memory()
    e2e_step = e2e_single_call(eng, h_img, rows, cols, angles, tfs, pfs, herm, h_out)
    for _ in range(max(1, args.warmup)):
        e2e_step()
    barrier(world)
    e2e_times = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_times.append(time.perf_counter() - t0)
    clk = clocks.stop()
    e2e_s = max_over_ranks(statistics.mean(e2e_times) * 1e3, world) / 1e3
    if rank != 0:
        return
    peak, peak_kind = measured_peak()
    alg_bytes = 4.0 * A * rows * cols + 4.0 * len(tfs) * n * A
    achieved = alg_bytes / (kern_ms / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": job_rate(len(tfs), world, ms), "unit": "sinograms/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded blob+noise, the reference ships no images)",
        "config": config_dict(args.workload, n, angles, tfs, pfs, world),
        "e2e": {"value": job_rate(len(tfs), world, e2e_s * 1e3), "unit": "sinograms/s",
                "h2d_bytes_per_step": int(rows * cols * 4),
                "d2h_bytes_per_step": int(2 * (n_out + n_herm) * 4),
                "call": "tt_transform_extended" if herm else "tt_transform"},
        "gpu_launches": launches * args.steps,
        "roofline": {"bound": "hbm", "kernel": "sino_kernel", "achieved": achieved,
                     "peak": peak, "peak_source": peak_kind, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "traffic_source": "not measured live: DRAM bytes of this kernel are in "
                                       "the committed ncu summary of this workload",
                     "algorithmic_bytes_per_launch": alg_bytes,
                     "padded_sweep_bytes_per_launch": 4.0 * A * n * n,
                     "kernel_ms": kern_ms},
        "clocks": clk,
    }
    if herm:
        line["hermite_sweeps"] = eng.last_sweeps
    line["images_per_s"] = line["value"] / len(tfs)
    if args.workload == "single4096":
        line["backward"] = backward_timing(eng, img_dev, rows, cols, angles, 3)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = single_cpu_leg(args.workload, img, angles, tfs, pfs, herm,
                                              args.cpu_seconds)
    print(json.dumps(line), flush=True)


def single_cpu_leg(name, img, angles, tfs, pfs, herm, seconds):
    secs, sinos, steps = 0.0, 0.0, 0
    while secs < seconds:
        if name == "single4096":
            st = cpu_angle_sample_steps(img, angles, tfs, pfs, 1, 12)
            sinos += st[0][1]
            desc = "12 angles of all T-functionals with P1-P3 per step (no orthonormal circus)"
        else:
            st = [x[:1] for x in cpu_single_steps(img, angles, [tfs[steps % len(tfs)]], pfs,
                                                   herm, 1)]
            sinos += 1
            desc = ("one sinogram per step (T-functionals in turn), all angles, P1-P3" +
                    (", nearest orthonormal sinogram and Hermite circus" if herm else ""))
        secs += st[0][0]
        steps += 1
    return {"value": sinos / secs, "unit": "sinograms/s", "cores": os.cpu_count() or 1,
            "kind": "port", "sample": f"{steps} steps, {secs:.1f} s: {desc}"}


def e2e_single_call(eng, h_img, rows, cols, angles, tfs, pfs, herm, h_out):
    """One drop-in C ABI call with host buffers: tt_transform (integer step,
    P1-P3) or tt_transform_extended (any angle list, P1-P3 beside the
    orthonormal Hermite circus of the same sinograms)."""
    import tracetransform_gb300 as tt
    from tracetransform_gb300 import _native
    lib = _native.lib()
    A = len(angles)
    ids = np.asarray(tfs, np.int32)
    pfa = (_native.PFunctionalC * len(pfs))()
    for i, p in enumerate(pfs):
        pfa[i].kind, pfa[i].order, pfa[i].center = p, -1, -1
    fp = lambda t, off=0: ctypes.cast(t.data_ptr() + 4 * off, ctypes.POINTER(ctypes.c_float))
    n_out = len(tfs) * len(pfs) * A
    n_herm = len(tfs) * len(herm) * A
    step = float(angles[1] - angles[0]) if A > 1 else 360.0
    if not herm and step == int(step):
        return lambda: _native.check(lib.tt_transform(
            eng.plan.handle, fp(h_img), rows, cols, int(step), _native.iptr(ids), len(ids), pfa,
            len(pfs), fp(h_out), fp(h_out, n_out)))
    ang = np.ascontiguousarray(angles, np.float32)
    orders = np.asarray(herm, np.int32)
    centers = np.zeros(len(tfs), np.int32)
    return lambda: _native.check(lib.tt_transform_extended(
        eng.plan.handle, fp(h_img), rows, cols, _native.fptr(ang), A, _native.iptr(ids),
        len(ids), pfa, len(pfs), _native.iptr(orders), len(orders), fp(h_out),
        fp(h_out, n_out), fp(h_out, 2 * n_out), fp(h_out, 2 * n_out + n_herm),
        _native.iptr(centers)))


def run_grad(args, world, rank, local_rank):
    """64 images of 256 x 256, T0-T2 x P1/P3 over 360 angles: MSE loss
    against a second seed's circus functions and the gradient to the images
    through tracetransform_gb300.autograd (the hand-written adjoint kernels)."""
    import torch
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    h_imgs, train_step, stream = grad_setup(dev)
    imgs = h_imgs.to(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    for _ in range(args.warmup):
        train_step(imgs.clone())
    torch.cuda.synchronize()
    barrier(world)
    clocks = ClockSampler(local_rank)
    clocks.start()
    fwd, bwd, tot = [], [], []
    for _ in range(args.steps):
        x_dev = imgs.clone()
        flush.zero_()
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        evs[0].record(stream)
        train_step(x_dev, evs)
        evs[2].record(stream)
        torch.cuda.synchronize()
        fwd.append(evs[0].elapsed_time(evs[1]))
        bwd.append(evs[1].elapsed_time(evs[2]))
        tot.append(evs[0].elapsed_time(evs[2]))
    ms = max_over_ranks(statistics.mean(tot), world)
    h_grad = torch.empty_like(h_imgs).pin_memory()
    e2e = []
    for i in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        loss, g = train_step(h_imgs.to(dev, non_blocking=True))
        h_grad.copy_(g, non_blocking=True)
        lv = loss.item()
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e.append(time.perf_counter() - t0)
    clk = clocks.stop()
    e2e_s = max_over_ranks(statistics.mean(e2e), world)
    if rank != 0:
        return
    n_sino = GRAD_IMAGES * len(GRAD_T)
    line = {
        "metric": METRIC, "value": job_rate(n_sino, world, ms), "unit": "sinograms/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded blob+noise, the reference ships no images)",
        "config": {"workload": "grad64", "images": GRAD_IMAGES,
                   "image": f"{GRAD_SIDE}x{GRAD_SIDE}", "angles": 360,
                   "t_functionals": GRAD_T, "p_functionals": GRAD_P,
                   "step": "forward (sinograms + medians, circus) + MSE + backward",
                   "l2": "flushed between timed steps (256 MiB write)",
                   "parallelism": f"replicas{world}" if world > 1 else "single"},
        "forward_ms": statistics.mean(fwd), "backward_ms": statistics.mean(bwd),
        "backward_over_forward": statistics.mean(bwd) / statistics.mean(fwd),
        "images_per_s": job_rate(GRAD_IMAGES, world, ms),
        "e2e": {"value": job_rate(n_sino, world, e2e_s * 1e3), "unit": "sinograms/s",
                "h2d_bytes_per_step": int(h_imgs.numel() * 4),
                "d2h_bytes_per_step": int(h_grad.numel() * 4 + 4), "loss": lv},
        "gpu_launches": (GRAD_IMAGES + 4) * args.steps,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def run_kernel_only(args):
    import torch
    from tracetransform_gb300.device import Engine, to_colmajor
    img, angles, tfs, _ = make_image(args.workload)
    if args.tfuncs:
        tfs = [int(t) for t in args.tfuncs.split(",")]
    eng = Engine(0)
    dev = to_colmajor(torch.from_numpy(np.ascontiguousarray(img)).cuda())
    for _ in range(args.kernel_only):
        eng.sinograms(dev, img.shape[0], img.shape[1], angles, tfs)
    torch.cuda.synchronize()


def run_profile_steps(args):
    import torch
    from tracetransform_gb300.device import Engine, to_colmajor
    if args.workload == "batch512":
        imgs, steps = make_batch()
        if args.images:
            imgs, steps = imgs[:args.images], steps[:args.images]
        bufs = [np.ascontiguousarray(im.ravel(order="F")) for im in imgs]
        offsets = np.zeros(len(bufs), np.int64)
        offsets[1:] = np.cumsum([b.size for b in bufs])[:-1]
        flat = torch.from_numpy(np.concatenate(bufs)).cuda()
        eng = Engine(0)
        if args.tile:
            eng.batch_tile(pin=tuple(int(v) for v in args.tile.split(",")))
        for _ in range(args.profile_steps):
            eng.transform_batch(flat, offsets, [im.shape[0] for im in imgs],
                                [im.shape[1] for im in imgs], steps, BATCH_T,
                                [(p, -1, -1) for p in BATCH_P])
        torch.cuda.synchronize()
        return
    if args.workload == "grad64":
        dev = torch.device("cuda", 0)
        h_imgs, train_step, _ = grad_setup(dev)
        imgs = h_imgs.to(dev)
        for _ in range(args.profile_steps):
            train_step(imgs.clone())
        torch.cuda.synchronize()
        return
    img, angles, tfs, pfs = make_image(args.workload)
    herm = WORKLOADS[args.workload][8]
    eng = Engine(0)
    dev = to_colmajor(torch.from_numpy(np.ascontiguousarray(img)).cuda())
    for _ in range(args.profile_steps):
        sino = eng.sinograms(dev, img.shape[0], img.shape[1], angles, tfs)
        eng.zscore(eng.circus(sino, [(p, 0, -1) for p in pfs]))
        if herm:
            eng.zscore(eng.circus_orthonormal(sino, herm)[0])
    torch.cuda.synchronize()


def main():
    args = parse_args()
    if args.kernel_only:
        run_kernel_only(args)
        return
    if args.profile_steps:
        run_profile_steps(args)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if world > 1 and rank != 0:
            return
        run_reference(args, world)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    if args.workload == "batch512":
        run_batch(args, world, rank, local_rank)
    elif args.workload == "grad64":
        run_grad(args, world, rank, local_rank)
    else:
        run_single(args, world, rank, local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
