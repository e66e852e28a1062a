#!/usr/bin/env python
"""Benchmark of the trace-transform sinogram + circus path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
    python bench.py --impl reference ...

A step is one pass of the hot path over one image: the fused rotate +
T-functional kernel (all sinograms), the P-functional kernel (all circus
functions) and the z-score kernel, plus -- for the 1024^2 and 4096^2
workloads -- the orthonormal Hermite circus (nearest orthonormal sinogram of
every sinogram, Hermite orders 1-5).  The metric is sinograms per second
(sinograms = images x T-functionals).  Prints one JSON line (rank 0).
Other workloads: batch512 (512 uneven images through the batched engine
against the plain per-image path) and grad64 (forward + backward of an MSE
loss over 64 images through tracetransform_gb300.autograd).

* value      device-resident throughput: the image already in HBM, CUDA events
             around each step, L2 flushed (256 MiB write) between steps
* e2e        the same metric through the C ABI drop-in tt_transform with host
             buffers (pinned): host->device image copy, compute, device->host
             circus + signatures inside the timed region
* roofline   the fused sinogram kernel: algorithmic bytes per launch
             (4 A H W image sweeps + 4 nT N A sinogram writes) / its
             event-timed duration, against the measured HBM copy bandwidth
* cpu_baseline  the CPU oracle (a C restatement of the reference's float path,
             OpenMP over angles as the reference's openmp/ port) on all host
             cores, timed on a subset of the angles and scaled to the image

--impl reference times that CPU implementation alone as the reference arm.
Multi-GPU (torchrun): every rank transforms its own image (weak scaling).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import re
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
DEFAULT_WORKLOAD = "single1024"
L2_FLUSH_BYTES = 256 << 20


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["engine", "reference"], default="engine")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["batch512", "grad64"],
                    default=DEFAULT_WORKLOAD)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--kernel-only", type=int, default=0, metavar="CALLS",
                    help="for profiler captures: run only the fused sinogram kernel CALLS "
                         "times on the workload and exit (prints no bench line)")
    ap.add_argument("--profile-steps", type=int, default=0, metavar="STEPS",
                    help="for profiler launch lists: run the workload's full device step "
                         "(sinograms, circus, z-scores, Hermite circus) STEPS times and exit")
    ap.add_argument("--tfuncs", default=None,
                    help="comma-separated T-functional ids overriding the workload's")
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="target CPU time of the baseline sample")
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


# ---------------------------------------------------------------------------
# CPU side (oracle): timed baseline / reference arm
# ---------------------------------------------------------------------------

def cpu_sample(img, angles, tfs, pfs, target_s, threads=0):
    """Time the oracle on a growing subset of angles (all angles, repeated,
    once the subset is complete) until it takes target_s; returns (seconds per
    full transform, sample description, threads)."""
    from oracle import oracle as O
    O.build()
    padded = O.pad(img)
    nthreads = threads or os.cpu_count() or 1
    k = min(len(angles), max(1, nthreads))
    reps = 1
    while True:
        sub = angles[:: max(1, len(angles) // k)][:k]
        t0 = time.perf_counter()
        for _ in range(reps):
            sino = O.sinograms(padded, sub, tfs, threads)
            for t in range(sino.shape[0]):
                O.circus(sino[t], [(p, 0, 0) for p in pfs], threads)
        dt = time.perf_counter() - t0
        if dt >= target_s:
            break
        grow = max(2.0, 1.2 * target_s / max(dt, 1e-3))
        if len(sub) >= len(angles):
            reps = int(reps * grow)
        else:
            k = min(len(angles), int(k * grow))
    per_image = dt / reps * len(angles) / len(sub)
    desc = (f"{reps} x {len(sub)} of {len(angles)} angles of the same image (all T and P "
            f"functionals), {dt:.1f} s, scaled by {len(angles) / len(sub) / reps:.3f}")
    return per_image, desc, nthreads


def cpu_hermite_seconds(img, angles, tfs, orders):
    """The oracle's nearest orthonormal sinogram (double Jacobi, one thread)
    and Hermite circus for the first T-functional's full sinogram, scaled by
    the number of T-functionals."""
    from oracle import oracle as O
    O.build()
    sino = O.sinograms(O.pad(img), angles, [tfs[0]])[0]
    t0 = time.perf_counter()
    nos, c = O.nos(sino)
    O.circus(nos, [(0, o, c) for o in orders])
    dt = time.perf_counter() - t0
    return dt * len(tfs), (f"orthonormal circus: nearest orthonormal sinogram + Hermite "
                           f"{orders} of one {sino.shape[0]}x{sino.shape[1]} sinogram, "
                           f"{dt:.1f} s, x{len(tfs)}")


def run_reference(args, world, rank):
    img, angles, tfs, pfs = make_image(args.workload)
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    n = O.pad_geometry(*img.shape)[0]
    target = max(1.0, args.cpu_seconds / max(1, args.steps))
    herm = WORKLOADS[args.workload][8]
    herm_s, herm_desc = cpu_hermite_seconds(img, angles, tfs, herm) if herm else (0.0, "")
    per = []
    desc = ""
    threads = os.cpu_count() or 1
    for i in range(args.warmup + args.steps):
        t, desc, threads = cpu_sample(img, angles, tfs, pfs, target)
        if i >= args.warmup:
            per.append(t + herm_s)
    if herm:
        desc += "; plus, timed once and added to every step, the " + herm_desc
    sec = statistics.median(per)
    value = len(tfs) / sec
    line = {"metric": METRIC, "value": value, "unit": "sinograms/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded blob+noise)", "impl": "reference",
            "config": config_dict(args.workload, n, angles, tfs, pfs, world),
            "cpu_baseline": {"value": value, "unit": "sinograms/s", "cores": threads, "kind": "port",
                             "sample": desc},
            "e2e": {"value": value, "unit": "sinograms/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------

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


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def committed_traffic(kernel, workload):
    """Per-launch DRAM bytes of a kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    try:
        txt = open(path).read()
    except OSError:
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", txt)
    return float(m.group(1)) if m else None


def run_engine(args, world, rank, local_rank):
    import torch
    import tracetransform_gb300 as tt
    from tracetransform_gb300 import _native
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
        circ = eng.circus(sino, pf)
        sig = eng.zscore(circ)
        if herm:  # the orthonormal (Hermite) circus beside P1-P3
            hc, _ = eng.circus_orthonormal(sino, herm, out=herm_out)
            return sig, circ, hc, eng.zscore(hc)
        return sig, circ

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
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    kern_ms = [a.elapsed_time(b) for a, b in ks]
    ms = sum(step_ms) / len(step_ms)
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
    launches *= args.steps

    # end to end through the C ABI drop-in, pinned host buffers
    lib = _native.lib()
    h_img = torch.from_numpy(np.ascontiguousarray(img.ravel(order="F"))).pin_memory()
    n_out = len(tfs) * len(pfs) * A
    h_circ = torch.empty(n_out, dtype=torch.float32).pin_memory()
    h_sig = torch.empty(n_out, dtype=torch.float32).pin_memory()
    ids = np.asarray(tfs, np.int32)
    pfa = (_native.PFunctionalC * len(pfs))()
    for i, p in enumerate(pfs):
        pfa[i].kind, pfa[i].order, pfa[i].center = p, -1, -1
    fp = lambda t: ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_float))
    step_deg = WORKLOADS[args.workload][5]

    h_herm = torch.empty(len(tfs) * len(herm) * A, dtype=torch.float32).pin_memory()
    h_hsig = torch.empty_like(h_herm).pin_memory()

    def e2e_step():
        if herm:  # device entry points (tt_transform keeps the reference's
            # rule that regular and orthonormal P-functionals do not mix)
            d = h_img.to(dev, non_blocking=True).view(cols, rows)
            eng.sinograms(d, rows, cols, angles, tfs, out=sino)
            c = eng.circus(sino, pf)
            z = eng.zscore(c)
            hc, _ = eng.circus_orthonormal(sino, herm, out=herm_out)
            hz = eng.zscore(hc)
            h_circ.copy_(c.view(-1), non_blocking=True)
            h_sig.copy_(z.view(-1), non_blocking=True)
            h_herm.copy_(hc.view(-1), non_blocking=True)
            h_hsig.copy_(hz.view(-1), non_blocking=True)
            torch.cuda.synchronize()
        elif float(step_deg) == int(step_deg):
            _native.check(lib.tt_transform(eng.plan.handle, fp(h_img), rows, cols, int(step_deg),
                                           _native.iptr(ids), len(ids), pfa, len(pfs), fp(h_circ),
                                           fp(h_sig)))
        else:  # fractional angle steps go through the device entry points
            d = h_img.to(dev, non_blocking=True).view(cols, rows)
            s = eng.sinograms(d, rows, cols, angles, tfs, out=sino)
            c = eng.circus(s, pf)
            z = eng.zscore(c)
            h_circ.copy_(c.view(-1), non_blocking=True)
            h_sig.copy_(z.view(-1), non_blocking=True)
            torch.cuda.synchronize()

    for _ in range(max(1, args.warmup)):
        e2e_step()
    torch.cuda.synchronize()
    barrier(world)
    e2e_times = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_times.append(time.perf_counter() - t0)
    clk = clocks.stop()
    e2e_s = max_over_ranks(sum(e2e_times) / len(e2e_times) * 1e3, world) / 1e3

    if rank != 0:
        return
    peak, peak_kind = measured_peak()
    alg_bytes = 4.0 * A * rows * cols + 4.0 * len(tfs) * n * A
    kern_s = (sum(kern_ms) / len(kern_ms)) / 1e3
    achieved = alg_bytes / kern_s / 1e9
    line = {
        "metric": METRIC, "value": job_rate(len(tfs), world, ms), "unit": "sinograms/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded blob+noise, the reference ships no images)",
        "config": config_dict(args.workload, n, angles, tfs, pfs, world),
        "e2e": {"value": job_rate(len(tfs), world, e2e_s * 1e3), "unit": "sinograms/s",
                "h2d_bytes_per_step": int(rows * cols * 4),
                "d2h_bytes_per_step": int(2 * (n_out + h_herm.numel()) * 4)},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": "sino_kernel", "achieved": achieved,
                     "peak": peak, "peak_source": peak_kind, "unit": "GB/s",
                     "frac": achieved / peak,
                     "traffic": committed_traffic("sino_kernel", args.workload),
                     "algorithmic_bytes_per_launch": alg_bytes,
                     "padded_sweep_bytes_per_launch": 4.0 * A * n * n,
                     "kernel_ms": kern_s * 1e3},
        "clocks": clk,
    }
    if herm:
        line["hermite_sweeps"] = eng.last_sweeps
    line["images_per_s"] = line["value"] / len(tfs)
    if args.workload in BACKWARD_TIMED:
        line["backward"] = backward_timing(eng, img_dev, rows, cols, angles,
                                           max(2, min(args.steps, 3)))
    if not args.no_cpu_baseline:
        per, desc, cores = cpu_sample(img, angles, tfs, pfs, args.cpu_seconds)
        per1, desc1, _ = cpu_sample(img, angles, tfs, pfs, args.cpu_seconds, threads=1)
        if herm:
            hs, hd = cpu_hermite_seconds(img, angles, tfs, herm)
            per += hs
            per1 += hs
            desc += "; plus the " + hd
            desc1 += "; plus the " + hd
        line["cpu_baseline"] = {"value": len(tfs) / per, "unit": "sinograms/s", "cores": cores,
                                "kind": "port", "sample": desc}
        line["cpu_baseline_1thread"] = {"value": len(tfs) / per1, "unit": "sinograms/s",
                                        "cores": 1, "kind": "port", "sample": desc1}
    print(json.dumps(line), flush=True)


BACKWARD_TIMED = {"single4096"}


def backward_timing(eng, img_dev, rows, cols, angles, steps):
    """Forward (T0-T2 sinograms with their medians, P1/P3 circus) and backward
    (P-stage adjoint, then the rotation adjoint with the rotations
    recomputed) of the differentiable functionals on the workload's image,
    timed with CUDA events on the launching stream."""
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


BATCH_T, BATCH_P = [0, 1, 2, 3, 4, 5], [1, 2, 3]


def make_batch():
    from tracetransform_gb300.synthetic import workload
    items = workload("batch512")
    return [im for im, _ in items], [int(s) for _, s in items]


def batch_config(imgs, steps, world):
    return {"workload": "batch512", "images": len(imgs),
            "sides": "rows, cols independently uniform in 64..512",
            "angles": "360 or 180 (step 1 or 2 degrees, p = 1/2)",
            "t_functionals": BATCH_T, "p_functionals": BATCH_P,
            "images_per_step_per_gpu": len(imgs),
            "l2": "inputs 170 MB > L2 and L2 flushed between timed steps",
            "parallelism": f"replicas{world}" if world > 1 else "single"}


def run_batch(args, world, rank, local_rank):
    """512 uneven images per step through the batched engine (one graph),
    against the same 512 images through the plain per-image path."""
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

    def batched():
        return eng.transform_batch(flat, offsets, rows, cols, steps, BATCH_T, pf)

    def timed(fn, k):
        ms = []
        for _ in range(k):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        return ms

    for _ in range(args.warmup):     # the first call builds, autotunes and captures
        batched()
    torch.cuda.synchronize()
    barrier(world)
    clocks = ClockSampler(local_rank)
    clocks.start()
    ms = statistics.mean(timed(batched, args.steps))

    # plain per-image device path: three launches per image, no graph
    views = [flat[int(o): int(o) + r * c].view(c, r) for o, r, c in zip(offsets, rows, cols)]
    angle_lists = {s: tt.angles_from_step(s) for s in set(steps)}

    def plain():
        for v, r, c, s in zip(views, rows, cols, steps):
            sino = eng.sinograms(v, r, c, angle_lists[s], BATCH_T)
            eng.zscore(eng.circus(sino, pf))

    plain()
    torch.cuda.synchronize()
    plain_ms = statistics.mean(timed(plain, max(1, min(3, args.steps))))

    # end to end: host buffers through the C ABI, batched and per image
    h_flat = torch.from_numpy(flat_h).pin_memory().numpy()
    tt.api.transform_batch_flat(h_flat, offsets, rows, cols, steps, BATCH_T, BATCH_P,
                                plan=eng.plan)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        tt.api.transform_batch_flat(h_flat, offsets, rows, cols, steps, BATCH_T, BATCH_P,
                                    plan=eng.plan)
    e2e_s = (time.perf_counter() - t0) / args.steps
    t0 = time.perf_counter()
    for im, s in zip(imgs, steps):
        tt.Transformer(im, "plain", s, False, plan=eng.plan).getTransform(
            [str(t) for t in BATCH_T], [str(p) for p in BATCH_P], write_data=False)
    e2e_plain_s = time.perf_counter() - t0
    clk = clocks.stop()
    ms = max_over_ranks(ms, world)
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
    achieved = alg / (ms / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": job_rate(n_sino, world, ms), "unit": "sinograms/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded blob+noise, the reference ships no images)",
        "config": batch_config(imgs, steps, world),
        "e2e": {"value": job_rate(n_sino, world, e2e_s * 1e3), "unit": "sinograms/s",
                "h2d_bytes_per_step": int(flat_h.nbytes),
                "d2h_bytes_per_step": int(2 * 4 * out_floats)},
        "plain_per_image": {"value": n_sino / (plain_ms / 1e3), "unit": "sinograms/s",
                            "ms_per_step": plain_ms,
                            "e2e_value": n_sino / e2e_plain_s,
                            "note": "the same 512 images, one tt_sinograms_device + "
                                    "tt_circus_device + tt_zscore_device per image; e2e: one "
                                    "tt_transform (host buffers) per image"},
        "batched_over_plain": plain_ms / ms,
        "images_per_s": job_rate(len(imgs), world, ms),
        "gpu_launches": 3 * args.steps,
        "roofline": {"bound": "hbm", "kernel": "batch graph (sino + circus + zscore)",
                     "achieved": achieved, "peak": peak, "peak_source": peak_kind,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                     "algorithmic_bytes_per_launch": alg, "kernel_ms": ms},
        "clocks": clk,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = batch_cpu_sample(imgs, steps, args.cpu_seconds)
    print(json.dumps(line), flush=True)


def batch_cpu_sample(imgs, steps, target_s):
    """The oracle on the first images of the batch until target_s, scaled to 512."""
    from oracle import oracle as O
    O.build()
    t0 = time.perf_counter()
    k = 0
    while k < len(imgs) and time.perf_counter() - t0 < target_s:
        O.transform(imgs[k], steps[k], BATCH_T, [(p, 0) for p in BATCH_P])
        k += 1
    dt = time.perf_counter() - t0
    per_batch = dt * len(imgs) / k
    return {"value": len(imgs) * len(BATCH_T) / per_batch, "unit": "sinograms/s",
            "cores": os.cpu_count() or 1, "kind": "port",
            "sample": f"{k} of {len(imgs)} images transformed, {dt:.1f} s, scaled by "
                      f"{len(imgs) / k:.1f}"}


def run_reference_batch(args, world):
    imgs, steps = make_batch()
    target = max(1.0, args.cpu_seconds / max(1, args.steps))
    samples = [batch_cpu_sample(imgs, steps, target) for _ in range(args.warmup + args.steps)]
    cb = samples[-1]
    value = statistics.median(s["value"] for s in samples[args.warmup:])
    cb["value"] = value
    line = {"metric": METRIC, "value": value, "unit": "sinograms/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * len(imgs) * len(BATCH_T) / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded blob+noise)", "impl": "reference",
            "config": batch_config(imgs, steps, world), "cpu_baseline": cb,
            "e2e": {"value": value, "unit": "sinograms/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


GRAD_T, GRAD_P, GRAD_IMAGES, GRAD_SIDE = [0, 1, 2], [1, 3], 64, 256


def make_grad_batch(seed0):
    from tracetransform_gb300.synthetic import blob_image
    return np.stack([np.ascontiguousarray(blob_image(GRAD_SIDE, GRAD_SIDE, 8, (8, 40),
                                                     (40, 200), seed0 + i))
                     for i in range(GRAD_IMAGES)])


def grad_config(world):
    return {"workload": "grad64", "images": GRAD_IMAGES, "image": f"{GRAD_SIDE}x{GRAD_SIDE}",
            "angles": 360, "t_functionals": GRAD_T, "p_functionals": GRAD_P,
            "loss": "MSE against the circus functions of a second seed's images, each (T, P) "
                    "circus function divided by its targets' mean magnitude",
            "step": "forward (sinograms + medians, circus) + loss + backward to the images",
            "images_per_step_per_gpu": GRAD_IMAGES,
            "l2": "flushed between timed steps (256 MiB write)",
            "parallelism": f"replicas{world}" if world > 1 else "single"}


def run_grad(args, world, rank, local_rank):
    """64 images of 256 x 256, T0-T2 x P1/P3 over 360 angles: MSE loss
    against a second seed's circus functions and the gradient to the images
    through tracetransform_gb300.autograd (the hand-written adjoint kernels)."""
    import torch
    import tracetransform_gb300 as tt
    from tracetransform_gb300 import autograd as tta

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    angles = tt.angles_from_step(1)
    h_imgs = torch.from_numpy(make_grad_batch(10)).pin_memory()
    imgs = h_imgs.to(dev)
    with torch.no_grad():
        target = tta.circus(torch.from_numpy(make_grad_batch(5000)).to(dev), angles, GRAD_T,
                            GRAD_P)
    # each (T, P) circus function in units of its targets' mean magnitude: the
    # raw P3 values of T2 sinograms (~1e23 here) would overflow a float32 MSE
    scale = target.abs().mean(dim=(0, 3), keepdim=True)
    target = target / scale
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    n = tt.pad_geometry(GRAD_SIDE, GRAD_SIDE)[0]
    A = len(angles)

    def train_step(x_dev, evs=None):
        x = x_dev.requires_grad_(True)
        loss = torch.nn.functional.mse_loss(tta.circus(x, angles, GRAD_T, GRAD_P) / scale,
                                            target)
        if evs:
            evs[1].record(stream)
        loss.backward()
        return loss, x.grad

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

    # the dominant backward kernels alone, over the whole batch: line
    # parameters + rotation adjoint (one tt_sinograms_backward_device call)
    eng = tta.engine_for(dev)
    grad_sino = torch.randn((GRAD_IMAGES, len(GRAD_T), A, n), dtype=torch.float32, device=dev)
    med = torch.empty(grad_sino.shape, dtype=torch.int32, device=dev)
    sino_tmp = torch.empty_like(grad_sino)
    cm = imgs.transpose(1, 2).contiguous()
    for b in range(GRAD_IMAGES):
        eng.sinograms(cm[b], GRAD_SIDE, GRAD_SIDE, angles, GRAD_T, medians=True,
                      out=sino_tmp[b], med_out=med[b])
    adj = []
    for _ in range(max(3, args.steps)):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        eng.sinograms_backward(grad_sino, med, GRAD_SIDE, GRAD_SIDE, angles, GRAD_T)
        b.record(stream)
        torch.cuda.synchronize()
        adj.append(a.elapsed_time(b))
    adj_ms = statistics.mean(adj)

    # end to end: pinned host images in, loss and image gradients out
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
    peak, peak_kind = measured_peak()
    # per image: sinogram gradients and medians read, line parameters written
    # and read once, image gradient written
    alg = GRAD_IMAGES * (4.0 * 2 * len(GRAD_T) * n * A + 16.0 * 2 * n * A
                         + 4.0 * GRAD_SIDE * GRAD_SIDE)
    achieved = alg / (adj_ms / 1e3) / 1e9
    # per image: one sinogram launch; per batch: circus, circus adjoint, line
    # parameters, rotation adjoint
    line = {
        "metric": METRIC, "value": job_rate(n_sino, world, ms), "unit": "sinograms/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded blob+noise, the reference ships no images)",
        "config": grad_config(world),
        "forward_ms": statistics.mean(fwd), "backward_ms": statistics.mean(bwd),
        "backward_over_forward": statistics.mean(bwd) / statistics.mean(fwd),
        "images_per_s": job_rate(GRAD_IMAGES, world, ms),
        "e2e": {"value": job_rate(n_sino, world, e2e_s * 1e3), "unit": "sinograms/s",
                "h2d_bytes_per_step": int(h_imgs.numel() * 4),
                "d2h_bytes_per_step": int(h_grad.numel() * 4 + 4), "loss": lv},
        "gpu_launches": (GRAD_IMAGES + 4) * args.steps,
        "roofline": {"bound": "hbm", "kernel": "line_params + adjoint_gather (64 images)",
                     "achieved": achieved, "peak": peak, "peak_source": peak_kind,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                     "algorithmic_bytes_per_launch": alg, "kernel_ms": adj_ms},
        "clocks": clk,
    }
    if not args.no_cpu_baseline:
        img = make_grad_batch(10)[0]
        per, desc, cores = cpu_sample(img, angles, GRAD_T, GRAD_P, args.cpu_seconds)
        line["cpu_baseline"] = {"value": len(GRAD_T) / per, "unit": "sinograms/s",
                                "cores": cores, "kind": "port",
                                "sample": desc + "; forward only (the reference has no "
                                                 "gradient)"}
    print(json.dumps(line), flush=True)


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
        bufs = [np.ascontiguousarray(im.ravel(order="F")) for im in imgs]
        offsets = np.zeros(len(bufs), np.int64)
        offsets[1:] = np.cumsum([b.size for b in bufs])[:-1]
        flat = torch.from_numpy(np.concatenate(bufs)).cuda()
        eng = Engine(0)
        for _ in range(args.profile_steps):
            eng.transform_batch(flat, offsets, [im.shape[0] for im in imgs],
                                [im.shape[1] for im in imgs], steps, BATCH_T,
                                [(p, -1, -1) for p in BATCH_P])
        torch.cuda.synchronize()
        return
    if args.workload == "grad64":
        import tracetransform_gb300 as tt
        from tracetransform_gb300 import autograd as tta
        angles = tt.angles_from_step(1)
        imgs = torch.from_numpy(make_grad_batch(10)).cuda()
        with torch.no_grad():
            target = tta.circus(torch.from_numpy(make_grad_batch(5000)).cuda(), angles, GRAD_T,
                                GRAD_P)
        scale = target.abs().mean(dim=(0, 3), keepdim=True)
        for _ in range(args.profile_steps):
            x = imgs.clone().requires_grad_(True)
            torch.nn.functional.mse_loss(tta.circus(x, angles, GRAD_T, GRAD_P) / scale,
                                         target / scale).backward()
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
        if args.workload == "batch512":
            run_reference_batch(args, world)
        elif args.workload == "grad64":
            print(json.dumps({"impl": "reference", "unavailable": "the reference computes no "
                              "gradients; grad64 has no reference arm"}), flush=True)
        else:
            run_reference(args, world, rank)
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
        run_engine(args, world, rank, local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
