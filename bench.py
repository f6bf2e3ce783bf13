#!/usr/bin/env python
"""NUFFT op+adj throughput of the GB300 backend on the 3D multi-coil workload.

Workload (one step): a SENSE forward NUFFT of a 128^3 complex64 image over 16
coils on a 4096 x 512 kooshball trajectory (2 097 152 samples, float32), then
the density-compensated SENSE adjoint back to one image; pipe density (10
iterations) is computed once before timing.  eps = 1e-6, upsampfac 2 (fine
grid 256^3, kernel width 7).  Synthetic seeded inputs stand in for scanner
data.  Metric: Msamples*coil/s of op+adj = samples x coils / step time.

``--impl reference`` times the CPU implementation of the same path (the C /
OpenMP restatement of the ES NUFFT that mri-nufft's finufft backend calls,
with scipy.fft) on the host cores, one coil per step.

Run with N GPUs through torchrun: every rank runs an independent replica of
the workload (the path has no exchange step), ``value`` is the whole-job
throughput (all ranks' units / max rank time).
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import __graft_entry__  # noqa: E402

METRIC = "NUFFT op+adj Msamples*coil/s (rel err <= 1e-4 vs FP64 NDFT)"
UNIT = "Msamples*coil/s"
WORKLOAD = "3D SENSE op+adj, 128^3 image, 16 coils, kooshball 4096x512 (2.1M samples), pipe density"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-density", action="store_true",
                   help="skip the pipe density (and its timing): a small case whose first "
                        "launches are the op / adj kernels, for profiler captures")
    p.add_argument("--spokes", type=int, default=4096)
    p.add_argument("--samples", type=int, default=512)
    p.add_argument("--coils", type=int, default=16)
    p.add_argument("--size", type=int, default=128)
    p.add_argument("--duration", type=float, default=60.0, help="c5: stream length in seconds")
    p.add_argument("--rate", type=float, default=50.0, help="c5: Poisson arrival rate (req/s)")
    p.add_argument("--saturated", type=int, default=300,
                   help="c5: requests of the saturated served-vs-plain comparison")
    p.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "c5", "gram", "stacked", "orc"],
                   help="c2: 3D 16-coil SENSE (default line); c1: 2D 256^2 single-coil radial; "
                        "c3: 32 uneven 2D instances, batched graph-captured launch vs per-call "
                        "loop; c4: differentiable forward+backward; c5: served CG stream; gram: Toeplitz "
                        "Gram operator vs op+adj; stacked: stack-of-stars; orc: off-resonance corrected")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    return rank, world, local


def slowest_rank_ms(ms, world, device):
    """The largest of every rank's time (all-reduce MAX on the default group)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist

    t = torch.tensor([ms], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t)


def replica_rate(units_per_rank, world, ms):
    """Whole-job throughput of ``world`` independent replicas, in millions of
    units per second: every rank's units over the slowest rank's step time."""
    return world * units_per_rank / (ms / 1e3) / 1e6


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,"
              "utilization.gpu")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, smax, util, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[0]))
                smax.append(float(r[1]))
            except (ValueError, IndexError):
                continue
            try:
                util.append(float(r[8]))
            except (ValueError, IndexError):
                pass
            for n, v in zip(names, r[4:8]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(smax) if smax else None,
            "reasons": sorted(reasons),
            "samples": len(sm),
            "gpu_util_pct": statistics.median(util) if util else None,
        }


def touched_cells(samples_pi, nf, w):
    """Number of fine-grid cells inside at least one sample's w^d footprint."""
    import torch

    d = samples_pi.shape[1]
    nf_t = torch.tensor(nf, device=samples_pi.device, dtype=torch.int64)
    mask = torch.zeros(int(np.prod(nf)), dtype=torch.bool, device=samples_pi.device)
    offs = torch.stack(torch.meshgrid(*[torch.arange(w, device=samples_pi.device)] * d,
                                      indexing="ij"), -1).reshape(-1, d)
    strides = [int(np.prod(nf[i + 1:])) for i in range(d)]
    for s0 in range(0, samples_pi.shape[0], 65536):
        k = samples_pi[s0:s0 + 65536].double()
        u = k * (nf_t.double() / (2 * np.pi))
        u = u - nf_t.double() * torch.floor(u / nf_t.double())
        i0 = torch.ceil(u - w / 2).long()
        cells = (i0[:, None, :] + offs[None]) % nf_t
        lin = sum(cells[..., i] * strides[i] for i in range(d))
        mask[lin.reshape(-1)] = True
    return int(mask.sum())


def run_reference(args):
    """CPU implementation of the same path on the host cores (rank 0 only)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    pkg = __graft_entry__.import_package()
    from mrinufft_gb300 import workloads
    from oracle import esnufft

    traj, shape, img, smaps = workloads.config2(args.spokes, args.samples, args.coils, args.size)
    ncores = os.cpu_count() or 1
    e = esnufft.EsNufft(traj.astype(np.float64) * 2 * np.pi, shape, dtype=np.float32, nthreads=ncores)
    M = traj.shape[0]
    nrm = np.sqrt(np.prod(shape) * 2 ** 3)
    dens = np.ones(M, np.float32)

    def step(c):
        y = e.type2(img * smaps[c]) / nrm
        return np.conj(smaps[c]) * e.type1(y * dens) / nrm

    for i in range(args.warmup):
        step(i % args.coils)
    t = time.perf_counter()
    for i in range(args.steps):
        step(i % args.coils)
    dt = (time.perf_counter() - t) / args.steps
    value = M * 1 / dt / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64",
        "data": "synthetic (seeded kooshball, ellipsoid phantom, Gaussian coil maps)",
        "config": {"workload": WORKLOAD, "step": "one coil of the 16 per step (bounded sample)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": ncores, "kind": "port",
                         "sample": f"op+adj of 1 coil of {args.coils} per step, {M} samples, "
                                   "C/OpenMP ES spreader + scipy.fft (finufft not installed)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def accuracy_vs_ndft(op, img, traj, shape, smaps=None, n_coils=1, rows=None, vox_per_axis=None,
                     seed=5):
    """Relative l2 error of the GPU op and adj against the FP64 NDFT of the
    oracle (the checker): op on ``rows`` seeded samples (all when None) of up
    to 4 seeded coils; adj of those coils' op output (other coils zero,
    compensated by the operator's own density) on a seeded product set of
    ``vox_per_axis`` indices per axis (all voxels when None).  Part of the
    CPU leg; a failure is reported in the line, not raised."""
    try:
        import torch
        from oracle import ndft

        shape = tuple(int(n) for n in shape)
        k = ndft.proper_trajectory_unit(traj)
        M = k.shape[0]
        nrm = ndft.norm_factor(shape)
        rng = np.random.default_rng(seed)
        rsel = np.sort(rng.choice(M, rows, replace=False)) if rows and rows < M else np.arange(M)
        sense = smaps is not None
        C = smaps.shape[0] if sense else n_coils
        coils = np.sort(rng.choice(C, min(C, 4), replace=False))
        x = torch.from_numpy(np.ascontiguousarray(img, dtype=np.complex64)).to(op.device)
        y = op._op_device(x.reshape((1, *shape) if sense else (1, 1, *shape)))
        yh = y[0].cpu().numpy()
        xs = np.asarray(img, dtype=np.complex128)
        e_op = []
        for c in coils:
            ref = ndft.ndft_type2(k[rsel], xs * (smaps[c] if sense else 1), shape) / nrm
            e_op.append(float(np.linalg.norm(yh[c, rsel] - ref) / np.linalg.norm(ref)))
        yk = torch.zeros_like(y)
        yk[0, coils] = y[0, coils]
        z = op._adj_device(yk)[0].cpu().numpy()
        idx = [np.sort(rng.choice(n, min(n, vox_per_axis or n), replace=False)) for n in shape]
        sub = np.ix_(*idx)
        d = op._density
        cin = yh[coils].astype(np.complex128) * (1.0 if d is None else d.cpu().numpy().astype(np.float64))
        t1 = ndft.ndft_type1_grid(k, cin, shape, idx) / nrm
        if sense:
            ref = sum(np.conj(smaps[c][sub]) * t1[q] for q, c in enumerate(coils))
            got = z[0][sub]
        else:
            ref, got = t1[0], z[coils[0]][sub]
        e_adj = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
        return {"op_rel_l2": max(e_op), "op_rel_l2_per_coil": e_op, "adj_rel_l2": e_adj,
                "coils": [int(c) for c in coils], "sample_rows": int(len(rsel)),
                "voxels": int(np.prod([len(i) for i in idx])), "reference": "FP64 NDFT (oracle)"}
    except Exception as exc:  # reported, never fatal to the bench line
        return {"error": f"{type(exc).__name__}: {exc}"}


def cpu_baseline(traj, shape, img, smaps, dens, n_coils):
    """Bounded sample of the CPU port: op+adj of 4 coils on all host cores."""
    from oracle import esnufft

    ncores = os.cpu_count() or 1
    e = esnufft.EsNufft(traj.astype(np.float64) * 2 * np.pi, shape, dtype=np.float32, nthreads=ncores)
    nrm = np.sqrt(np.prod(shape) * 2 ** len(shape))
    nc = min(4, n_coils)
    t = time.perf_counter()
    for c in range(nc):
        y = e.type2(img * smaps[c]) / nrm
        _ = np.conj(smaps[c]) * e.type1(y * dens) / nrm
    dt = time.perf_counter() - t
    return {"value": traj.shape[0] * nc / dt / 1e6, "unit": UNIT, "cores": ncores, "kind": "port",
            "sample": f"op+adj of {nc} of {n_coils} coils, {traj.shape[0]} samples "
                      f"({dt:.1f} s), C/OpenMP ES spreader + scipy.fft"}


def measure_pipe(pkg, samples_d, shape, device, iters=10, reps=5):
    """Warm timing of the pipe density estimate (10 iterations of
    w <- w / |interp(spread(w))| on the image-size grid) on a resident
    spread-only plan, CUDA events over ``reps`` calls after an untimed one,
    with the per-stage times of the spread and interp kernels; and the whole
    ``MRIGB300.pipe`` call (plan creation, sort, iterations, normalisation
    NUFFT pair) timed warm on the host."""
    import torch

    dev = samples_d.device
    M = samples_d.shape[0]
    pplan = pkg.NufftPlan(shape, eps=1e-6, upsampfac=2.0, ntrans=1, spread_only=True, device=device)
    pplan.setpts(samples_d)
    nrm2 = float(np.prod(shape) * 2 ** len(shape))
    w = torch.ones(M, dtype=torch.complex64, device=dev)
    pplan.pipe(w, iters, 1.0 / nrm2)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    pplan.profile(True)
    e0.record()
    for _ in range(reps):
        w.fill_(1.0)
        pplan.pipe(w, iters, 1.0 / nrm2)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    st = {s_: pplan.profile_read(s_) for s_ in ("spread", "interp", "zero")}
    pplan.profile(False)
    info = pplan.info()
    G_t = touched_cells(samples_d, info["nf"], info["width"])
    spread_ms = st["spread"][0] / max(1, st["spread"][1])
    bytes_spread = 4 * len(shape) * M + 8 * M + 8 * G_t
    t0 = time.perf_counter()
    pkg.MRIGB300.pipe(samples_d, shape, max_iter=iters, device=device)
    torch.cuda.synchronize()
    whole_ms = (time.perf_counter() - t0) * 1e3
    return {"iterations": iters, "ms_per_call": ms, "ms_per_iteration": ms / iters,
            "stage_ms_per_iteration": {k_: v[0] / (reps * iters) for k_, v in st.items()},
            "grid": list(info["nf"]), "touched_cells": G_t,
            "spread_algorithmic_bytes": bytes_spread,
            "spread_achieved_gbs": bytes_spread / (spread_ms / 1e3) / 1e9,
            "whole_call_warm_ms": whole_ms}


def run_gb300(args):
    import torch
    import torch.distributed as dist

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)
    __graft_entry__.build()
    pkg = __graft_entry__.import_package()
    from mrinufft_gb300 import workloads

    traj, shape, img, smaps = workloads.config2(args.spokes, args.samples, args.coils, args.size)
    M, C = traj.shape[0], args.coils

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dens = None
    if not args.no_density:
        dens = pkg.MRIGB300.pipe(torch.from_numpy(traj).to(dev), shape, max_iter=10, device=local)
    torch.cuda.synchronize()
    pipe_cold_ms = (time.perf_counter() - t0) * 1e3

    op = pkg.MRIGB300(traj, shape, n_coils=C, smaps=smaps,
                      density=False if dens is None else dens, squeeze_dims=False, device=local)
    plan = op.plan
    img_d = torch.from_numpy(img).to(dev).reshape(1, *shape)
    pipe = None if args.no_density else measure_pipe(pkg, op._samples_d, shape, local)

    def step():
        y = op._op_device(img_d)
        return op._adj_device(y)

    for _ in range(max(args.warmup, 0)):
        step()
    torch.cuda.synchronize()
    info = plan.info()
    G_t = touched_cells(op._samples_d, info["nf"], info["width"])

    # ---- kernel-only timed region (inputs resident in HBM, > L2) ----
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    plan.profile(True)
    stream = torch.cuda.current_stream(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1) / args.steps
    stages = {s: plan.profile_read(s) for s in ("pad", "fft", "interp", "spread", "crop", "zero")}
    _, launches = plan.profile_read(None)
    plan.profile(False)
    ms = slowest_rank_ms(ms, world, dev)
    value = replica_rate(M * C, world, ms)

    # ---- end to end through the public API with pinned host buffers ----
    img_h = torch.from_numpy(img).reshape(1, *shape).pin_memory()
    out_h = torch.empty((1, 1, *shape), dtype=torch.complex64).pin_memory()
    img_dd = torch.empty_like(img_d)

    def step_e2e():
        img_dd.copy_(img_h, non_blocking=True)
        x = op.adj_op(op.op(img_dd))
        out_h.copy_(x, non_blocking=True)

    for _ in range(max(args.warmup, 1)):
        step_e2e()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    e0.record(stream)
    for _ in range(args.steps):
        step_e2e()
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    e2e_ms = slowest_rank_ms(e2e_ms, world, dev)
    e2e_value = replica_rate(M * C, world, e2e_ms)

    # ---- end to end with numpy host arrays (mri-nufft's CPU-array calling
    # convention: pageable numpy in, numpy out, every copy inside the call) ----
    img_np = np.ascontiguousarray(img.reshape(1, *shape))

    def step_np():
        return op.adj_op(op.op(img_np))

    for _ in range(max(args.warmup, 1)):
        step_np()
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    nsteps_np = max(3, args.steps // 2)
    for _ in range(nsteps_np):
        out_np = step_np()
    np_ms = (time.perf_counter() - t0) * 1e3 / nsteps_np
    np_ms = slowest_rank_ms(np_ms, world, dev)
    e2e_np = {"value": replica_rate(M * C, world, np_ms), "unit": UNIT, "ms_per_step": np_ms,
              "steps": nsteps_np,
              "h2d_bytes_per_step": img_np.nbytes + M * C * 8,
              "d2h_bytes_per_step": M * C * 8 + int(np.asarray(out_np).nbytes),
              "call": "op.adj_op(op.op(numpy image)) -> numpy image; host-timed; numpy "
                      "results in page-locked memory, op's k-space copied out per coil group"}

    # ---- roofline of the dominant kernel ----
    peaks_path = ROOT / "MEASURED_PEAKS.json"
    if peaks_path.exists():
        peak = float(json.loads(peaks_path.read_text())["hbm_gbs"])
        peak_src = "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    T = op._ntrans
    bytes_per_launch = 4 * 3 * M + 8 * T * M + 8 * T * G_t
    kern = {}
    for s in ("interp", "spread"):
        tms, n = stages[s]
        if n:
            per = tms / n
            kern[s] = {"ms_per_launch": per, "launches": n,
                       "achieved_gbs": bytes_per_launch / (per / 1e3) / 1e9}
    dom = max(kern, key=lambda s: stages[s][0])
    traffic = None
    tf = ROOT / "profiles" / "traffic_c2.json"
    if tf.exists():
        traffic = json.loads(tf.read_text()).get(dom)
    roof = {"bound": "hbm", "kernel": dom, "achieved": kern[dom]["achieved_gbs"], "peak": peak,
            "unit": "GB/s", "frac": kern[dom]["achieved_gbs"] / peak, "traffic": traffic,
            "peak_source": peak_src,
            "algorithmic_bytes_per_launch": bytes_per_launch,
            "other": {k: v for k, v in kern.items() if k != dom}}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64",
        "data": "synthetic (seeded kooshball, ellipsoid phantom, Gaussian coil maps)",
        "config": {"workload": WORKLOAD, "samples": M, "coils": C, "image": list(shape),
                   "fine_grid": list(info["nf"]), "kernel_width": info["width"], "eps": 1e-6,
                   "touched_fine_cells": G_t, "coils_per_pass": T,
                   "l2": "inputs > L2 (fine grids 2.1 GB, k-space 268 MB)",
                   "parallelism": f"replicas x{world}"},
        "stage_ms_per_step": {s: v[0] / args.steps for s, v in stages.items()},
        "gpu_launches": launches,
        "clocks": clocks,
        "roofline": roof,
        # the headline end-to-end number: numpy host arrays through the
        # plugin's op / adj_op (the reference's calling convention), every
        # host <-> device copy inside the call
        "e2e": e2e_np,
        "e2e_pinned": {"value": e2e_value, "unit": UNIT, "ms_per_step": e2e_ms,
                       "h2d_bytes_per_step": img_h.numel() * 8,
                       "d2h_bytes_per_step": out_h.numel() * 8,
                       "call": "op.adj_op(op.op(x)) on a device copy of a pinned host image, "
                               "result copied back to pinned host memory; CUDA events"},
        "pipe": None if pipe is None else dict(pipe, cold_ms=pipe_cold_ms, peak_gbs=peak,
                                               roofline_frac=pipe["spread_achieved_gbs"] / peak),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(traj, shape, img, smaps,
                                            np.ones(M, np.float32) if dens is None
                                            else dens.cpu().numpy(), C)
        line["accuracy"] = accuracy_vs_ndft(op, img, traj, shape, smaps=smaps, rows=4096,
                                            vox_per_axis=16)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_c3(args):
    """32 uneven 2D SENSE instances: batched (persistent, graph-captured) vs
    the plain per-call backend, op + adj of every instance per step."""
    import torch

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    __graft_entry__.build()
    pkg = __graft_entry__.import_package()
    from mrinufft_gb300 import workloads
    from mrinufft_gb300.batched import BatchedNufft

    insts = workloads.config3(32, seed=0)
    units = sum(i["samples"].shape[0] * i["smaps"].shape[0] for i in insts)
    t0 = time.perf_counter()
    bat = BatchedNufft(insts)
    tune_s = time.perf_counter() - t0
    bat.set_images([i["image"] for i in insts])
    bat.capture()
    pers = BatchedNufft(insts, mode="persistent")
    pers.set_images([i["image"] for i in insts])
    pers.capture()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    ms_graph = timed(bat.replay)
    ms_eager = timed(bat.step)
    ms_pers = timed(pers.replay)
    ops = [pkg.MRIGB300(i["samples"], i["shape"], n_coils=i["smaps"].shape[0], smaps=i["smaps"],
                        squeeze_dims=False) for i in insts]
    imgs = [torch.from_numpy(i["image"]).to(dev).reshape(1, *i["shape"]) for i in insts]

    def plain():
        for op, x in zip(ops, imgs):
            op._adj_device(op._op_device(x))

    ms_plain = timed(plain)
    line = {
        "metric": METRIC, "value": units / (ms_graph / 1e3) / 1e6, "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_graph,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64",
        "data": "synthetic (seeded spirals / radials, ellipse phantoms, Gaussian coil maps)",
        "config": {"workload": "32 uneven 2D SENSE instances (grids 128-384, coils 1-32), "
                               "op+adj per step", "sample_coils_per_step": units,
                   "autotune_s": tune_s},
        "batched_graph_ms": ms_graph, "batched_eager_ms": ms_eager,
        "persistent_worktable_graph_ms": ms_pers, "plain_per_call_ms": ms_plain,
        "batched_mode": f"{len(bat.streams)} streams, one CUDA graph",
        "speedup_vs_plain": ms_plain / ms_graph,
    }
    print(json.dumps(line), flush=True)


def _timed_steps(fn, steps, warmup, flush):
    """Per-step CUDA-event times of fn() with an L2 flush (a write larger
    than L2) between steps, outside the timed spans; returns ms per step."""
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(steps)]
    for a, b in evs:
        flush.zero_()
        a.record()
        fn()
        b.record()
    torch.cuda.synchronize()
    return float(np.mean([a.elapsed_time(b) for a, b in evs]))


def run_c1(args):
    """2D 256^2 single coil, radial 100 x 500 (50 000 samples): op + adj."""
    import torch

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    __graft_entry__.build()
    pkg = __graft_entry__.import_package()
    from mrinufft_gb300 import workloads

    traj, shape, img = workloads.config1()
    M = traj.shape[0]
    op = pkg.MRIGB300(traj, shape, squeeze_dims=False)
    x = torch.from_numpy(img).to(dev).reshape(1, 1, *shape)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    steps = max(args.steps, 100)
    ms = _timed_steps(lambda: op._adj_device(op._op_device(x)), steps, max(args.warmup, 3), flush)
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import esnufft

        ncores = os.cpu_count() or 1
        e = esnufft.EsNufft(traj.astype(np.float64) * 2 * np.pi, shape, dtype=np.float32,
                            nthreads=ncores)
        nrm = np.sqrt(np.prod(shape) * 4)
        t = time.perf_counter()
        reps = 5
        for _ in range(reps):
            _ = e.type1(e.type2(img) / nrm) / nrm
        dt = (time.perf_counter() - t) / reps
        cpu = {"value": M / dt / 1e6, "unit": UNIT, "cores": ncores, "kind": "port",
               "sample": f"{reps} op+adj steps, C/OpenMP ES spreader + scipy.fft"}
        # the reference's own CPU accuracy oracle for this case: MRInumpy's
        # FP64 NDFT (nudft_numpy.py:58-81), as restated by the oracle
        from oracle import ndft

        ku = ndft.proper_trajectory_unit(traj)
        t = time.perf_counter()
        yy = ndft.ndft_type2(ku, img, shape)
        _ = ndft.ndft_type1(ku, yy, shape)
        cpu["ndft_fp64"] = {"s_per_op_adj": time.perf_counter() - t,
                            "value": M / (time.perf_counter() - t) / 1e6, "unit": UNIT,
                            "sample": "one exact FP64 op+adj (factorised NDFT of the oracle, "
                                      "restating MRInumpy's implicit type 1 / type 2)"}
    acc = accuracy_vs_ndft(op, img, traj, shape) if not args.no_cpu_baseline else None
    line = {
        "metric": METRIC, "value": M / (ms / 1e3) / 1e6, "unit": UNIT, "n_gpus": 1,
        "steps": steps, "warmup": max(args.warmup, 3), "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64",
        "data": "synthetic (radial 100 x 500, ellipse phantom)",
        "config": {"workload": "2D 256^2 single coil, radial 100x500 (50 000 samples), op+adj",
                   "l2": "flushed between steps (256 MB write)"},
        "cpu_baseline": cpu,
    }
    if acc is not None:
        line["accuracy"] = acc
    print(json.dumps(line), flush=True)


def run_c4(args):
    """Differentiable form: 256^2, 8 coils, spiral 64 x 2048 (131 072 samples);
    loss ||A(x) - y||^2 with gradients for the image and the trajectory."""
    import torch

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    __graft_entry__.build()
    pkg = __graft_entry__.import_package()
    from mrinufft_gb300 import workloads

    shape, C = (256, 256), 8
    traj = workloads.spiral_2d(64, 2048, power=2).reshape(-1, 2).astype(np.float32)
    M = traj.shape[0]
    smaps = workloads.coil_maps(shape, C, seed=4)
    img = workloads.phantom(shape, seed=4)
    nufft = pkg.MRIGB300(traj, shape, n_coils=C, smaps=smaps, squeeze_dims=False)
    rng = np.random.default_rng(4)
    pert = traj + 1e-3 * rng.standard_normal(traj.shape).astype(np.float32)
    y = pkg.MRIGB300(pert, shape, n_coils=C, smaps=smaps, squeeze_dims=False).op(img)
    yt = torch.from_numpy(np.asarray(y)).to(dev).reshape(1, C, M)
    ad = nufft.make_autograd(wrt_data=True, wrt_traj=True)
    x0 = torch.from_numpy(img).to(dev).reshape(1, 1, *shape)

    def step():
        x = x0.clone().requires_grad_(True)
        if ad.samples.grad is not None:
            ad.samples.grad = None
        loss = torch.sum(torch.abs(ad.op(x) - yt) ** 2)
        loss.backward()
        return x.grad, ad.samples.grad

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    ms = _timed_steps(step, max(args.steps, 50), max(args.warmup, 3), flush)
    line = {
        "metric": "differentiable NUFFT forward+backward Msamples*coil/s (grads wrt image and trajectory)",
        "value": M * C / (ms / 1e3) / 1e6, "unit": UNIT, "n_gpus": 1, "steps": max(args.steps, 50),
        "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64",
        "data": "synthetic (Galilean spiral 64 x 2048, ellipse phantom, Gaussian coil maps, "
                "k-space from a 1e-3-perturbed trajectory)",
        "config": {"workload": "2D 256^2, 8 coils, spiral 64x2048 (131 072 samples); "
                               "loss |A(x) - y|^2, backward for x and the trajectory",
                   "nufft_calls_per_step": "1 forward + 1 adjoint (image grad) + 2 gradient "
                                           "interpolations (trajectory grad)",
                   "l2": "flushed between steps (256 MB write)"},
    }
    print(json.dumps(line), flush=True)


def run_gram(args):
    """Toeplitz Gram operator on the 3D workload: A^H A x for 16 coils by the
    Toeplitz embedding (pad, FFT, multiply, inverse FFT, crop; on 256^3
    circulant grids five fused line-transform passes) against one forward
    plus one adjoint NUFFT."""
    import torch

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    __graft_entry__.build()
    pkg = __graft_entry__.import_package()
    from mrinufft_gb300 import workloads

    traj, shape, img, smaps = workloads.config2(args.spokes, args.samples, args.coils, args.size)
    M, C = traj.shape[0], smaps.shape[0]
    op = pkg.MRIGB300(traj, shape, n_coils=C, smaps=smaps, squeeze_dims=False)
    x = torch.from_numpy(img).to(dev).reshape(1, *shape)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    toep = op._toeplitz()
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(max(args.warmup, 3)):
            fn()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    toep.profile(True)
    ms_toep = timed(lambda: op._gram_device(x))
    stages = {s: toep.profile_read(s) for s in ("pad", "fft", "kmul", "crop")}
    toep.profile(False)
    ms_nufft = timed(lambda: op._adj_device(op._op_device(x)))
    G = int(np.prod(toep.grid))
    peaks_path = ROOT / "MEASURED_PEAKS.json"
    peak = float(json.loads(peaks_path.read_text())["hbm_gbs"]) if peaks_path.exists() else 6800.0
    if stages["kmul"][1]:
        # pad, cuFFT, a separate multiply pass (the dominant kernel), cuFFT, crop
        kmul_ms = stages["kmul"][0] / stages["kmul"][1]
        kmul_bytes = 16 * op._ntrans * G + 4 * G
        roof = {"bound": "hbm", "kernel": "kmul", "achieved": kmul_bytes / (kmul_ms / 1e3) / 1e9,
                "peak": peak, "unit": "GB/s", "frac": kmul_bytes / (kmul_ms / 1e3) / 1e9 / peak,
                "algorithmic_bytes_per_launch": kmul_bytes}
    else:
        # 256^3 circulant grids: five fused line-transform passes per coil
        # pass (pad + z, y, x * K * x^-1, y, z + crop); algorithmic bytes of
        # one Gram application: image (read, written), maps (read twice),
        # per coil 4 x the z-line data (n0 n1 256 cells) and 4 x the x-mode
        # planes (n0 256^2 cells), and K once
        N3 = int(np.prod(shape))
        T = op._ntrans
        zl = shape[0] * shape[1] * 256 * 8
        xp = shape[0] * 256 * 256 * 8
        passes = -(-C // T)
        gram_bytes = 16 * N3 + 16 * C * N3 + C * (4 * zl + 4 * xp) + passes * 4 * G
        fft_ms = stages["fft"][0] / args.steps
        roof = {"bound": "hbm", "kernel": "fused Gram passes (pad+z, y, x*K*x^-1, y, z+crop)",
                "achieved": gram_bytes / (fft_ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                "frac": gram_bytes / (fft_ms / 1e3) / 1e9 / peak,
                "algorithmic_bytes_per_step": gram_bytes}
    line = {
        "metric": "Gram operator A^H A x Msamples*coil/s equivalent (Toeplitz embedding)",
        "value": M * C / (ms_toep / 1e3) / 1e6, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms_toep, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64",
        "data": "synthetic (seeded kooshball, ellipsoid phantom, Gaussian coil maps)",
        "config": {"workload": f"3D SENSE Gram, {shape[0]}^3 image, {C} coils, kooshball "
                               f"{args.spokes}x{args.samples}", "circulant_grid": list(toep.grid),
                   "kernel_build_s": build_s},
        "nufft_op_adj_ms": ms_nufft, "speedup_vs_nufft": ms_nufft / ms_toep,
        "stage_ms_per_step": {s: v[0] / args.steps for s, v in stages.items()},
        "roofline": roof,
    }
    print(json.dumps(line), flush=True)


def run_stacked(args):
    """Stacked NUFFT (stack-of-stars): radial 256 x 512 in-plane trajectory on
    all 64 planes of a 256 x 256 x 64 image, 16 coils; op + adj per step."""
    import torch

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    __graft_entry__.build()
    pkg = __graft_entry__.import_package()
    from mrinufft_gb300 import workloads

    shape, C = (256, 256, 64), 16
    s2 = workloads.radial_2d(256, 512).reshape(-1, 2).astype(np.float32)
    smaps = workloads.coil_maps(shape, C, seed=6)
    img = workloads.phantom(shape, seed=6)
    op = pkg.MRIStackedGB300(s2, shape, smaps=smaps, n_coils=C, z_index=None)
    M = op.n_samples
    x = torch.from_numpy(img).to(dev).reshape(1, *shape)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(max(args.warmup, 3)):
        op._adj_device(op._op_device(x))
    torch.cuda.synchronize()
    plan2 = op.operator.plan
    plan2.profile(True)
    e0.record()
    for _ in range(args.steps):
        op._adj_device(op._op_device(x))
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    stages = {s: plan2.profile_read(s)[0] / args.steps for s in ("pad", "fft", "interp", "spread", "crop", "zero")}
    plan2.profile(False)
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import esnufft

        ncores = os.cpu_count() or 1
        e = esnufft.EsNufft(s2.astype(np.float64) * 2 * np.pi, shape[:2], dtype=np.float32, nthreads=ncores)
        nrm = np.sqrt(np.prod(shape[:2]) * 4)
        planes = 8
        z = np.fft.fftshift(np.fft.fft(np.fft.ifftshift(img * smaps[0], axes=-1), axis=-1,
                                       norm="ortho"), axes=-1) / np.sqrt(2)
        t = time.perf_counter()
        for k in range(planes):
            _ = e.type1(e.type2(np.ascontiguousarray(z[..., k])) / nrm) / nrm
        dt = time.perf_counter() - t
        cpu = {"value": s2.shape[0] * planes / dt / 1e6, "unit": UNIT, "cores": ncores, "kind": "port",
               "sample": f"2D op+adj of {planes} planes of 1 coil (C/OpenMP ES spreader + scipy.fft); "
                         "z-FFT not timed"}
    line = {
        "metric": "stacked NUFFT op+adj Msamples*coil/s", "value": M * C / (ms / 1e3) / 1e6, "unit": UNIT,
        "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64",
        "data": "synthetic (radial 256 x 512 on 64 planes, ellipsoid phantom, Gaussian coil maps)",
        "config": {"workload": "stack-of-stars 256x256x64, 16 coils, 8.4M samples, op+adj",
                   "planes_2d_per_call": C * 64, "l2": "inputs > L2 (2D fine grids 2.1 GB)"},
        "stage_ms_per_step_2d": stages,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


def run_orc(args):
    """Off-resonance corrected SENSE op + adj: 2D 256^2 spiral 48 x 4096
    (196 608 samples, 12.3 ms readout), 16 coils, smooth +-120 Hz field map,
    "svd" interpolators; against the uncorrected op + adj."""
    import torch

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    __graft_entry__.build()
    pkg = __graft_entry__.import_package()
    from mrinufft_gb300 import workloads

    shape, C, NK = (256, 256), 16, 4096
    traj = workloads.spiral_2d(48, NK, power=2).reshape(-1, 2).astype(np.float32)
    M = traj.shape[0]
    smaps = workloads.coil_maps(shape, C, seed=8)
    img = workloads.phantom(shape, seed=8)
    yy, xx = np.meshgrid(np.linspace(-1, 1, shape[0]), np.linspace(-1, 1, shape[1]), indexing="ij")
    b0 = 120.0 * np.sin(2.0 * xx) * np.cos(1.5 * yy)
    t = np.arange(NK) * 3e-6
    op = pkg.MRIGB300(traj, shape, n_coils=C, smaps=smaps, squeeze_dims=False)
    t0 = time.perf_counter()
    cor = pkg.MRIFourierCorrectedGB300(op, b0_map=b0, readout_time=t, interpolator="svd")
    setup_s = time.perf_counter() - t0
    x = torch.from_numpy(img).to(dev).reshape(1, 1, *shape)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(max(args.warmup, 3)):
            fn()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    ms = timed(lambda: cor._adj_device(cor._op_device(x)))
    ms_plain = timed(lambda: op._adj_device(op._op_device(x)))
    L = cor.n_interpolators
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import esnufft

        ncores = os.cpu_count() or 1
        e = esnufft.EsNufft(traj.astype(np.float64) * 2 * np.pi, shape, dtype=np.float32, nthreads=ncores)
        nrm = np.sqrt(np.prod(shape) * 4)
        Bh, Ch = cor.B.cpu().numpy(), cor.C.cpu().numpy()
        tc = time.perf_counter()
        y = sum(e.type2(Ch[l] * img * smaps[0]).reshape(-1, NK) * Bh[:, l] for l in range(L)) / nrm
        _ = sum(np.conj(Ch[l]) * e.type1((y * np.conj(Bh[:, l])).reshape(-1)) for l in range(L)) / nrm
        dt = time.perf_counter() - tc
        cpu = {"value": M / dt / 1e6, "unit": UNIT, "cores": ncores, "kind": "port",
               "sample": f"corrected op+adj of 1 of {C} coils ({L} interpolators), C/OpenMP ES + scipy.fft"}
    line = {
        "metric": "off-resonance corrected op+adj Msamples*coil/s", "value": M * C / (ms / 1e3) / 1e6,
        "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64",
        "data": "synthetic (spiral 48 x 4096, ellipse phantom, Gaussian coil maps, smooth field map)",
        "config": {"workload": "2D 256^2 SENSE, 16 coils, 196 608 samples, +-120 Hz, 12.3 ms readout, svd",
                   "interpolators": L, "factorisation_s": setup_s},
        "uncorrected_op_adj_ms": ms_plain, "cost_vs_uncorrected": ms / ms_plain,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


def c5_templates(dev):
    """Request templates of the served mix: 2D 256^2 radial 256x512 with 8, 16,
    24 or 32 coils (70 %), 2D 384^2 spiral 32x4096 with 16 coils (20 %), 3D
    128^3 kooshball 2048x512 with 8 coils (10 %); k-space from each template's
    phantom through the forward operator plus complex noise."""
    import torch

    pkg = __graft_entry__.import_package()
    from mrinufft_gb300 import workloads

    out = []
    for i, (key, prob, kind, shape, C) in enumerate(workloads.SERVE_MIX):
        traj, smaps, x = workloads.serve_template(i)
        op = pkg.MRIGB300(traj, shape, n_coils=C, smaps=smaps, squeeze_dims=False, device=dev.index)
        y = op.op(torch.from_numpy(x).to(dev)).reshape(C, -1)
        y = y + 0.01 * torch.randn_like(y)
        # k-space arrives in pinned host memory (copied to the device per request)
        out.append({"key": key, "prob": prob, "samples": traj, "shape": shape, "smaps": smaps,
                    "kspace": y.cpu().pin_memory()})
        del op
    return out


def run_c5(args):
    """Served CG reconstructions on a Poisson stream, and the saturated
    comparison with the plain per-call backend."""
    import torch

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    __graft_entry__.build()
    pkg = __graft_entry__.import_package()
    from mrinufft_gb300.serving import ReconRequest, ReconServer

    tpl = c5_templates(dev)
    probs = np.array([t["prob"] for t in tpl])
    rng = np.random.default_rng(50)

    def make(n, arrivals):
        picks = rng.choice(len(tpl), size=n, p=probs / probs.sum())
        reqs = []
        for i, (k, a) in enumerate(zip(picks, arrivals)):
            t = tpl[k]
            reqs.append(ReconRequest(rid=i, samples=t["samples"], shape=t["shape"], kspace=t["kspace"],
                                     smaps=t["smaps"], seed=i, traj_key=t["key"], smaps_key=t["key"],
                                     arrival=float(a)))
        return reqs

    # warm the kernels; every server below builds its resident plans before
    # requests arrive (prewarm), as a long-running service holds them
    warm = make(len(tpl) * 2, np.zeros(len(tpl) * 2))
    ReconServer(max_active=32).run(warm, realtime=False)
    torch.cuda.synchronize()
    # Poisson stream
    gaps = rng.exponential(1.0 / args.rate, size=int(args.rate * args.duration * 1.2) + 10)
    arr = np.cumsum(gaps)
    arr = arr[arr < args.duration]
    srv = ReconServer(hbm_budget_bytes=150e9, max_active=32)
    stream_reqs = make(len(arr), arr)
    srv.prewarm(stream_reqs)
    done = srv.run(stream_reqs, realtime=True)
    stream = ReconServer.stats(done)
    stream["ledger_peak_bytes"] = srv.ledger.peak
    # saturated: every request present at t = 0, served with both iteration
    # forms and run through the plain per-call backend with both
    nsat = args.saturated
    sat_reqs = make(nsat, np.zeros(nsat))

    def served(gram):
        reqs = [ReconRequest(rid=r.rid, samples=r.samples, shape=r.shape, kspace=r.kspace,
                             smaps=r.smaps, seed=r.seed, traj_key=r.traj_key, smaps_key=r.smaps_key)
                for r in sat_reqs]
        srv2 = ReconServer(hbm_budget_bytes=150e9, max_active=32, gram=gram)
        srv2.prewarm(reqs)
        ReconServer(max_active=32, gram=gram).run(make(len(tpl), np.zeros(len(tpl))), realtime=False)
        torch.cuda.synchronize()
        sampler = ClockSampler(0)
        sampler.start()
        t0 = time.perf_counter()
        srv2.run(reqs, realtime=False)
        dt = time.perf_counter() - t0
        return dt, sampler.stop(), srv2.ledger.peak

    served_s, served_clk, peak_bytes = served("toeplitz")
    served_nufft_s, served_nufft_clk, _ = served("nufft")
    # plain per-call backend on the same requests (host-synchronised CG loop)
    ops = {}
    for t in tpl:  # the plain backend's operators exist before the requests arrive
        ops[t["key"]] = pkg.MRIGB300(t["samples"], t["shape"], n_coils=t["smaps"].shape[0],
                                     smaps=t["smaps"], device=0)
        ops[t["key"]].pinv_solver(t["kspace"].to(dev), optim="cg", max_iter=2)
        ops[t["key"]].pinv_solver(t["kspace"].to(dev), optim="cg", max_iter=2, toeplitz=True)
    torch.cuda.synchronize()

    def plain(toeplitz):
        sampler = ClockSampler(0)
        sampler.start()
        t0 = time.perf_counter()
        for r in sat_reqs:
            np.random.seed(r.seed)
            ops[r.traj_key].pinv_solver(r.kspace.to(dev, non_blocking=True), optim="cg", max_iter=10,
                                        toeplitz=toeplitz)
        torch.cuda.synchronize()
        return time.perf_counter() - t0, sampler.stop()

    plain_s, plain_clk = plain(False)
    plain_toep_s, plain_toep_clk = plain(True)
    line = {
        "metric": "served CG reconstructions: p50/p99 latency (ms) and recon/s",
        "value": nsat / served_s, "unit": "recon/s", "n_gpus": 1, "steps": nsat, "warmup": len(tpl) * 2,
        "higher_is_better": True, "dtype": "c64",
        "data": "synthetic (seeded radial / spiral / kooshball templates, phantoms, coil maps)",
        "config": {"workload": "Poisson %.0f req/s for %.0f s; 70%% 2D 256^2 radial 256x512 8-32 coils, "
                               "20%% 2D 384^2 spiral 32x4096 16 coils, 10%% 3D 128^3 kooshball "
                               "2048x512 8 coils; CG 10 iterations; 150 GB budget"
                               % (args.rate, args.duration), "max_active": 32},
        "stream": stream,
        "saturated": {
            "requests": nsat,
            "served_toeplitz_recon_per_s": nsat / served_s,
            "served_nufft_recon_per_s": nsat / served_nufft_s,
            "plain_per_call_nufft_recon_per_s": nsat / plain_s,
            "plain_per_call_toeplitz_recon_per_s": nsat / plain_toep_s,
            "speedup_served_vs_plain": plain_s / served_s,
            "speedup_batching_only_toeplitz": plain_toep_s / served_s,
            "speedup_batching_only_nufft": plain_s / served_nufft_s,
            "speedup_toeplitz_only_plain": plain_s / plain_toep_s,
            "ledger_peak_bytes": peak_bytes,
            "served_clocks": served_clk, "served_nufft_clocks": served_nufft_clk,
            "plain_clocks": plain_clk, "plain_toeplitz_clocks": plain_toep_clk},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "c1":
        run_c1(args)
    elif args.workload == "c3":
        run_c3(args)
    elif args.workload == "c4":
        run_c4(args)
    elif args.workload == "gram":
        run_gram(args)
    elif args.workload == "stacked":
        run_stacked(args)
    elif args.workload == "orc":
        run_orc(args)
    elif args.workload == "c5":
        run_c5(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
