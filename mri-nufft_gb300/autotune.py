"""Autotuner of bin sizes, interpolation method and subproblem size.

For a problem class — (dim, image size, sampling density, coil count) — it
times the candidate configurations on the instance's own trajectory (one
forward + one adjoint of random data per candidate, CUDA events, best of a
few repetitions) and keeps the fastest.  Results are cached in a JSON file
(``GBN_TUNE_CACHE`` or ``~/.cache/mrinufft_gb300/tune.json``) so a class is
timed once per machine.  Sampling density is bucketed by powers of two of
samples per fine-grid cell.
"""

from __future__ import annotations

import json
import math
import os
from pathlib import Path

import torch

from .params import fine_shape
from .plan import NufftPlan

CANDIDATES = {
    # "auto" is the dimension's default kernel (2D: warp-cooperative direct
    # interpolation; 3D: shared-memory tiles); in 2D the bins set the sort
    # order (locality) of the direct kernels
    2: [
        {"bins": (32, 32), "interp": "auto", "maxsub": 512},
        {"bins": (16, 16), "interp": "auto", "maxsub": 512},
        {"bins": (64, 64), "interp": "auto", "maxsub": 1024},
        {"bins": (8, 8), "interp": "auto", "maxsub": 512},
    ],
    3: [
        {"bins": (8, 8, 8), "interp": "auto", "maxsub": 512},
        {"bins": (9, 9, 9), "interp": "auto", "maxsub": 512},
        {"bins": (8, 8, 8), "interp": "warp_direct", "maxsub": 512},
        {"bins": (9, 9, 9), "interp": "warp_direct", "maxsub": 512},
    ],
}


def default_cache_path() -> Path:
    env = os.environ.get("GBN_TUNE_CACHE")
    if env:
        return Path(env)
    return Path.home() / ".cache" / "mrinufft_gb300" / "tune.json"


class Autotuner:
    def __init__(self, cache_path=None, reps=3, eps=1e-6, persist=True, interp_methods=None):
        self.path = Path(cache_path) if cache_path else default_cache_path()
        self.interp_methods = None if interp_methods is None else tuple(interp_methods)
        self.reps = reps
        self.eps = eps
        self.persist = persist
        self.cache = {}
        if self.path.exists():
            try:
                self.cache = json.loads(self.path.read_text())
            except (OSError, ValueError):
                self.cache = {}

    def key(self, shape, M, C):
        G = 1
        for n in fine_shape(shape, self.eps):
            G *= n
        bucket = int(round(math.log2(max(M, 1) / G))) if M > 0 else -99
        meth = "all" if self.interp_methods is None else "+".join(self.interp_methods)
        return (f"{len(shape)}d:{'x'.join(map(str, shape))}:dens2^{bucket}:c{C}:eps{self.eps:g}"
                f":{meth}")

    def _time(self, shape, k, C, cfg):
        dev = k.device
        plan = NufftPlan(shape, eps=self.eps, ntrans=C, device=dev.index)
        plan.tune(bins=cfg["bins"], interp=cfg["interp"], maxsub_cap=cfg["maxsub"])
        plan.setpts(k)
        M = k.shape[0]
        g = torch.Generator(device=dev).manual_seed(0)
        x = torch.randn((C, *shape), dtype=torch.complex64, device=dev, generator=g)
        y = torch.empty((C, M), dtype=torch.complex64, device=dev)
        z = torch.empty_like(x)
        plan.op(x, None, y, 1, C, 1.0)
        plan.adj(y, None, None, z, 1, C, 1.0)
        best = float("inf")
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for _ in range(self.reps):
            e0.record()
            plan.op(x, None, y, 1, C, 1.0)
            plan.adj(y, None, None, z, 1, C, 1.0)
            e1.record()
            torch.cuda.synchronize(dev)
            best = min(best, e0.elapsed_time(e1))
        return best

    def best(self, shape, k, C):
        """Fastest configuration for (shape, samples k (M, d) radians on the GPU, C coils)."""
        shape = tuple(int(v) for v in shape)
        key = self.key(shape, k.shape[0], C)
        if key in self.cache:
            c = self.cache[key]
            return {"bins": tuple(c["bins"]), "interp": c["interp"], "maxsub": c["maxsub"]}
        timings = []
        for cfg in CANDIDATES[len(shape)]:
            if self.interp_methods is not None and cfg["interp"] not in self.interp_methods:
                continue
            try:
                t = self._time(shape, k, C, cfg)
            except (ValueError, MemoryError):
                continue
            timings.append((t, cfg))
        t, cfg = min(timings, key=lambda x: x[0])
        self.cache[key] = {"bins": list(cfg["bins"]), "interp": cfg["interp"],
                           "maxsub": cfg["maxsub"], "ms": t,
                           "timings": {f"{c['bins']}/{c['interp']}": tt for tt, c in timings}}
        if self.persist:
            try:
                self.path.parent.mkdir(parents=True, exist_ok=True)
                self.path.write_text(json.dumps(self.cache, indent=1, sort_keys=True))
            except OSError:
                pass
        return dict(cfg)
