"""Batched form: many uneven NUFFT instances in persistent launches.

``BatchedNufft`` holds independent SENSE (or calibrationless) problems of
different image sizes, sample counts and coil counts.  One op or adj of the
whole batch is one persistent launch per stage of ``libgbnufft.so``
(``gbn_batch_op`` / ``gbn_batch_adj``: pad, interp; zero, spread, crop)
driven by per-instance work tables, plus one cuFFT call per instance; the
op + adj step can be captured once in a CUDA graph and replayed.  Bin sizes
and the interpolation method of every instance come from ``autotune``.

The reference has no such form: its only batching is ``n_trans`` chunks of
one trajectory (``operators/base.py:904-914``, ``cufinufft.py:259-269``); the
per-instance semantics are those of ``MRIGB300.op`` / ``adj_op``.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _array, _lib
from ._traj import proper_trajectory
from .autotune import Autotuner
from .plan import NufftPlan


class BatchedNufft:
    """Op / adj of many independent instances at once.

    instances: sequence of dicts with keys ``samples`` ((M, d), unit or
        radians), ``shape``, optional ``smaps`` ((C, *shape)), ``n_coils``
        (calibrationless when no maps) and ``density`` ((M,)).
    """

    def __init__(self, instances, eps=1e-6, device=None, autotune=True, tuner=None):
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.eps = eps
        self.plans, self.imgs, self.ksps, self.smaps, self.dens = [], [], [], [], []
        self.shapes, self.coils, self.sense, self.scales = [], [], [], []
        # the batched kernels are the dimension's defaults: tune bins and subproblem size
        tuner = tuner if tuner is not None else (
            Autotuner(eps=eps, interp_methods=("auto",)) if autotune else None)
        dims = set()
        for inst in instances:
            shape = tuple(int(v) for v in inst["shape"])
            dims.add(len(shape))
            s = proper_trajectory(inst["samples"], "pi")
            k = _array.to_tensor(s, self.device, torch.float32).reshape(-1, len(shape))
            smaps = inst.get("smaps")
            C = int(smaps.shape[0]) if smaps is not None else int(inst.get("n_coils", 1))
            plan = NufftPlan(shape, eps=eps, ntrans=C, device=self.device.index)
            if tuner is not None:
                cfg = tuner.best(shape, k, C)
                plan.tune(bins=cfg["bins"], interp=cfg["interp"], maxsub_cap=cfg["maxsub"])
            plan.setpts(k)
            self.plans.append(plan)
            self.shapes.append(shape)
            self.coils.append(C)
            self.sense.append(smaps is not None)
            self.imgs.append(torch.zeros(((1 if smaps is not None else C), *shape),
                                         dtype=torch.complex64, device=self.device))
            self.ksps.append(torch.zeros((C, k.shape[0]), dtype=torch.complex64, device=self.device))
            self.smaps.append(None if smaps is None else _array.to_tensor(smaps, self.device, torch.complex64))
            d = inst.get("density")
            self.dens.append(None if d is None else _array.to_tensor(d, self.device, torch.float32))
            self.scales.append(1.0 / float(np.sqrt(np.prod(shape) * 2 ** len(shape))))
        if len(dims) != 1:
            raise ValueError("all instances of a batch must share the dimension")
        self.lib = _lib.load()
        n = len(self.plans)
        arr = (ctypes.c_void_p * n)(*[p._h.value for p in self.plans])
        self._h = ctypes.c_void_p()
        _lib.check(self.lib.gbn_batch_create(n, arr, ctypes.byref(self._h)), "gbn_batch_create")
        self._bind()
        self.graph = None

    def _bind(self):
        n = len(self.plans)
        vp = ctypes.c_void_p
        imgs = (vp * n)(*[t.data_ptr() for t in self.imgs])
        smaps = (vp * n)(*[0 if t is None else t.data_ptr() for t in self.smaps])
        ksps = (vp * n)(*[t.data_ptr() for t in self.ksps])
        dens = (vp * n)(*[0 if t is None else t.data_ptr() for t in self.dens])
        scales = (ctypes.c_float * n)(*self.scales)
        coils = (ctypes.c_int * n)(*self.coils)
        _lib.check(self.lib.gbn_batch_bind(self._h, imgs, smaps, ksps, dens, scales, coils),
                   "gbn_batch_bind")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self.lib.gbn_batch_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    @property
    def n_samples_coils(self) -> int:
        return int(sum(k.numel() for k in self.ksps))

    def set_images(self, images):
        for buf, x in zip(self.imgs, images):
            buf.copy_(_array.to_tensor(x, self.device, torch.complex64).reshape(buf.shape))

    def set_kspace(self, kspaces):
        for buf, y in zip(self.ksps, kspaces):
            buf.copy_(_array.to_tensor(y, self.device, torch.complex64).reshape(buf.shape))

    def op(self):
        """k-space of every instance from its bound image (in ``self.ksps``)."""
        _lib.check(self.lib.gbn_batch_op(self._h, self.stream), "gbn_batch_op")
        return self.ksps

    def adj(self):
        """Adjoint of every instance's bound k-space (into ``self.imgs``)."""
        _lib.check(self.lib.gbn_batch_adj(self._h, self.stream), "gbn_batch_adj")
        return self.imgs

    def step(self):
        """op then adj of every instance (the batched benchmark step)."""
        self.op()
        self.adj()

    def capture(self):
        """Capture ``step`` in a CUDA graph; ``replay()`` then runs it."""
        self.step()  # warm up: cuFFT plans and kernel attributes exist before capture
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            g.capture_begin()
            self.step()
            g.capture_end()
        torch.cuda.current_stream(self.device).wait_stream(s)
        self.graph = g
        return g

    def replay(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()
