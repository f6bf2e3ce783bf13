"""Batched form: many uneven NUFFT instances per launch sequence.

``BatchedNufft`` holds independent SENSE (or calibrationless) problems of
different image sizes, sample counts and coil counts, in one of two modes:

* ``"streams"`` (default): every instance keeps its own plan and runs the
  plain backend's kernels (streaming spreaders, tile / warp interpolation,
  pruned FFTs); the instances are spread over ``n_streams`` CUDA streams by
  a longest-first greedy split of their work, so that small instances
  overlap on the GPU, and the whole op + adj step is captured in one CUDA
  graph (fork / join by events) and replayed;
* ``"persistent"``: one persistent launch per stage of ``libgbnufft.so``
  (``gbn_batch_op`` / ``gbn_batch_adj``: pad, interp; zero, spread, crop)
  driven by per-instance work tables, plus one cuFFT call per fine-grid
  size group; also capturable in a CUDA graph.

Bin sizes and the interpolation method of every instance come from
``autotune``.

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

    def __init__(self, instances, eps=1e-6, device=None, autotune=True, tuner=None,
                 mode="streams", n_streams=4):
        if mode not in ("streams", "persistent"):
            raise ValueError("mode must be 'streams' or 'persistent'")
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.eps = eps
        self.mode = mode
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
        self._h = ctypes.c_void_p()
        self.graph = None
        if mode == "persistent":
            n = len(self.plans)
            arr = (ctypes.c_void_p * n)(*[p._h.value for p in self.plans])
            _lib.check(self.lib.gbn_batch_create(n, arr, ctypes.byref(self._h)), "gbn_batch_create")
            self._bind()
            return
        # longest-first greedy split of the instances over the streams, by
        # work ~ samples x coils + fine cells x coils
        work = []
        for plan, C, ksp in zip(self.plans, self.coils, self.ksps):
            nf = plan.info()["nf"]
            work.append(ksp.numel() + C * int(np.prod(nf)))
        n_streams = max(1, min(int(n_streams), len(self.plans)))
        loads = [0] * n_streams
        self.groups = [[] for _ in range(n_streams)]
        for i in sorted(range(len(work)), key=lambda i: -work[i]):
            k = int(np.argmin(loads))
            self.groups[k].append(i)
            loads[k] += work[i]
        self.streams = [torch.cuda.Stream(self.device) for _ in range(n_streams)]

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

    def _op_one(self, i):
        C = self.coils[i]
        x = self.imgs[i]
        self.plans[i].op(x, self.smaps[i], self.ksps[i], 1, C, self.scales[i])

    def _adj_one(self, i):
        C = self.coils[i]
        self.plans[i].adj(self.ksps[i], self.dens[i], self.smaps[i], self.imgs[i], 1, C, self.scales[i])

    def _fork(self, fn):
        """Run fn(i) for every instance on its stream, joined to the current one."""
        cur = torch.cuda.current_stream(self.device)
        start = torch.cuda.Event()
        start.record(cur)
        ends = []
        for st, grp in zip(self.streams, self.groups):
            st.wait_event(start)
            with torch.cuda.stream(st):
                for i in grp:
                    fn(i)
            e = torch.cuda.Event()
            e.record(st)
            ends.append(e)
        for e in ends:
            cur.wait_event(e)

    def op(self):
        """k-space of every instance from its bound image (in ``self.ksps``)."""
        if self.mode == "persistent":
            _lib.check(self.lib.gbn_batch_op(self._h, self.stream), "gbn_batch_op")
        else:
            self._fork(self._op_one)
        return self.ksps

    def adj(self):
        """Adjoint of every instance's bound k-space (into ``self.imgs``)."""
        if self.mode == "persistent":
            _lib.check(self.lib.gbn_batch_adj(self._h, self.stream), "gbn_batch_adj")
        else:
            self._fork(self._adj_one)
        return self.imgs

    def step(self):
        """op then adj of every instance (the batched benchmark step)."""
        if self.mode == "persistent":
            self.op()
            self.adj()
        else:
            self._fork(lambda i: (self._op_one(i), self._adj_one(i)))

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
