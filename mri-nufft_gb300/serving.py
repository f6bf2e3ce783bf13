"""Served form: continuous batching of CG reconstructions on one GPU.

``ReconServer`` accepts CG data-consistency reconstructions (the work of
``pinv_solver(optim="cg")``, ``extras/optim.py:801-902``, with its power-method
Lipschitz estimate, ``operators/base.py:1155-1221``) of different dims, sizes
and coil counts as they arrive:

* admission: a request is admitted when a slot is free and its device bytes
  fit the HBM budget next to the requests already on the GPU; otherwise it
  waits in the queue;
* residency: sorted trajectories stay on the device in a pool of plans keyed
  by trajectory (requests of one protocol reuse the bin sort), and each
  admitted request keeps its coil maps, k-space and CG state on the device;
* continuous batching: every scheduling tick issues the next unit of work
  (one power iteration or one CG iteration) of every admitted request, each
  request on its own CUDA stream, so the work of many requests overlaps on
  the device; a request that finishes frees its slot and memory at once and
  a waiting one is admitted at the next tick;
* no host synchronisation inside a solve: the power-method normalisation,
  the CG step (Polak-Ribiere beta with numpy's complex ``max(0, beta)``, the
  ``tol`` early exit) and their FP64 reductions run on the device
  (``gbn_power_step``, ``gbn_cg_update``, ``gbn_dotu_f64``, ``gbn_norm2_f64``);
* FFT-only iterations (default): the power method and the CG gradients use
  the Toeplitz embedding of the Gram operator (``gbn_toep_*``; A^H W A x as
  a circulant convolution on a 2N grid), so an iteration runs FFTs and one
  multiply per coil instead of a spread and an interpolation.  The CG
  gradient A^H A x - A^H y takes A^H y from one adjoint transform at the
  start.  The Toeplitz kernel of a trajectory is built once and pooled with
  its sorted plan.  ``gram="nufft"`` keeps the NUFFT data-consistency
  iterations of ``pinv_solver(optim="cg")`` instead;
* HBM budget: an :class:`HbmLedger` charges every resident sorted
  trajectory (pooled or in use), every resident coil map and the state of
  every admitted request; requests wait, and idle pooled trajectories are
  freed, so that the total never exceeds the budget.

Each result equals the same request run alone (and ``MRIGB300.pinv_solver``
with the same power-method start vector) up to float rounding.
"""

from __future__ import annotations

import ctypes
import time
from collections import defaultdict, deque
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _array, _lib
from ._traj import proper_trajectory
from .params import fine_cells
from .plan import NufftPlan, _ptr


@dataclass
class ReconRequest:
    """One CG reconstruction (SENSE when ``smaps`` is given)."""

    rid: int
    samples: object           # (M, d), unit or radians
    shape: tuple
    kspace: object            # (C, M)
    smaps: object = None      # (C, *shape)
    density: object = None    # (M,)
    max_iter: int = 10
    tol: float = 1e-4
    seed: int = 0             # power-method start vector
    traj_key: object = None   # requests with equal keys share a sorted trajectory
    smaps_key: object = None  # requests with equal keys share resident coil maps
    arrival: float = 0.0
    result: torch.Tensor = None
    t_admit: float = None
    t_done: float = None
    lipschitz: float = None

    @property
    def n_coils(self):
        return int(self.kspace.shape[0]) if self.kspace.ndim > 1 else 1


def start_vector(shape, seed):
    """1j * U[0,1) + U[0,1), the start vector of the GPU backends'
    ``get_lipschitz_cst`` (cufinufft.py:1265-1266), from a seeded generator
    (imaginary part drawn first, both parts rounded to float32)."""
    rs = np.random.RandomState(seed)
    x = np.empty(shape, np.complex64)
    x.imag = rs.random_sample(shape)
    x.real = rs.random_sample(shape)
    return x


def plan_set_bytes(shape, M, C, eps=1e-6):
    """Device bytes of one resident sorted trajectory for C coils: the NUFFT
    plan (C fine grids, sorted coordinates, permutation, bin and subproblem
    tables) and its Toeplitz embedding (C circulant grids and the kernel
    spectrum).  An upper bound of what the library allocates for them."""
    G = fine_cells(shape, eps)
    d = len(shape)
    plan = 8 * C * G + M * (16 + 4 * d) + 64 * (G // 64 + 1024) + (1 << 20)
    toep = 8 * C * G + 4 * G + (1 << 20)
    return int(plan + toep)


def smaps_bytes(shape, C):
    return int(8 * C * int(np.prod(shape)))


def solve_bytes(shape, M, C, density=False, cached_smaps=False, gram="toeplitz", eps=1e-6):
    """Device bytes of one admitted request besides its sorted trajectory:
    coil maps (unless resident), k-space, density and, for a request with
    density, the weighted Toeplitz kernel of its power method; the CG and
    power-method vectors."""
    N = int(np.prod(shape))
    b = 8 * C * M + 8 * N * 12 + 8 * M
    if not cached_smaps:
        b += smaps_bytes(shape, C)
    if density:
        b += 4 * M
        if gram == "toeplitz":
            b += 8 * C * fine_cells(shape, eps) + 4 * fine_cells(shape, eps)
    return int(b)


def request_bytes(shape, M, C, eps=1e-6):
    """Device bytes of a request that brings its own sorted trajectory and
    coil maps (the most it can add to the device)."""
    return plan_set_bytes(shape, M, C, eps) + solve_bytes(shape, M, C, eps=eps)


class HbmLedger:
    """Device bytes a server holds, against its HBM budget.

    ``resident`` counts what outlives a request: every sorted trajectory with
    its Toeplitz embedding that the server has built (admitted or waiting in
    the pool) and the coil maps kept by key; ``active`` the per-request
    state of admitted requests.  Admission and pre-building only proceed
    when ``resident + active + need`` stays within the budget, so the sum
    never exceeds it (``peak`` records the largest total seen)."""

    def __init__(self, budget):
        self.budget = float(budget)
        self.resident = 0
        self.active = 0
        self.peak = 0

    @property
    def total(self):
        return self.resident + self.active

    def fits(self, need):
        return self.total + need <= self.budget

    def _mark(self):
        self.peak = max(self.peak, self.total)

    def add_resident(self, b):
        self.resident += int(b)
        self._mark()

    def drop_resident(self, b):
        self.resident -= int(b)

    def add_active(self, b):
        self.active += int(b)
        self._mark()

    def drop_active(self, b):
        self.active -= int(b)


class _PlanSet:
    """A sorted trajectory: the NUFFT plan and, for the Toeplitz iterations,
    the Toeplitz embedding of its unweighted Gram operator."""

    def __init__(self, plan, gram, nbytes):
        from .plan import ToeplitzKernel

        self.plan = plan
        self.toep = ToeplitzKernel(plan, None) if gram == "toeplitz" else None
        self.bytes = int(nbytes)


class _Solve:
    """Device state and unit generator of one admitted request."""

    def __init__(self, server, req, pset, stream, nbytes):
        self.server, self.req, self.stream = server, req, stream
        self.pset, self.plan = pset, pset.plan
        self.dev = server.device
        self.lib = server.lib
        self.gram = server.gram
        shape = tuple(int(v) for v in req.shape)
        self.shape = shape
        C = req.n_coils
        self.C = C
        with torch.cuda.stream(stream):
            self.y = _array.to_tensor(req.kspace, self.dev, torch.complex64).reshape(C, -1)
            self.smaps = None if req.smaps is None else server._smaps_of(req, C, shape)
            self.dens = (None if req.density is None
                         else _array.to_tensor(req.density, self.dev, torch.float32).reshape(-1))
            x0 = req._x0.result() if getattr(req, "_x0", None) is not None else start_vector(shape, req.seed)
            self.x0 = torch.from_numpy(x0).to(self.dev)
        self.M = self.y.shape[1]
        self.scale = 1.0 / float(np.sqrt(np.prod(shape) * 2 ** len(shape)))
        self.bytes = int(nbytes)
        self._sth = None
        self.gen = self._units()
        self.event = None

    def _st(self):
        if self._sth is None:
            self._sth = ctypes.c_void_p(self.stream.cuda_stream)
        return self._sth

    def _ck(self, status, what):
        _lib.check(status, what)

    def _dots(self, gnew, grad, st, n):
        """state[0..6] of gbn_cg_update: dot(g_new, g_new), dot(g_new, g),
        dot(g, g) (non-conjugating) and |g_new|^2, on the device."""
        sth = self._st()
        self._ck(self.lib.gbn_dotu_f64(_ptr(gnew), _ptr(gnew), n, 0, _ptr(st[0:2]), sth), "dot")
        self._ck(self.lib.gbn_dotu_f64(_ptr(gnew), _ptr(grad), n, 0, _ptr(st[2:4]), sth), "dot")
        self._ck(self.lib.gbn_dotu_f64(_ptr(grad), _ptr(grad), n, 0, _ptr(st[4:6]), sth), "dot")
        self._ck(self.lib.gbn_norm2_f64(_ptr(gnew), n, _ptr(st[6:7]), sth), "norm2")

    def _units(self):
        dev, plan, shape, C = self.dev, self.plan, self.shape, self.C
        n = int(np.prod(shape))
        sense = self.smaps is not None
        img_shape = (1, *shape) if sense else (C, *shape)
        nimg = int(np.prod(img_shape))
        f32 = dict(dtype=torch.float32, device=dev)
        c64 = dict(dtype=torch.complex64, device=dev)
        f64 = dict(dtype=torch.float64, device=dev)
        scale2 = self.scale * self.scale
        toeplitz = self.gram == "toeplitz"
        toep = self.pset.toep
        toep_w = toep
        if toeplitz and self.dens is not None:
            from .plan import ToeplitzKernel

            toep_w = ToeplitzKernel(plan, self.dens)  # A^H D A of the power method
        L = torch.zeros(1, **f32)
        pst = torch.zeros(4, **f64)
        x = torch.empty((1, *shape), **c64)
        xn = torch.empty((1, *shape), **c64)
        ktmp = torch.empty((1, self.M), **c64)
        # -- power method on the single-coil, map-free operator with density
        self._ck(self.lib.gbn_norm2_f64(_ptr(self.x0), n, _ptr(pst), self._st()), "norm2")
        self._ck(self.lib.gbn_power_step(n, _ptr(self.x0), _ptr(x), _ptr(pst), _ptr(L), self._st()),
                 "power step")
        yield
        sth = self._st()
        for _ in range(10):
            if toeplitz:
                toep_w.power_iter(x, xn, pst, L, scale2, sth)
            else:
                plan.op(x, None, ktmp, 1, 1, self.scale)
                plan.adj(ktmp, self.dens, None, xn, 1, 1, self.scale)
                self._ck(self.lib.gbn_norm2_f64(_ptr(xn), n, _ptr(pst), sth), "norm2")
                self._ck(self.lib.gbn_power_step(n, _ptr(xn), _ptr(x), _ptr(pst), _ptr(L), sth),
                         "power step")
            yield
        self.L = L
        # -- start image: scaled density-compensated adjoint (optim.py:151-165)
        image = torch.zeros(img_shape, **c64)
        y = self.y.reshape(1, C, self.M)
        if self.dens is not None:
            plan.adj(y, self.dens, self.smaps, image, 1, C, self.scale)
            yy = torch.empty((1, C, self.M), **c64)
            plan.op(image.reshape(1 if sense else C, *shape), self.smaps, yy, 1, C, self.scale)
            nrm = torch.empty(2, **f64)
            self._ck(self.lib.gbn_norm2_f64(_ptr(y), y.numel(), _ptr(nrm[0:1]), self._st()), "norm2")
            self._ck(self.lib.gbn_norm2_f64(_ptr(yy), yy.numel(), _ptr(nrm[1:2]), self._st()), "norm2")
            self._ck(self.lib.gbn_scale_ratio(nimg, _ptr(image), _ptr(nrm[0:1]), _ptr(nrm[1:2]),
                                              self._st()), "scale")
            yield
        # -- CG iterations without density (optim.py:838-842)
        grad = torch.empty(img_shape, **c64)
        gnew = torch.empty(img_shape, **c64)
        xin = image.reshape(1 if sense else C, *shape)
        if toeplitz:
            # A^H (A x - y) = A^H A x - A^H y with A^H y from one adjoint
            rhs = torch.empty(img_shape, **c64)
            plan.adj(y, None, self.smaps, rhs, 1, C, self.scale)
            toep.apply(xin, self.smaps, grad, 1, C, scale2)
            grad -= rhs
        else:
            plan.dc(xin, y, None, self.smaps, grad, 1, C, self.scale)
        velocity = grad / L
        image -= velocity
        st = torch.zeros(8, **f64)
        yield
        tol = float(self.req.tol)
        for _ in range(self.req.max_iter):
            if toeplitz:
                toep.cg_iter(image, self.smaps, rhs, grad, gnew, velocity, st, L, 1, C, scale2, tol, sth)
            else:
                plan.dc(xin, y, None, self.smaps, gnew, 1, C, self.scale)
                self._dots(gnew, grad, st, nimg)
                self._ck(self.lib.gbn_cg_update(nimg, _ptr(gnew), _ptr(grad), _ptr(velocity),
                                                _ptr(image), _ptr(st), _ptr(L), tol, sth), "cg update")
            yield
        self.image = image
        self.event = torch.cuda.Event()
        self.event.record(self.stream)

    def step(self):
        """Issue the next unit; False once every unit is issued."""
        with torch.cuda.stream(self.stream):
            try:
                next(self.gen)
                return True
            except StopIteration:
                return False


class ReconServer:
    """Continuous-batching CG reconstruction service on one GPU.

    ``gram="toeplitz"`` (default) runs the power method and the CG gradients
    on the Toeplitz embedding of the Gram operator; ``gram="nufft"`` runs
    them as in ``pinv_solver(optim="cg")``, a forward and an adjoint NUFFT
    per iteration (data consistency), with the same device-side steps.
    Everything the server keeps on the device is charged to an
    :class:`HbmLedger` against ``hbm_budget_bytes``."""

    def __init__(self, hbm_budget_bytes=150e9, max_active=32, device=None, eps=1e-6,
                 gram="toeplitz"):
        if gram not in ("toeplitz", "nufft"):
            raise ValueError("gram must be 'toeplitz' or 'nufft'")
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.gram = gram
        self.ledger = HbmLedger(hbm_budget_bytes)
        self.max_active = int(max_active)
        self.eps = eps
        self.lib = _lib.load()
        self.queue = deque()
        self.active = []
        self.finishing = []
        self.done = []
        self.plans = defaultdict(list)   # (traj key, shape, coils) -> free sorted plans
        self.smaps_cache = {}            # smaps key -> resident coil maps
        self.rng_pool = ThreadPoolExecutor(max_workers=4)
        self.streams = [None] * self.max_active  # created on first use
        self.free_streams = list(range(self.max_active))
        self.t0 = time.perf_counter()

    @property
    def budget(self):
        return self.ledger.budget

    def _stream(self, i):
        if self.streams[i] is None:
            self.streams[i] = torch.cuda.Stream(self.device)
        return self.streams[i]

    def now(self):
        return time.perf_counter() - self.t0

    @staticmethod
    def _key(req):
        shape = tuple(int(v) for v in req.shape)
        return (req.traj_key if req.traj_key is not None else ("rid", req.rid), shape, req.n_coils)

    def _pset_bytes(self, req):
        return plan_set_bytes(tuple(req.shape), int(np.asarray(req.kspace.shape)[-1]), req.n_coils,
                              self.eps)

    def prewarm(self, requests, per_key=None):
        """Build the resident sorted plans (and Toeplitz kernels) that
        ``requests`` will need before they arrive, so that admission never
        sorts a trajectory on a request's critical path: ``per_key`` plan sets
        per trajectory key, by default the key's share of the slots (its
        share of ``requests`` times ``max_active``, plus 2).  Building stops
        where the next plan set would not fit the HBM budget."""
        counts, first = defaultdict(int), {}
        for r in requests:
            key = self._key(r)
            counts[key] += 1
            first.setdefault(key, r)
        n = max(1, len(requests))
        for key, r in first.items():
            want = (int(per_key) if per_key is not None
                    else min(self.max_active, int(np.ceil(self.max_active * counts[key] / n)) + 2))
            with torch.cuda.stream(self._stream(0)):
                while len(self.plans[key]) < want and self.ledger.fits(self._pset_bytes(r)):
                    self.plans[key].append(self._build_plan(r, self._stream(0)))
        torch.cuda.synchronize(self.device)

    def submit(self, req: ReconRequest):
        # the power-method start vector is drawn on a host thread while the
        # request waits; admission takes requests whose vector is ready
        req._x0 = self.rng_pool.submit(start_vector, tuple(int(v) for v in req.shape), req.seed)
        self.queue.append(req)

    def _smaps_of(self, req, C, shape):
        """Device coil maps of a request; maps with a ``smaps_key`` stay
        resident for later requests with the same key."""
        if req.smaps_key is not None and self.smaps_cache.get(req.smaps_key) is not None:
            return self.smaps_cache[req.smaps_key]
        t = _array.to_tensor(req.smaps, self.device, torch.complex64).reshape(C, *shape)
        if req.smaps_key is not None:
            self.smaps_cache[req.smaps_key] = t  # charged to the ledger at admission
        return t

    def _build_plan(self, req, stream):
        shape = tuple(int(v) for v in req.shape)
        nbytes = self._pset_bytes(req)
        with torch.cuda.stream(stream):
            plan = NufftPlan(shape, eps=self.eps, ntrans=req.n_coils, device=self.device.index)
            s = proper_trajectory(req.samples, "pi")
            k = _array.to_tensor(s, self.device, torch.float32).reshape(-1, len(shape))
            plan.setpts(k)
            pset = _PlanSet(plan, self.gram, nbytes)
        self.ledger.add_resident(pset.bytes)
        return pset

    def _need(self, req):
        """Bytes that admitting ``req`` adds: (its solver state, its coil maps
        kept resident under their key, a sorted trajectory unless one is
        pooled)."""
        shape = tuple(int(v) for v in req.shape)
        M = int(np.asarray(req.kspace.shape)[-1])
        keep = req.smaps is not None and req.smaps_key is not None and req.smaps_key not in self.smaps_cache
        cached = req.smaps is None or req.smaps_key is not None
        solve = solve_bytes(shape, M, req.n_coils, density=req.density is not None,
                            cached_smaps=cached, gram=self.gram, eps=self.eps)
        smaps_res = smaps_bytes(shape, req.n_coils) if keep else 0
        pset = 0 if self.plans[self._key(req)] else self._pset_bytes(req)
        return solve, smaps_res, pset

    def _evict_for(self, need, keep_key):
        """Free pooled (idle) plan sets of other trajectories, then of the
        request's own, until ``need`` more bytes fit."""
        for own in (False, True):
            for key in list(self.plans):
                if (key == keep_key) != own:
                    continue
                pool = self.plans[key]
                # the request's own pool keeps the plan set its need assumed
                while len(pool) > int(own) and not self.ledger.fits(need):
                    p = pool.pop()
                    self.ledger.drop_resident(p.bytes)
                    del p
                if self.ledger.fits(need):
                    return True
        return self.ledger.fits(need)

    def _admit(self):
        while self.queue and self.free_streams:
            req = self.queue[0]
            if not req._x0.done():
                break
            solve_b, smaps_b, pset_b = self._need(req)
            need = solve_b + smaps_b + pset_b
            if not self.ledger.fits(need) and not self._evict_for(need, self._key(req)):
                if not (self.active or self.finishing):
                    raise RuntimeError(
                        f"request {req.rid} needs {need} device bytes, more than the HBM budget "
                        f"of {int(self.budget)} holds with {self.ledger.resident} resident")
                break
            self.queue.popleft()
            si = self.free_streams.pop()
            stream = self._stream(si)
            key = self._key(req)
            pset = self.plans[key].pop() if self.plans[key] else self._build_plan(req, stream)
            if smaps_b:  # coil maps that stay resident under their key
                self.smaps_cache[req.smaps_key] = None
                self.ledger.add_resident(smaps_b)
            solve = _Solve(self, req, pset, stream, solve_b)
            solve.key, solve.si = key, si
            self.ledger.add_active(solve.bytes)
            req.t_admit = self.now()
            self.active.append(solve)

    def _retire(self):
        still = []
        for s in self.finishing:
            if s.event.query():
                s.req.result = s.image
                s.req.lipschitz = s.L
                s.req.t_done = self.now()
                self.ledger.drop_active(s.bytes)
                self.plans[s.key].append(s.pset)
                self.free_streams.append(s.si)
                self.done.append(s.req)
            else:
                still.append(s)
        self.finishing = still

    def tick(self):
        """Admit, issue one unit of every admitted request, retire finished ones."""
        self._admit()
        running = []
        for s in self.active:
            if s.step():
                running.append(s)
            else:
                self.finishing.append(s)
        self.active = running
        self._retire()

    def idle(self):
        return not (self.queue or self.active or self.finishing)

    def run(self, requests, realtime=True, poll_s=0.0005):
        """Serve ``requests`` (arrival times in seconds from now when
        ``realtime``, else all at once) until every one is done."""
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        self.t0 = time.perf_counter()
        while pending or not self.idle():
            now = self.now()
            while pending and (not realtime or pending[0].arrival <= now):
                self.submit(pending.popleft())
            if self.idle():
                if pending:
                    time.sleep(max(0.0, min(poll_s * 10, pending[0].arrival - now)))
                continue
            self.tick()
            if not self.active:
                time.sleep(poll_s)
        torch.cuda.synchronize(self.device)
        return self.done

    @staticmethod
    def stats(done, wall_s=None):
        lat = np.array([(r.t_done - r.arrival) * 1e3 for r in done])
        t_end = max(r.t_done for r in done)
        t_begin = min(r.arrival for r in done)
        wall = wall_s if wall_s is not None else (t_end - t_begin)
        return {
            "requests": len(done),
            "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()),
            "recon_per_s": len(done) / wall if wall > 0 else float("nan"),
            "wall_s": wall,
        }
