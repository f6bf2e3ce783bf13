"""Python handle of one GB300 NUFFT plan (``gbn_plan`` of ``include/gbnufft.h``).

Plays the role of mri-nufft's raw plan layer (``RawFinufftPlan``,
``src/mrinufft/operators/interfaces/finufft.py:23-80``; ``RawCufinufftPlan``,
``src/mrinufft/operators/interfaces/cufinufft.py:51-137``): it owns the
device-side state of one trajectory (bin-sorted points, fine grids, cuFFT
plans) and forwards every call to the C ABI on torch's current CUDA stream.
Arguments are torch CUDA tensors; only their raw pointers cross the ABI.
"""

from __future__ import annotations

import ctypes

import torch

from . import _lib


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


class NufftPlan:
    """A plan for 2D / 3D type-1 and type-2 transforms of one image shape."""

    def __init__(self, shape, eps=1e-6, upsampfac=2.0, ntrans=1, spread_only=False, device=None):
        self.shape = tuple(int(s) for s in shape)
        self.ndim = len(self.shape)
        if self.ndim not in (2, 3):
            raise ValueError("the GB300 backend supports 2D and 3D images")
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.eps = float(eps)
        self.upsampfac = float(upsampfac)
        self.ntrans = int(ntrans)
        self.spread_only = bool(spread_only)
        self._h = ctypes.c_void_p()
        self.lib = _lib.load()
        dims = (ctypes.c_int64 * self.ndim)(*self.shape)
        _lib.check(
            self.lib.gbn_plan_create(
                self.ndim, dims, self.upsampfac, self.eps, self.ntrans,
                int(self.spread_only), self.device.index, ctypes.byref(self._h)
            ),
            "gbn_plan_create",
        )
        self._coords = None
        self.n_samples = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self.lib.gbn_plan_destroy(h)
            except Exception:  # interpreter shutdown
                pass
            self._h = None

    @property
    def stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    # ------------------------------------------------------------------ info
    def info(self):
        w = ctypes.c_int()
        beta = ctypes.c_double()
        nf = (ctypes.c_int64 * 3)()
        bins = (ctypes.c_int * 3)()
        _lib.check(self.lib.gbn_plan_info(self._h, ctypes.byref(w), ctypes.byref(beta), nf, bins),
                   "gbn_plan_info")
        return {
            "width": w.value,
            "beta": beta.value,
            "nf": tuple(nf[: self.ndim]),
            "bins": tuple(bins[: self.ndim]),
        }

    @property
    def device_bytes(self) -> int:
        b = ctypes.c_int64()
        _lib.check(self.lib.gbn_plan_device_bytes(self._h, ctypes.byref(b)), "gbn_plan_device_bytes")
        return b.value

    # ---------------------------------------------------------------- tuning
    # "auto": the default kernel of the dimension (2D: warp-cooperative direct,
    # 3D: shared-memory tiles)
    METHODS = {"auto": 0, "direct": 1, "double_buffered": 3, "warp_direct": 4, "warp_tile": 5}

    def tune(self, bins=None, interp=None, maxsub_cap=0):
        """Set bin sizes (fine cells per axis), interpolation method and the
        largest subproblem; points must be set again afterwards."""
        b = None if bins is None else (ctypes.c_int * self.ndim)(*[int(v) for v in bins])
        m = -1 if interp is None else self.METHODS[interp]
        _lib.check(self.lib.gbn_plan_tune(self._h, b, m, int(maxsub_cap)), "gbn_plan_tune")
        if self._coords is not None and (bins is not None or maxsub_cap):
            self._reset_points()

    def _reset_points(self):
        cols = self._coords
        M = self.n_samples
        _lib.check(
            self.lib.gbn_setpts(self._h, M, _ptr(cols[0]), _ptr(cols[1]), _ptr(cols[2]), self.stream),
            "gbn_setpts",
        )

    # ------------------------------------------------------------- profiling
    def profile(self, enable: bool = True):
        """Start (clear) or stop per-stage CUDA-event timing."""
        _lib.check(self.lib.gbn_profile(self._h, int(enable)), "gbn_profile")

    def profile_read(self, stage: str | None = None):
        """(device ms, launches) of a stage, or of all stages and the number of
        this library's kernel launches when ``stage`` is None."""
        ms = ctypes.c_double()
        n = ctypes.c_int64()
        idx = -1 if stage is None else _lib.STAGES[stage]
        _lib.check(self.lib.gbn_profile_read(self._h, idx, ctypes.byref(ms), ctypes.byref(n)),
                   "gbn_profile_read")
        return ms.value, n.value

    # ---------------------------------------------------------------- points
    def setpts(self, samples: torch.Tensor):
        """Set the (M, d) float32 CUDA sample coordinates in radians."""
        if samples.ndim != 2 or samples.shape[1] != self.ndim:
            raise ValueError(f"samples must have shape (M, {self.ndim})")
        cols = [samples[:, d].to(self.device, torch.float32).contiguous() for d in range(self.ndim)]
        while len(cols) < 3:
            cols.append(None)
        M = samples.shape[0]
        _lib.check(
            self.lib.gbn_setpts(self._h, M, _ptr(cols[0]), _ptr(cols[1]), _ptr(cols[2]), self.stream),
            "gbn_setpts",
        )
        self._coords = cols
        self.n_samples = M

    # ------------------------------------------------------------ transforms
    def op(self, img, smaps, out, n_batchs, n_coils, scale, isign=-1):
        _lib.check(
            self.lib.gbn_op(self._h, _ptr(img), _ptr(smaps), _ptr(out), n_batchs, n_coils,
                            float(scale), int(isign), self.stream),
            "gbn_op",
        )
        return out

    def adj(self, ksp, density, smaps, out, n_batchs, n_coils, scale, isign=1):
        _lib.check(
            self.lib.gbn_adj(self._h, _ptr(ksp), _ptr(density), _ptr(smaps), _ptr(out), n_batchs,
                             n_coils, float(scale), int(isign), self.stream),
            "gbn_adj",
        )
        return out

    def dc(self, img, obs, density, smaps, out, n_batchs, n_coils, scale):
        _lib.check(
            self.lib.gbn_dc(self._h, _ptr(img), _ptr(obs), _ptr(density), _ptr(smaps), _ptr(out),
                            n_batchs, n_coils, float(scale), self.stream),
            "gbn_dc",
        )
        return out

    def pipe(self, w, iters, scale2):
        _lib.check(self.lib.gbn_pipe(self._h, _ptr(w), int(iters), float(scale2), self.stream),
                   "gbn_pipe")
        return w

    def grad_traj_op(self, img, smaps, dy, grad, n_batchs, n_coils, scale):
        _lib.check(
            self.lib.gbn_grad_traj_op(self._h, _ptr(img), _ptr(smaps), _ptr(dy), _ptr(grad),
                                      n_batchs, n_coils, float(scale), self.stream),
            "gbn_grad_traj_op",
        )
        return grad

    def grad_traj_adj(self, dx, smaps, y, grad, n_batchs, n_coils, scale):
        _lib.check(
            self.lib.gbn_grad_traj_adj(self._h, _ptr(dx), _ptr(smaps), _ptr(y), _ptr(grad),
                                       n_batchs, n_coils, float(scale), self.stream),
            "gbn_grad_traj_adj",
        )
        return grad


class ToeplitzKernel:
    """Toeplitz embedding of a plan's Gram operator A^H W A (``gbn_toep``).

    Restates mri-nufft's ``compute_toeplitz_kernel`` / ``apply_toeplitz_kernel``
    (``src/mrinufft/operators/toeplitz.py:35-96, 193-269``): the real kernel
    spectrum on a circulant grid of nf >= 2N cells per axis, applied as
    zero-pad -> FFT -> multiply -> inverse FFT -> crop for every coil of a call.
    ``weights`` (M,) float32 CUDA tensor or None (ones).
    """

    def __init__(self, plan: NufftPlan, weights: torch.Tensor | None = None):
        if plan._coords is None:
            raise ValueError("the plan has no points")
        self.plan = plan
        self.lib = plan.lib
        self.device = plan.device
        self._h = ctypes.c_void_p()
        cols = plan._coords
        w = None if weights is None else weights.to(self.device, torch.float32).contiguous()
        _lib.check(
            self.lib.gbn_toep_create(plan._h, plan.n_samples, _ptr(cols[0]), _ptr(cols[1]),
                                     _ptr(cols[2]), _ptr(w), ctypes.byref(self._h), plan.stream),
            "gbn_toep_create",
        )
        nf = (ctypes.c_int64 * 3)()
        _lib.check(self.lib.gbn_toep_info(self._h, nf), "gbn_toep_info")
        self.grid = tuple(int(v) for v in nf[: plan.ndim])

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self.lib.gbn_toep_destroy(h)
            except Exception:  # interpreter shutdown
                pass
            self._h = None

    def profile(self, enable: bool = True):
        """Stage timing of the circulant-grid plan (see NufftPlan.profile)."""
        _lib.check(self.lib.gbn_profile(self._inner(), int(enable)), "gbn_profile")

    def profile_read(self, stage: str | None = None):
        ms = ctypes.c_double()
        n = ctypes.c_int64()
        idx = -1 if stage is None else _lib.STAGES[stage]
        _lib.check(self.lib.gbn_profile_read(self._inner(), idx, ctypes.byref(ms), ctypes.byref(n)),
                   "gbn_profile_read")
        return ms.value, n.value

    def _inner(self):
        h = ctypes.c_void_p()
        _lib.check(self.lib.gbn_toep_plan(self._h, ctypes.byref(h)), "gbn_toep_plan")
        return h

    def inner_device_bytes(self) -> int:
        """Device bytes of the embedding (circulant grids and kernel spectrum)."""
        b = ctypes.c_int64()
        _lib.check(self.lib.gbn_plan_device_bytes(self._inner(), ctypes.byref(b)),
                   "gbn_plan_device_bytes")
        return b.value

    def kernel(self) -> torch.Tensor:
        """The real kernel spectrum, shape ``grid`` (device, float32)."""
        out = torch.empty(self.grid, dtype=torch.float32, device=self.device)
        _lib.check(self.lib.gbn_toep_kernel(self._h, _ptr(out), self.plan.stream), "gbn_toep_kernel")
        return out

    def apply(self, img, smaps, out, n_batchs, n_coils, scale):
        _lib.check(
            self.lib.gbn_toep_apply(self._h, _ptr(img), _ptr(smaps), _ptr(out), n_batchs, n_coils,
                                    float(scale), self.plan.stream),
            "gbn_toep_apply",
        )
        return out

    def cg_iter(self, image, smaps, rhs, grad, grad_new, velocity, state, lipschitz, n_batchs,
                n_coils, scale, tol, stream=None):
        """One CG iteration with the gradient A^H A x - rhs (``gbn_toep_cg_iter``);
        ``stream``: a ctypes stream handle (default: torch's current stream)."""
        _lib.check(
            self.lib.gbn_toep_cg_iter(self._h, _ptr(image), _ptr(smaps), _ptr(rhs), _ptr(grad),
                                      _ptr(grad_new), _ptr(velocity), _ptr(state), _ptr(lipschitz),
                                      n_batchs, n_coils, float(scale), float(tol),
                                      self.plan.stream if stream is None else stream),
            "gbn_toep_cg_iter",
        )

    def power_iter(self, x, x_new, state, lipschitz, scale, stream=None):
        """One power-method iteration on A^H W A (``gbn_toep_power_iter``)."""
        _lib.check(
            self.lib.gbn_toep_power_iter(self._h, _ptr(x), _ptr(x_new), _ptr(state), _ptr(lipschitz),
                                         float(scale), self.plan.stream if stream is None else stream),
            "gbn_toep_power_iter",
        )


def norm2_f64(x: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """sum |x|^2 accumulated in FP64 on the device (returns a 1-element float64 tensor)."""
    if out is None:
        out = torch.empty(1, dtype=torch.float64, device=x.device)
    x = x.contiguous()
    _lib.check(
        _lib.load().gbn_norm2_f64(_ptr(x), x.numel(), _ptr(out),
                                  ctypes.c_void_p(torch.cuda.current_stream(x.device).cuda_stream)),
        "gbn_norm2_f64",
    )
    return out


def dotu_f64(a: torch.Tensor, b: torch.Tensor, conj_a=False, out: torch.Tensor | None = None):
    """sum a*b (numpy.dot semantics for complex) in FP64 -> 2-element float64 tensor (re, im)."""
    if out is None:
        out = torch.empty(2, dtype=torch.float64, device=a.device)
    a = a.contiguous()
    b = b.contiguous()
    if a.numel() != b.numel():
        raise ValueError("dot of vectors of different sizes")
    _lib.check(
        _lib.load().gbn_dotu_f64(_ptr(a), _ptr(b), a.numel(), int(conj_a), _ptr(out),
                                 ctypes.c_void_p(torch.cuda.current_stream(a.device).cuda_stream)),
        "gbn_dotu_f64",
    )
    return out
