"""The GB300 NUFFT operator: mri-nufft's backend contract on hand-written CUDA.

``MRIGB300`` (backend name ``"gb300"``) implements the operator surface that
mri-nufft callers use (``src/mrinufft/operators/base.py:182-877`` and the
GPU backend ``src/mrinufft/operators/interfaces/cufinufft.py:140-1331``):

* ``op`` / ``adj_op`` / ``data_consistency`` over ``(n_batchs, n_coils)``
  with or without SENSE maps, density compensation and the
  ``1/sqrt(prod(N) 2^d)`` normalisation (base.py:949-1139);
* ``pipe`` density estimation (finufft.py:195-245, cufinufft.py:1281-1331);
* ``get_lipschitz_cst`` (power method, base.py:626-665, 1155-1221) and
  ``pinv_solver`` with the CG solver (extras/optim.py:801-902);
* ``update_samples``, ``smaps`` / ``density`` setters, ``toggle_grad_traj``
  and ``make_autograd``.

Every coil and batch item of a call is handled by one C-ABI call into
``libgbnufft.so`` (no per-coil Python loop); numpy / torch / cupy arrays are
accepted and the result comes back in the caller's array type.
"""

from __future__ import annotations

import logging
import warnings
from contextlib import contextmanager

import numpy as np
import torch

from . import _array
from ._traj import proper_trajectory
from .params import fine_cells
from .plan import NufftPlan, dotu_f64, norm2_f64

logger = logging.getLogger("mrinufft_gb300")

try:  # register in mri-nufft's backend table when it is installed
    from mrinufft.operators.base import FourierOperatorBase as _Base  # type: ignore

    HAVE_MRINUFFT = True
except Exception:  # pragma: no cover - depends on the environment
    from ._base import FourierOperatorBase as _Base

    HAVE_MRINUFFT = False


def _cuda_available() -> bool:
    try:
        return bool(torch.cuda.is_available())
    except Exception:
        return False


DEFAULT_FINE_BUDGET = 4 << 30  # bytes of fine grids per plan


class MRIGB300(_Base):
    """MRI NUFFT operator on GB300 (sm_103a) kernels.

    Parameters follow mri-nufft's finufft / cufinufft backends:

    samples: (M, d) or (..., d) array, in [-0.5, 0.5) or [-pi, pi)
    shape: image shape (2D or 3D)
    density: False | True ("pipe") | array | dict | callable
    n_coils, n_batchs, n_trans: as in mri-nufft (n_trans is kept for
        compatibility; all coils of a call are processed in passes sized by
        the fine-grid memory budget)
    smaps: (n_coils, *shape) coil maps or None
    squeeze_dims: drop singleton batch / coil axes of outputs
    eps, upsampfac: NUFFT accuracy and oversampling
    device: CUDA device ordinal (default: current)
    fine_budget_bytes: bound on fine-grid memory of one plan
    """

    backend = "gb300"
    available = _cuda_available()
    autograd_available = True

    def __init__(
        self,
        samples,
        shape,
        density=False,
        n_coils=1,
        n_batchs=1,
        n_trans=1,
        smaps=None,
        squeeze_dims=True,
        eps=1e-6,
        upsampfac=2.0,
        device=None,
        fine_budget_bytes=DEFAULT_FINE_BUDGET,
        **kwargs,
    ):
        if not self.available:
            raise RuntimeError("'gb300' backend is not available (no CUDA device).")
        super().__init__()
        self.shape = shape
        if len(self.shape) not in (2, 3):
            raise ValueError("the gb300 backend supports 2D and 3D images")
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self.eps = float(eps)
        self.upsampfac = float(upsampfac)
        self.n_batchs = n_batchs
        self.n_coils = n_coils
        self.n_trans = n_trans
        self.squeeze_dims = squeeze_dims
        self._isign = -1
        self._toep = None
        self._toep_unweighted = None
        self._toeplitz_kernel = None
        self.dtype = np.float32
        self._set_samples(samples)
        G = fine_cells(self.shape, self.eps, self.upsampfac)
        cap = max(1, int(fine_budget_bytes // (8 * G)))
        self._ntrans = max(1, min(max(n_batchs * n_coils, n_trans), cap, 64))
        self._plan = NufftPlan(self.shape, self.eps, self.upsampfac, self._ntrans, device=self.device.index)
        self._plan.setpts(self._samples_d)
        self.compute_density(density)
        self.compute_smaps(smaps)

    # ----------------------------------------------------------------- state
    def _set_samples(self, samples, unsafe=False):
        if unsafe:
            s = samples
        else:
            s = proper_trajectory(samples, normalize="pi")
        if s.shape[-1] != len(self.shape):
            raise ValueError(f"samples must have {len(self.shape)} columns")
        t = _array.to_tensor(s, self.device, torch.float32).reshape(-1, len(self.shape))
        self._samples_d = t
        self._samples = np.asfortranarray(t.cpu().numpy())

    @property
    def samples(self):
        return self._samples

    @samples.setter
    def samples(self, new_samples):
        self.update_samples(new_samples)

    @property
    def n_samples(self):
        return self._samples_d.shape[0]

    def update_samples(self, new_samples, *, unsafe=False):
        """Replace the trajectory and re-sort it on the device
        (base.py:809-830, finufft.py:150-181)."""
        self._set_samples(new_samples, unsafe=unsafe)
        self._plan.setpts(self._samples_d)
        self._toep = None
        self._toep_unweighted = None
        self._toeplitz_kernel = None
        self.compute_density(self._density_method)

    @property
    def smaps(self):
        return self._smaps

    @smaps.setter
    def smaps(self, new_smaps):
        if new_smaps is None:
            self._smaps = None
            return
        t = _array.to_tensor(new_smaps, self.device, torch.complex64)
        C = t.shape[0]
        if tuple(t.shape[1:]) != self.shape:
            raise ValueError("Smaps should match image shape.")
        if C != self._n_coils:
            self._n_coils = C
            logger.warning("updating number of coils via Smaps.")
        self._smaps = t.reshape(C, *self.shape)

    def compute_smaps(self, method=None):
        """Set coil maps from an array (numpy, torch or cupy) or a method
        (base.py:407-448)."""
        if method is None:
            self.smaps = None
            return
        if isinstance(method, (np.ndarray, torch.Tensor)) or _array.is_device_array(method):
            self.smaps = method
            return
        if callable(method):
            self.smaps = method(self.samples, self.shape, density=self.density, backend=self.backend)
            return
        kwargs = {}
        if isinstance(method, dict):
            kwargs = dict(method)
            method = kwargs.pop("name")
        from .smaps import METHODS

        if method in METHODS:  # estimated on the device by this package
            fn = METHODS[method]
            kwargs.setdefault("device", self.device.index)
        else:
            try:
                from mrinufft.extras import get_smaps  # type: ignore
            except Exception as e:
                raise ValueError(f"Unknown smaps method: {method}") from e
            fn = get_smaps(method)
        self.smaps = fn(self.samples, self.shape, density=self.density, backend=self.backend, **kwargs)

    @property
    def density(self):
        return self._density

    @density.setter
    def density(self, new_density):
        self._toep = None
        self._toeplitz_kernel = None
        if new_density is None:
            self._density = None
            return
        if len(new_density) != self.n_samples:
            raise ValueError("Density and samples should have the same length")
        if isinstance(new_density, np.ndarray) and np.iscomplexobj(new_density):
            new_density = new_density.real
        t = _array.to_tensor(new_density, self.device, torch.float32 if not (
            isinstance(new_density, torch.Tensor) and new_density.is_complex()) else torch.complex64)
        if t.is_complex():
            t = t.real.contiguous()
        self._density = t.reshape(-1)

    def compute_density(self, method=None):
        """Set density compensation (base.py:576-624); True / "pipe" runs the
        pipe estimate on the GPU."""
        kwargs = {}
        self._toep = None
        self._toeplitz_kernel = None
        if method is None or method is False:
            self._density = None
            return
        if isinstance(method, (np.ndarray, torch.Tensor)) or _array.is_device_array(method):
            self.density = method
            return
        if method is True or method == "pipe":
            fn = type(self).pipe
        elif isinstance(method, dict):
            kwargs = dict(method)
            name = kwargs.pop("name")
            if name == "pipe":
                fn = type(self).pipe
                kwargs.pop("backend", None)
            else:
                fn = self._registry_density(name)
        elif isinstance(method, str):
            fn = self._registry_density(method)
        elif callable(method):
            fn = method
        else:
            raise ValueError(f"Unknown density method: {method}")
        self.density = fn(self._samples_d, self.shape, **kwargs)
        if self._density_method is None:
            self._density_method = {"name": "pipe", **kwargs} if fn == type(self).pipe else method

    @staticmethod
    def _registry_density(name):
        try:
            from mrinufft.density import get_density  # type: ignore
        except Exception as e:
            raise ValueError(f"Unknown density method: {name}") from e
        return get_density(name)

    @property
    def norm_factor(self):
        return np.sqrt(np.prod(self.shape) * 2 ** len(self.shape))

    @property
    def inv_norm_factor(self):
        return 1.0 / self.norm_factor

    @property
    def raw_op(self):
        return self._plan

    @property
    def plan(self) -> NufftPlan:
        return self._plan

    def _safe_squeeze(self, arr):
        if self.squeeze_dims:
            if arr.ndim > 1 and arr.shape[1] == 1:
                arr = arr.squeeze(1)
            if arr.ndim > 0 and arr.shape[0] == 1:
                arr = arr.squeeze(0)
        return arr

    # -------------------------------------------------------------- operators
    def _img_tensor(self, data):
        x = _array.to_tensor(data, self.device, torch.complex64)
        B, C = self.n_batchs, self.n_coils
        if self.uses_sense:
            return x.reshape(B, *self.shape)
        return x.reshape(B * C, *self.shape)

    def _ksp_tensor(self, coeffs):
        x = _array.to_tensor(coeffs, self.device, torch.complex64)
        return x.reshape(self.n_batchs, self.n_coils, self.n_samples)

    def _op_device(self, img: torch.Tensor) -> torch.Tensor:
        """Normalised forward transform of device images -> (B, C, M)."""
        B, C = self.n_batchs, self.n_coils
        out = torch.empty((B, C, self.n_samples), dtype=torch.complex64, device=self.device)
        self._plan.op(img, self._smaps, out, B, C, self.inv_norm_factor, isign=self._isign)
        return out

    def _adj_device(self, ksp: torch.Tensor, density=True) -> torch.Tensor:
        B, C = self.n_batchs, self.n_coils
        shape = (B, 1, *self.shape) if self.uses_sense else (B, C, *self.shape)
        out = torch.empty(shape, dtype=torch.complex64, device=self.device)
        self._plan.adj(ksp, self._density if density else None, self._smaps, out, B, C,
                       self.inv_norm_factor, isign=-self._isign)
        return out

    def op(self, data, ksp=None):
        r"""Forward operator: for every batch b and coil l, :math:`F S_l x_b`."""
        self.check_shape(image=data, ksp=ksp)
        like = _array.interface_of(data)
        if like.kind == "numpy" and ksp is None and self._host_groups() > 1:
            return self._safe_squeeze(self._op_host(data))
        ret = self._safe_squeeze(self._op_device(self._img_tensor(data)))
        return self._emit(ret, like, ksp)

    def adj_op(self, coeffs, img=None):
        """Adjoint operator (density compensated when density is set)."""
        self.check_shape(image=img, ksp=coeffs)
        like = _array.interface_of(coeffs)
        ret = self._safe_squeeze(self._adj_device(self._ksp_tensor(coeffs)))
        return self._emit(ret, like, img)

    # --------------------------------------------- host arrays, overlapped
    # Host (numpy) k-space of many coils is large (16 coils x 2.1 M samples
    # = 268 MB).  op of a numpy image transforms the coils in groups and
    # copies each group's k-space into the page-locked result on a copy
    # stream while the GPU works on the next group (3D kooshball, 16 coils:
    # 7.6 against 8.1 ms per call).  adj_op makes one call over all coils:
    # its kernels need the k-space before they start, and group calls would
    # cost more than the copy they hide (2.2 ms per 4-coil group against
    # 2.0 ms per pass of one call, whose kernels stage each sample's geometry
    # once for every coil).
    HOST_OVERLAP_BYTES = 32 << 20

    def _host_groups(self):
        C = self.n_coils
        if (not _array.PINNED_RESULTS or C < 2
                or 8 * C * self.n_samples * self.n_batchs < self.HOST_OVERLAP_BYTES):
            return 1
        return min(4, C)

    def _copy_stream(self):
        if getattr(self, "_copy_st", None) is None:
            self._copy_st = torch.cuda.Stream(self.device)
        return self._copy_st

    def _coil_groups(self):
        C, n = self.n_coils, self._host_groups()
        step = -(-C // n)
        return [(c0, min(C, c0 + step)) for c0 in range(0, C, step)]

    def _op_host(self, data):
        """op of a numpy image: groups of coils, the device-to-host copy of a
        group's k-space overlapping the next group's transforms."""
        B, C, M = self.n_batchs, self.n_coils, self.n_samples
        out = _array.pinned_empty((B, C, M), torch.complex64)
        if out is None:  # the host cannot lock that much memory: one call, pageable copy
            return _array.from_tensor(self._op_device(self._img_tensor(data)), _array.Interface("numpy"))
        x = self._img_tensor(data)
        dev_k = torch.empty((B, C, M), dtype=torch.complex64, device=self.device)
        main = torch.cuda.current_stream(self.device)
        side = self._copy_stream()
        for b in range(B):
            for c0, c1 in self._coil_groups():
                if self.uses_sense:
                    img, sm = x[b:b + 1], self._smaps[c0:c1]
                else:
                    img, sm = x[b * C + c0:b * C + c1], None
                self._plan.op(img, sm, dev_k[b, c0:c1], 1, c1 - c0, self.inv_norm_factor,
                              isign=self._isign)
                side.wait_stream(main)
                with torch.cuda.stream(side):
                    out[b, c0:c1].copy_(dev_k[b, c0:c1], non_blocking=True)
        side.synchronize()
        return out.numpy()

    def _op(self, image, coeffs):
        """Unnormalised type-2 transforms of an (n, *shape) image stack."""
        x = _array.to_tensor(image, self.device, torch.complex64).reshape(-1, *self.shape)
        out = torch.empty((x.shape[0], self.n_samples), dtype=torch.complex64, device=self.device)
        self._plan.op(x, None, out, 1, x.shape[0], 1.0, isign=self._isign)
        return self._emit(out, _array.interface_of(image), coeffs)

    def _adj_op(self, coeffs, image):
        """Unnormalised, density-compensated type-1 transforms (base.py:1068-1073)."""
        y = _array.to_tensor(coeffs, self.device, torch.complex64).reshape(-1, self.n_samples)
        out = torch.empty((y.shape[0], *self.shape), dtype=torch.complex64, device=self.device)
        self._plan.adj(y, self._density, None, out, 1, y.shape[0], 1.0, isign=-self._isign)
        return self._emit(out, _array.interface_of(coeffs), image)

    def _emit(self, ret, like, out_buf=None):
        if out_buf is not None:
            if isinstance(out_buf, torch.Tensor):
                out_buf.copy_(ret.reshape(out_buf.shape))
                return out_buf
            if isinstance(out_buf, np.ndarray):
                np.copyto(out_buf, ret.reshape(out_buf.shape).cpu().numpy())
                return out_buf
        return _array.from_tensor(ret, like)

    def data_consistency(self, image_data, obs_data):
        """Gradient of the data-consistency term A^H(Ax - y), fused per pass."""
        like = _array.interface_of(image_data)
        x = self._img_tensor(image_data)
        y = self._ksp_tensor(obs_data)
        out = torch.empty(self.img_full_shape, dtype=torch.complex64, device=self.device)
        B, C = self.n_batchs, self.n_coils
        self._plan.dc(x, y, self._density, self._smaps, out, B, C, self.inv_norm_factor)
        return _array.from_tensor(self._safe_squeeze(out), like)

    def gram_op(self, data, toeplitz=True):
        """Gram operator A^H W A x (base.py:315-363).  ``toeplitz=True`` uses
        the Toeplitz embedding (FFTs and one multiply per coil, no
        spreading or interpolation); ``toeplitz=False`` one forward and one
        adjoint transform."""
        self.check_shape(image=data)
        if not toeplitz:
            return self.adj_op(self.op(data))
        like = _array.interface_of(data)
        x = self._img_tensor(data)
        out = self._gram_device(x)
        return _array.from_tensor(self._safe_squeeze(out), like)

    def _gram_device(self, x: torch.Tensor) -> torch.Tensor:
        """Toeplitz Gram of device images ((B, *N) SENSE or (B*C, *N))."""
        B, C = self.n_batchs, self.n_coils
        out = torch.empty(self.img_full_shape, dtype=torch.complex64, device=self.device)
        self._toeplitz().apply(x, self._smaps, out, B, C, self.inv_norm_factor ** 2)
        return out

    def _toeplitz(self):
        if self._toep is None:
            from .plan import ToeplitzKernel

            self._toep = ToeplitzKernel(self._plan, self._density)
            self._toep_weighted = self._density is not None
        return self._toep

    def compute_toeplitz_kernel(self):
        """Compute and set the Toeplitz kernel (base.py:444-449,
        toeplitz.py:35-96): the real spectrum of A^H W A on the circulant grid
        (shape 2N where 2N is 2-3-5 smooth), W the density (ones when unset),
        scaled by 1/norm_factor^2 as in the reference.  Returned as a numpy
        array."""
        self._toep = None
        k = self._toeplitz().kernel() * float(self.inv_norm_factor ** 2)
        self._toeplitz_kernel = k.cpu().numpy()
        return self._toeplitz_kernel

    # ------------------------------------------------------------ gradients
    def toggle_grad_traj(self):
        """Switch to the isign=+1 plan with conjugated maps and back
        (base.py:1224-1238, finufft.py:183-193)."""
        if self.uses_sense:
            self._smaps = self._smaps.conj().resolve_conj()
        self._isign = -self._isign

    @contextmanager
    def grad_traj_plan(self):
        self.toggle_grad_traj()
        try:
            yield
        finally:
            self.toggle_grad_traj()

    def _make_plan_grad(self, **kwargs):
        """Gradient plans share the forward plan; isign is a call argument."""

    def with_off_resonance_correction(self, readout_time, b0_map=None, r2star_map=None, mask=None,
                                      interpolator="svd"):
        """Off-resonance corrected operator around this one (base.py:385-398)."""
        from .offres import MRIFourierCorrectedGB300

        return MRIFourierCorrectedGB300(self, b0_map, readout_time, r2star_map, mask, interpolator)

    def make_autograd(self, *, wrt_data=True, wrt_traj=False, paired_batch=False):
        from .autodiff import MRINufftAutoGrad

        return MRINufftAutoGrad(self, wrt_data=wrt_data, wrt_traj=wrt_traj, paired_batch=paired_batch)

    # ------------------------------------------------------------- solvers
    def get_lipschitz_cst(self, max_iter=10, toeplitz=False, **kwargs):
        """Largest eigenvalue of A^H A (single coil, no maps, with density)
        by the power method of base.py:1155-1221 with FP64 norms, from the
        GPU backends' start vector (cufinufft.py:1239-1279).  ``toeplitz``
        (an option of this backend) applies A^H W A through the Toeplitz
        embedding."""
        x = 1j * np.random.random(self.shape).astype(np.complex64)
        x += np.random.random(self.shape).astype(np.complex64)
        x = torch.from_numpy(x).to(self.device)
        return power_method(max_iter, self, x, toeplitz=toeplitz)

    def _unweighted_toeplitz(self):
        """Toeplitz embedding of A^H A without density (CG iterations run
        with density disabled, extras/optim.py:838-842)."""
        if self._toep is not None and not self._toep_weighted:
            return self._toep
        if self._toep_unweighted is None:
            from .plan import ToeplitzKernel

            self._toep_unweighted = ToeplitzKernel(self._plan, None)
        return self._toep_unweighted

    def pinv_solver(self, kspace_data, optim="lsqr", **kwargs):
        """Least-squares reconstruction (base.py:667-690).  ``optim="lsqr"``
        (the default) and ``optim="cg"`` run the device solvers of
        :mod:`mrinufft_gb300.optim`; other solvers come from mri-nufft when
        it is installed."""
        if optim in ("cg", "lsqr"):
            from . import optim as _optim

            return getattr(_optim, optim)(self, kspace_data, **kwargs)
        try:
            from mrinufft.extras import get_optimizer  # type: ignore
        except Exception as e:
            raise ValueError(f"optimizer {optim!r} needs mri-nufft installed") from e
        return get_optimizer(optim)(operator=self, kspace_data=kspace_data, **kwargs)

    @classmethod
    def pipe(cls, kspace_loc, volume_shape, max_iter=10, osf=2, normalize=True, **kwargs):
        """Pipe density compensation (finufft.py:195-245): ``max_iter``
        iterations of w <- w / |interp(spread(w))| on the image-size grid with
        the kernel of oversampling ``osf``, then normalisation so that the
        density-weighted PSF of a full NUFFT has unit mean."""
        device = kwargs.pop("device", None)
        eps = kwargs.get("eps", 1e-6)
        like = _array.interface_of(kspace_loc)
        volume_shape = tuple(int(v) for v in volume_shape)
        dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        s = proper_trajectory(kspace_loc, normalize="pi")
        s = _array.to_tensor(s, dev, torch.float32).reshape(-1, len(volume_shape))
        grid = NufftPlan(volume_shape, eps=eps, upsampfac=float(osf), ntrans=1, spread_only=True,
                         device=dev.index)
        grid.setpts(s)
        w = torch.ones(s.shape[0], dtype=torch.complex64, device=dev)
        nf = np.sqrt(np.prod(volume_shape) * 2 ** len(volume_shape))
        grid.pipe(w, max_iter, 1.0 / (nf * nf))
        if normalize:
            test_op = cls(samples=s, shape=volume_shape, device=dev.index, **kwargs)
            test_im = torch.ones(volume_shape, dtype=torch.complex64, device=dev)
            recon = test_op.adj_op(w * test_op.op(test_im))
            w = w / torch.mean(torch.abs(recon))
        out = torch.abs(w).reshape(-1)
        if like.kind == "numpy":
            return out.cpu().numpy()
        return _array.from_tensor(out, like)

    def __repr__(self):
        return (
            "MRIGB300(\n"
            f"  shape: {self.shape}\n"
            f"  n_coils: {self.n_coils}\n"
            f"  n_samples: {self.n_samples}\n"
            f"  n_batchs: {self.n_batchs}\n"
            f"  uses_density: {self.uses_density}\n"
            f"  uses_sense: {self.uses_sense}\n"
            f"  eps: {self.eps:.0e}\n"
            ")"
        )


def power_method(max_iter, operator: MRIGB300, x: torch.Tensor, toeplitz=False):
    """Power iteration for the Lipschitz constant on the device, restating
    ``operators/base.py:1155-1221`` on a single-coil, map-free copy of the
    operator configuration (base.py:647-665).  Returns a host float."""
    B, C, smaps, sq = operator.n_batchs, operator.n_coils, operator._smaps, operator.squeeze_dims
    operator._smaps = None
    operator._n_coils = 1
    operator._n_batchs = 1
    operator.squeeze_dims = True
    try:
        x = x.reshape(1, *operator.shape).to(torch.complex64).contiguous()
        x_norm = float(norm2_f64(x).sqrt())
        x = x / x_norm
        x_new_norm = x_norm
        i = 0
        for i in range(max_iter):  # noqa: B007
            if toeplitz:
                x_new = operator._gram_device(x).reshape(1, *operator.shape)
            else:
                x_new = operator._adj_device(operator._op_device(x)).reshape(1, *operator.shape)
            x_new_norm = float(norm2_f64(x_new).sqrt())
            x_new = x_new / x_new_norm
            if abs(x_norm - x_new_norm) < 1e-6:
                break
            x_norm = x_new_norm
            x = x_new
        if i == max_iter - 1:
            warnings.warn("Lipschitz constant did not converge")
        return x_new_norm
    finally:
        operator._smaps = smaps
        operator._n_coils = C
        operator._n_batchs = B
        operator.squeeze_dims = sq
