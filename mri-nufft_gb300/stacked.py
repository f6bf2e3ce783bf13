"""Stacked NUFFT on the GB300 library (stack-of-stars / stack-of-spirals).

Restates mri-nufft's ``MRIStackedNUFFT`` / ``MRIStackedNUFFTGPU``
(``src/mrinufft/operators/stacked.py:36-837``): a 2D trajectory repeated on
the ``z_index`` planes of a 3D image whose last axis is Cartesian.  The
forward operator is, per coil, a centred orthonormal DFT along z divided by
sqrt(2) (stacked.py:178-194) followed by a 2D NUFFT of every kept plane; the
adjoint scatters the planes back, inverts the DFT and combines the coils.

Every call is two C-ABI calls per batch item: ``gbn_stack_fwd`` /
``gbn_stack_adj`` (fused SENSE multiply, z shift, cuFFT along z, plane
gather / scatter, coil combine) and one 2D ``gbn_op`` / ``gbn_adj`` over
all ``n_coils * len(z_index)`` planes.  Backend name ``"stacked-gb300"``.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _array, _lib
from ._traj import proper_trajectory
from .operator import MRIGB300, _Base, _cuda_available
from .plan import _ptr


def traj3d2stacked(samples, dim_z, n_samples=0):
    """3D stacked trajectory -> (2D trajectory, z_index) (stacked.py:840-869):
    the distinct z values in order of appearance, ``n_samples`` samples per
    plane (default: all samples / number of planes), z mapped to the plane
    index ``int32(z * dim_z + dim_z // 2)`` with z in [-0.5, 0.5)."""
    samples = np.asarray(samples).reshape(-1, 3)
    z_kspace, idx = np.unique(samples[:, 2], return_index=True)
    z_kspace = z_kspace[np.argsort(idx)]
    if n_samples == 0:
        n_samples = int(np.prod(samples.shape[:-1])) // len(z_kspace)
    traj2d = samples[:n_samples, :2]
    z_kspace = np.asarray(proper_trajectory(z_kspace.reshape(-1, 1), "unit")).flatten()
    z_index = np.int32(z_kspace * dim_z + dim_z // 2)
    return traj2d, z_index


def stacked2traj3d(samples2d, z_indexes, dim_z):
    """2D trajectory and plane indices -> flattened 3D trajectory
    (stacked.py:872-902)."""
    z_kspace = (np.asarray(z_indexes) - dim_z // 2) / dim_z
    locs = np.asarray(proper_trajectory(samples2d, normalize="unit"))
    out = np.zeros((len(z_kspace), len(locs), 3), dtype=locs.dtype)
    for i, z in enumerate(z_kspace):
        out[i, :, :2] = locs
        out[i, :, 2] = z
    return out


class MRIStackedGB300(_Base):
    """Stacked NUFFT operator on GB300 kernels.

    Parameters follow ``MRIStackedNUFFTGPU``: ``samples`` (2D with
    ``z_index``, or 3D with ``z_index="auto"``), ``shape`` (nx, ny, nz),
    ``smaps``, ``n_coils``, ``n_batchs``, ``z_index`` (``"auto"``, a boolean
    mask or integer indices of the kept planes, ``None`` for all),
    ``squeeze_dims``, ``density`` (of the 2D trajectory) and the 2D NUFFT's
    ``eps`` / ``upsampfac``.
    """

    backend = "stacked-gb300"
    available = _cuda_available()
    autograd_available = False

    def __init__(self, samples, shape, smaps=None, n_coils=1, n_batchs=1, n_trans=1,
                 z_index="auto", squeeze_dims=False, density=False, device=None, **kwargs):
        if not self.available:
            raise RuntimeError("'stacked-gb300' backend is not available (no CUDA device).")
        super().__init__()
        self.shape = shape
        if len(self.shape) != 3:
            raise ValueError("the stacked operator needs a 3D image shape")
        self.n_coils = n_coils
        self.n_batchs = n_batchs
        self.n_trans = n_trans
        self.squeeze_dims = squeeze_dims
        self.dtype = np.float32
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        samples2d, zi = self._init_samples(samples, z_index, self.shape)
        self._samples2d = np.asarray(samples2d).reshape(-1, 2)
        self.z_index = np.asarray(zi, dtype=np.int64)
        self.operator = MRIGB300(self._samples2d, self.shape[:2], n_coils=self.n_coils * len(self.z_index),
                                 smaps=None, squeeze_dims=True, density=density, device=self.device.index,
                                 **kwargs)
        self._stack = ctypes.c_void_p()
        self.lib = _lib.load()
        dims = (ctypes.c_int64 * 3)(*self.shape)
        zarr = (ctypes.c_int * len(self.z_index))(*[int(v) for v in self.z_index])
        _lib.check(self.lib.gbn_stack_create(dims, zarr, len(self.z_index), self.device.index,
                                             ctypes.byref(self._stack)), "gbn_stack_create")
        self.smaps = smaps

    def __del__(self):
        h = getattr(self, "_stack", None)
        if h is not None and h.value:
            try:
                self.lib.gbn_stack_destroy(h)
            except Exception:  # interpreter shutdown
                pass
            self._stack = None

    @staticmethod
    def _init_samples(samples, z_index, shape):
        samples_dim = np.asarray(samples).shape[-1]
        auto_z = isinstance(z_index, str) and z_index == "auto"
        if samples_dim == 3 and auto_z:
            return traj3d2stacked(samples, shape[-1])
        if samples_dim == 2 and not auto_z:
            if z_index is None:
                z_index = np.ones(shape[-1], dtype=bool)
            try:
                zi = np.arange(shape[-1])[z_index]
            except IndexError as e:
                raise ValueError("z-index should be a boolean array of length shape[-1], "
                                 "or an array of integer.") from e
            return samples, zi
        raise ValueError("Invalid samples or z-index")

    # ------------------------------------------------------------------ state
    @property
    def smaps(self):
        return self._smaps

    @smaps.setter
    def smaps(self, new_smaps):
        if new_smaps is None:
            self._smaps = None
            return
        t = _array.to_tensor(new_smaps, self.device, torch.complex64)
        if tuple(t.shape[1:]) != self.shape:
            raise ValueError("Smaps should match image shape.")
        self._smaps = t.reshape(-1, *self.shape).contiguous()
        self.n_coils = self._smaps.shape[0]

    @property
    def density(self):
        return self.operator.density

    @property
    def n_samples(self):
        return len(self._samples2d) * len(self.z_index)

    @property
    def samples(self):
        """(n_planes, n_samples2d, 3) samples with z in [-0.5, 0.5) (stacked.py:442-465)."""
        out = np.zeros((len(self.z_index), len(self._samples2d), 3), dtype=self._samples2d.dtype)
        for i, idx in enumerate(self.z_index):
            out[i, :, :2] = self._samples2d
            out[i, :, 2] = idx / self.shape[-1] - 0.5
        return out

    @property
    def norm_factor(self):
        return np.sqrt(np.prod(self.shape) * 2 ** 3)

    def _st(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    # ------------------------------------------------------------- operators
    def _op_device(self, x: torch.Tensor) -> torch.Tensor:
        B, C, NZ, NS = self.n_batchs, self.n_coils, len(self.z_index), len(self._samples2d)
        sense = self._smaps is not None
        x = x.reshape((B, *self.shape) if sense else (B, C, *self.shape))
        planes = torch.empty((C * NZ, *self.shape[:2]), dtype=torch.complex64, device=self.device)
        out = torch.empty((B, C * NZ, NS), dtype=torch.complex64, device=self.device)
        op2 = self.operator
        for b in range(B):
            _lib.check(self.lib.gbn_stack_fwd(self._stack, _ptr(x[b]), _ptr(self._smaps), _ptr(planes),
                                              C, self._st()), "gbn_stack_fwd")
            op2._plan.op(planes, None, out[b], 1, C * NZ, op2.inv_norm_factor, isign=op2._isign)
        return out.reshape(B, C, NZ * NS)

    def _adj_device(self, ksp: torch.Tensor, density=True) -> torch.Tensor:
        B, C, NZ, NS = self.n_batchs, self.n_coils, len(self.z_index), len(self._samples2d)
        sense = self._smaps is not None
        ksp = ksp.reshape(B, C * NZ, NS)
        planes = torch.empty((C * NZ, *self.shape[:2]), dtype=torch.complex64, device=self.device)
        out = torch.empty((B, *self.shape) if sense else (B, C, *self.shape), dtype=torch.complex64,
                          device=self.device)
        op2 = self.operator
        dens = op2._density if density else None
        for b in range(B):
            op2._plan.adj(ksp[b], dens, None, planes, 1, C * NZ, op2.inv_norm_factor,
                          isign=-op2._isign)
            _lib.check(self.lib.gbn_stack_adj(self._stack, _ptr(planes), _ptr(self._smaps), _ptr(out[b]),
                                              C, 0, self._st()), "gbn_stack_adj")
        return out

    def op(self, data, ksp=None):
        """Forward operator: (B, *shape) with maps or (B, C, *shape) -> (B, C, NZ * NS)."""
        self.check_shape(image=data, ksp=ksp)
        like = _array.interface_of(data)
        x = _array.to_tensor(data, self.device, torch.complex64)
        ret = self._safe_squeeze(self._op_device(x))
        return self._emit(ret, like, ksp)

    def adj_op(self, coeffs, img=None):
        """Adjoint operator (density compensated when the 2D operator has density)."""
        self.check_shape(image=img, ksp=coeffs)
        like = _array.interface_of(coeffs)
        y = _array.to_tensor(coeffs, self.device, torch.complex64)
        ret = self._safe_squeeze(self._adj_device(y))
        return self._emit(ret, like, img)

    def data_consistency(self, image_data, obs_data):
        """A^H (A x - y) (base.py:1075-1085)."""
        like = _array.interface_of(image_data)
        x = _array.to_tensor(image_data, self.device, torch.complex64)
        y = _array.to_tensor(obs_data, self.device, torch.complex64).reshape(self.n_batchs, self.n_coils, -1)
        r = self._op_device(x) - y
        return _array.from_tensor(self._safe_squeeze(self._adj_device(r)), like)

    def get_lipschitz_cst(self, max_iter=10):
        """The 2D operator's Lipschitz constant, as the reference (stacked.py:418-438)."""
        return self.operator.get_lipschitz_cst(max_iter)

    def _emit(self, ret, like, out_buf=None):
        if out_buf is not None:
            if isinstance(out_buf, torch.Tensor):
                out_buf.copy_(ret.reshape(out_buf.shape))
                return out_buf
            if isinstance(out_buf, np.ndarray):
                np.copyto(out_buf, ret.reshape(out_buf.shape).cpu().numpy())
                return out_buf
        return _array.from_tensor(ret, like)
