"""Stand-alone statement of mri-nufft's operator contract.

When ``mrinufft`` is importable, the GB300 operator subclasses its
``FourierOperatorBase`` and registers in its backend table, so that
``mrinufft.get_operator("gb300")`` returns it.  Without ``mrinufft`` the
operator derives from the class below, which restates the same contract
(``src/mrinufft/operators/base.py:45-877``): the backend registry filled by
``__init_subclass__`` (211-218), ``get_operator`` (86-179), shape checking
(225-260), squeezing (262-273), shape / coil / batch properties (702-746),
the normalisation factor (837-850) and the autograd constructors (536-574,
863-877).  Method names, argument meaning and exceptions are the
reference's.
"""

from __future__ import annotations

from functools import partial

import numpy as np

DTYPE_R2C = {"float32": "complex64", "float64": "complex128"}


class FourierOperatorBase:
    """Minimal FourierOperatorBase: registry, shapes and normalisation."""

    interfaces: dict = {}
    autograd_available = False

    def __init__(self, *args, **kwargs):
        if not self.available:
            raise RuntimeError(f"'{self.backend}' backend is not available.")
        self._smaps = None
        self._density = None
        self._n_coils = 1
        self._n_batchs = 1
        self.n_trans = 1
        self.squeeze_dims = False
        self._density_method = None
        self._grad_wrt_data = False
        self._grad_wrt_traj = False
        self._grad_wrt_field_map = False

    def __init_subclass__(cls):
        super().__init_subclass__()
        available = getattr(cls, "available", True)
        if callable(available):
            available = available()
        if backend := getattr(cls, "backend", None):
            cls.interfaces[backend] = (available, cls)

    def check_shape(self, *, image=None, ksp=None):
        if image is not None:
            image_shape = tuple(image.shape[-len(self.shape):])
            if image_shape != self.shape:
                raise ValueError(
                    f"Image shape {image_shape} is not compatible "
                    f"with the operator shape {self.shape}"
                )
        if ksp is not None:
            if ksp.shape[-1] != self.n_samples:
                raise ValueError(
                    f"Kspace samples {ksp.shape[-1]} is not compatible "
                    f"with the operator samples {self.n_samples}"
                )
        if image is None and ksp is None:
            raise ValueError("Nothing to check, provides image or ksp arguments")

    def _safe_squeeze(self, arr):
        if self.squeeze_dims:
            if arr.shape[1] == 1 if arr.ndim > 1 else False:
                arr = arr.squeeze(1)
            if arr.shape[0] == 1 if arr.ndim > 0 else False:
                arr = arr.squeeze(0)
        return arr

    @property
    def uses_sense(self):
        return self._smaps is not None

    @property
    def uses_density(self):
        return self.density is not None

    @property
    def ndim(self):
        return len(self._shape)

    @property
    def shape(self):
        return self._shape

    @shape.setter
    def shape(self, shape):
        self._shape = tuple(int(i) for i in shape)

    @property
    def n_coils(self):
        return self._n_coils

    @n_coils.setter
    def n_coils(self, n_coils):
        if n_coils < 1 or not int(n_coils) == n_coils:
            raise ValueError(f"n_coils should be a positive integer, {type(n_coils)}")
        self._n_coils = int(n_coils)

    @property
    def n_batchs(self):
        return self._n_batchs

    @n_batchs.setter
    def n_batchs(self, n_batchs):
        if n_batchs < 1 or not int(n_batchs) == n_batchs:
            raise ValueError(f"n_batchs should be a positive integer, {type(n_batchs)}")
        self._n_batchs = int(n_batchs)

    @property
    def img_full_shape(self):
        return (self.n_batchs, (1 if self.uses_sense else self.n_coils)) + self.shape

    @property
    def ksp_full_shape(self):
        return (self.n_batchs, self.n_coils, self.n_samples)

    @property
    def dtype(self):
        return self._dtype

    @dtype.setter
    def dtype(self, new_dtype):
        self._dtype = np.dtype(new_dtype)

    @property
    def cpx_dtype(self):
        return np.dtype(DTYPE_R2C[str(self.dtype)])

    @property
    def norm_factor(self):
        return np.sqrt(np.prod(self.shape) * (2 ** len(self.shape)))

    @property
    def inv_norm_factor(self):
        return 1.0 / self.norm_factor

    def make_autograd(self, *, wrt_data=True, wrt_traj=False, paired_batch=False):
        if not self.autograd_available:
            raise ValueError("Backend does not support auto-differentiation.")
        from .autodiff import MRINufftAutoGrad

        return MRINufftAutoGrad(self, wrt_data=wrt_data, wrt_traj=wrt_traj,
                                paired_batch=paired_batch)

    @classmethod
    def with_autograd(cls, wrt_data=True, wrt_traj=False, paired_batch=False, *args, **kwargs):
        return cls(*args, **kwargs).make_autograd(
            wrt_data=wrt_data, wrt_traj=wrt_traj, paired_batch=paired_batch
        )

    def __repr__(self):
        return (
            f"{self.__class__.__name__}(\n"
            f"  shape: {self.shape}\n"
            f"  n_coils: {self.n_coils}\n"
            f"  n_samples: {self.n_samples}\n"
            f"  uses_sense: {self.uses_sense}\n"
            ")"
        )


def get_operator(backend_name, wrt_data=False, wrt_traj=False, paired_batch=False, *args, **kwargs):
    """Registry lookup restating ``operators/base.py:86-179`` (no stacked backends)."""
    backend_name = backend_name.lower()
    try:
        available, operator = FourierOperatorBase.interfaces[backend_name]
    except KeyError as exc:
        raise ValueError(f"backend {backend_name} does not exist") from exc
    if not available:
        raise ValueError(f"backend {backend_name} found, but dependencies are not met.")
    if args or kwargs:
        operator = operator(*args, **kwargs)
    if wrt_data or wrt_traj:
        if isinstance(operator, partial):
            raise ValueError("Cannot create autograd of a partial operator.")
        if isinstance(operator, FourierOperatorBase):
            operator = operator.make_autograd(wrt_data=wrt_data, wrt_traj=wrt_traj,
                                              paired_batch=paired_batch)
        else:
            operator = partial(operator.with_autograd, wrt_data, wrt_traj, paired_batch)
    return operator
