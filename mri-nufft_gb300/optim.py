"""Conjugate-gradient reconstruction on the device.

Restates mri-nufft's ``cg`` (``src/mrinufft/extras/optim.py:801-902``) and
``_scaled_dcp`` (151-165) with all state resident on the GPU:

* step 1/L with L from ``operator.get_lipschitz_cst()``;
* when density is set, the start image is the scaled density-compensated
  adjoint and density is disabled during the iterations (838-842);
* ``velocity = tol * velocity + grad / L`` before the loop (855);
* Polak-Ribiere ``beta = dot(g_new, g_new - g) / dot(g, g)`` with
  numpy's non-conjugating complex ``dot`` and ``max(0, beta)`` decided by
  numpy's complex ordering (real part first, then imaginary part), so a kept
  beta keeps its imaginary part (875-879);
* stop when ``||g_new|| <= tol``.

Dot products and norms accumulate in FP64 (``gbn_dotu_f64`` /
``gbn_norm2_f64``); image updates are complex64.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _array
from .plan import dotu_f64, norm2_f64


def _complex_max0(beta: complex) -> complex:
    """``max(0, beta)`` under numpy's lexicographic complex ordering."""
    if beta.real > 0 or (beta.real == 0 and beta.imag > 0):
        return beta
    return 0.0


def scaled_dcp(operator, ksp: torch.Tensor) -> torch.Tensor:
    """x = A^H y * ||y|| / ||A A^H y|| (optim.py:151-165), on the device."""
    x = operator._adj_device(ksp)
    B, C, N = operator.n_batchs, operator.n_coils, operator.shape
    y = operator._op_device(x.reshape(B, *N) if operator.uses_sense else x.reshape(B * C, *N))
    ny = float(norm2_f64(ksp).sqrt())
    nyy = float(norm2_f64(y).sqrt())
    return x * (ny / nyy)


def cg(operator, kspace_data, damp=0.0, x0=None, x_init=None, max_iter=10, tol=1e-4,
       progressbar=False, callback=None):
    """Nonlinear CG with fixed step 1/L; returns an image in the input's array type."""
    like = _array.interface_of(kspace_data)
    dev = operator.device
    L = float(operator.get_lipschitz_cst())
    y = _array.to_tensor(kspace_data, dev, torch.complex64).reshape(operator.ksp_full_shape)
    old_density = None
    if operator.uses_density:
        if x_init is None:
            x_init = scaled_dcp(operator, y)
        old_density = operator._density
        operator._density = None
    shape = operator.img_full_shape
    try:
        if x_init is None:
            image = torch.zeros(shape, dtype=torch.complex64, device=dev)
        else:
            image = _array.to_tensor(x_init, dev, torch.complex64).reshape(shape)
        x0_t = None if x0 is None else _array.to_tensor(x0, dev, torch.complex64).reshape(shape)
        velocity = torch.zeros_like(image)

        def grad_of(img):
            g = dc(operator, img, y)
            if damp:
                g = g + damp * (img - x0_t if x0_t is not None else img)
            return g

        grad = grad_of(image)
        velocity = tol * velocity + grad / L
        image = image - velocity
        results = []
        for _ in range(max_iter):
            grad_new = grad_of(image)
            if float(norm2_f64(grad_new).sqrt()) <= tol:
                break
            num = dotu_f64(grad_new, grad_new) - dotu_f64(grad_new, grad)
            den = dotu_f64(grad, grad)
            n = num.cpu().numpy()
            d = den.cpu().numpy()
            beta = complex(n[0], n[1]) / complex(d[0], d[1])
            beta = _complex_max0(beta)
            velocity = grad_new + beta * velocity
            image = image - velocity / L
            grad = grad_new
            if callback is not None:
                results.append(callback(_array.from_tensor(image, like), operator, kspace_data,
                                        damp=damp, x0=x0))
        if operator.squeeze_dims:
            image = operator._safe_squeeze(image)
        out = _array.from_tensor(image, like)
    finally:
        if old_density is not None:
            operator._density = old_density
    if results:
        return out, results
    return out


def dc(operator, img: torch.Tensor, y: torch.Tensor) -> torch.Tensor:
    """Data-consistency gradient of device tensors in the full shapes."""
    B, C = operator.n_batchs, operator.n_coils
    x = img.reshape(B, *operator.shape) if operator.uses_sense else img.reshape(B * C, *operator.shape)
    out = torch.empty(operator.img_full_shape, dtype=torch.complex64, device=operator.device)
    operator.plan.dc(x.contiguous(), y, operator._density, operator._smaps, out, B, C,
                     operator.inv_norm_factor)
    return out
