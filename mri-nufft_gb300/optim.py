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
       progressbar=False, callback=None, toeplitz=False):
    """Nonlinear CG with fixed step 1/L; returns an image in the input's array type.

    ``toeplitz=True`` (an option of this backend, off by default) takes the
    power method and the gradients A^H A x - A^H y from the Toeplitz
    embedding of the Gram operator (A^H y from one adjoint at the start)
    instead of a forward and an adjoint NUFFT per iteration; the iteration
    is otherwise the same."""
    like = _array.interface_of(kspace_data)
    dev = operator.device
    L = float(operator.get_lipschitz_cst(toeplitz=toeplitz))
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
        if toeplitz:
            gram = operator._unweighted_toeplitz()
            rhs = operator._adj_device(y, density=False)
            B, C = operator.n_batchs, operator.n_coils

        def grad_of(img):
            if toeplitz:
                x = img.reshape(B, *operator.shape) if operator.uses_sense else img.reshape(B * C, *operator.shape)
                g = torch.empty(shape, dtype=torch.complex64, device=dev)
                gram.apply(x.contiguous(), operator._smaps, g, B, C, operator.inv_norm_factor ** 2)
                g = g - rhs.reshape(shape)
            else:
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


def _norms(x: torch.Tensor) -> np.ndarray:
    """FP64 l2 norm of every batch item (leading axis) of a device tensor."""
    return np.array([float(norm2_f64(x[b].contiguous()).sqrt()) for b in range(x.shape[0])])


def _bcl(s, like: torch.Tensor) -> torch.Tensor:
    """Per-batch scalars broadcast from the leading axis (optim.py:68-86)."""
    t = torch.as_tensor(np.asarray(s, dtype=np.float64), dtype=torch.float32, device=like.device)
    return t.reshape(t.shape + (1,) * (like.ndim - t.ndim))


def _sym_ortho(a, b):
    """Stable Givens rotation (optim.py:213-246), batch-wise."""
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    if np.any(b == 0):
        return np.sign(a), 0.0, np.abs(a)
    if np.any(a == 0):
        return 0.0, np.sign(b), np.abs(b)
    if np.any(np.abs(b) > np.abs(a)):
        tau = a / b
        s = np.sign(b) / np.sqrt(1 + tau * tau)
        return s * tau, s, b / s
    tau = b / a
    c = np.sign(a) / np.sqrt(1 + tau * tau)
    return c, c * tau, a / c


def lsqr(operator, kspace_data, damp=0.0, atol=1e-6, btol=1e-6, conlim=1e8, max_iter=100,
         x0=None, x_init=None, callback=None, progressbar=False):
    """LSQR of mri-nufft (``extras/optim.py:249-495``, Paige & Saunders) on
    the device: the vectors u, v, w, x and every transform stay on the GPU,
    the per-batch norms accumulate in FP64 and the scalar recurrences run on
    the host, batch-wise as in the reference (including its stopping tests
    and its handling of density: start from the scaled density-compensated
    adjoint, density disabled during the iterations)."""
    like = _array.interface_of(kspace_data)
    dev = operator.device
    y = _array.to_tensor(kspace_data, dev, torch.complex64).reshape(operator.ksp_full_shape)
    old_density = None
    if operator.uses_density:
        if x_init is None:
            x_init = scaled_dcp(operator, y)
        old_density = operator._density
        operator._density = None
    B, C = operator.n_batchs, operator.n_coils
    shape = operator.img_full_shape

    def A(img):
        x = img.reshape(B, *operator.shape) if operator.uses_sense else img.reshape(B * C, *operator.shape)
        return operator._op_device(x.contiguous()).reshape(operator.ksp_full_shape)

    def AH(k):
        return operator._adj_device(k.contiguous()).reshape(shape)

    results = []
    try:
        ctol = 1 / conlim if conlim > 0 else 0
        eps = np.finfo(np.float32).eps
        u = y.clone()
        bnorm = _norms(u)
        if x_init is None:
            x = (torch.zeros(shape, dtype=torch.complex64, device=dev) if x0 is None
                 else _array.to_tensor(x0, dev, torch.complex64).reshape(shape).clone())
        else:
            x = _array.to_tensor(x_init, dev, torch.complex64).reshape(shape).clone()
        x0_t = None if x0 is None else _array.to_tensor(x0, dev, torch.complex64).reshape(shape)
        beta = bnorm.copy()
        if x0_t is not None:
            u -= A(x0_t)
            beta = _norms(u)
        if np.all(beta) > 0:
            u /= _bcl(beta, u)
            v = AH(u)
            alpha = _norms(v)
        else:
            v = x.clone()
            alpha = np.zeros(v.shape[0])
        if np.any((alpha * beta) == 0):
            return _finish(operator, x, like, results, old_density)
        if np.all(alpha) > 0:
            v /= _bcl(alpha, v)
        w = v.clone()
        rhobar = alpha
        phibar = rnorm = beta
        ddnorm = res2 = xnorm = xxnorm = z = anorm = acond = 0.0
        dampsq = damp ** 2
        cs2, sn2 = -1.0, 0.0
        for _ in range(max_iter):
            u *= -_bcl(alpha, u)
            u += A(v)
            beta = _norms(u)
            if np.all(beta) > 0:
                u /= _bcl(beta, u)
                anorm = np.sqrt(anorm ** 2 + alpha ** 2 + beta ** 2 + dampsq)
                v *= -_bcl(beta, v)
                v += AH(u)
                alpha = _norms(v)
                if np.all(alpha) > 0:
                    v /= _bcl(alpha, v)
            if damp:
                rhobar1 = np.sqrt(rhobar ** 2 + dampsq)
                cs1 = rhobar / rhobar1
                sn1 = damp / rhobar1
                psi = sn1 * phibar
                phibar = cs1 * phibar
            else:
                rhobar1 = rhobar
                psi = 0.0
            cs, sn, rho = _sym_ortho(rhobar1, beta)
            theta = sn * alpha
            rhobar = -cs * alpha
            phi = cs * phibar
            phibar = sn * phibar
            tau = sn * phi
            t1 = phi / rho
            t2 = -theta / rho
            dk = w / _bcl(rho, w)
            x += _bcl(t1, w) * w
            w *= _bcl(t2, w)
            w += v
            ddnorm = ddnorm + _norms(dk) ** 2
            delta = sn2 * rho
            gambar = -cs2 * rho
            rhs = phi - delta * z
            zbar = rhs / gambar
            xnorm = np.sqrt(xxnorm + zbar ** 2)
            gamma = np.sqrt(gambar ** 2 + theta ** 2)
            cs2 = gambar / gamma
            sn2 = theta / gamma
            z = rhs / gamma
            xxnorm = xxnorm + z ** 2
            acond = anorm * np.sqrt(ddnorm)
            res1 = phibar ** 2
            res2 = res2 + psi ** 2
            rnorm = np.sqrt(res1 + res2)
            arnorm = alpha * np.abs(tau)
            test1 = rnorm / bnorm
            test2 = arnorm / (anorm * rnorm + eps)
            test3 = 1 / (acond + eps)
            t1 = test1 / (1 + anorm * xnorm / bnorm)
            rtol = btol + atol * anorm * xnorm / bnorm
            if callback is not None:
                results.append(callback(_array.from_tensor(x, like), operator, kspace_data,
                                        damp=damp, x0=x0))
            if (np.all(1 + test3 <= 1) or np.all(1 + test2 <= 1) or np.all(1 + t1 <= 1)
                    or np.all(test3 <= ctol) or np.all(test2 <= atol) or np.all(test1 <= rtol)):
                break
        return _finish(operator, x, like, results, old_density)
    finally:
        if old_density is not None:
            operator._density = old_density


def _finish(operator, x, like, results, old_density):
    if operator.squeeze_dims:
        x = operator._safe_squeeze(x)
    out = _array.from_tensor(x, like)
    if results:
        return out, results
    return out
