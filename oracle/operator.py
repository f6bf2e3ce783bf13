"""Operator-level oracle on the FP64 NDFT — TEST INFRASTRUCTURE ONLY.

Restates the per-coil / per-batch semantics of mri-nufft's
``FourierOperatorSimple`` (``src/mrinufft/operators/base.py:949-1139``) and
its CG solver (``src/mrinufft/extras/optim.py:151-165, 801-902``) and power
method (``base.py:1155-1221``) on top of the exact NDFT of
``oracle/ndft.py``, in complex128.  Imported only by tests, the smoke check
and the bench's CPU baseline leg.
"""

from __future__ import annotations

import numpy as np

from . import ndft


class NDFTOperator:
    """FP64 reference operator with SENSE maps, batches and density."""

    def __init__(self, samples, shape, n_coils=1, n_batchs=1, smaps=None, density=None,
                 grid="ndft"):
        self.samples = ndft.proper_trajectory_unit(samples)
        self.shape = tuple(int(s) for s in shape)
        self.n_coils = n_coils if smaps is None else smaps.shape[0]
        self.n_batchs = n_batchs
        self.smaps = None if smaps is None else np.asarray(smaps, dtype=np.complex128)
        self.density = None if density is None else np.asarray(density, dtype=np.float64)
        self.norm = ndft.norm_factor(self.shape)
        self.grid = grid

    @property
    def M(self):
        return self.samples.shape[0]

    def _t2(self, x):
        return ndft.ndft_type2(self.samples, x, self.shape, grid=self.grid)

    def _t1(self, c):
        return ndft.ndft_type1(self.samples, c, self.shape, grid=self.grid)

    def op(self, x):
        """(B, 1|C, *N) -> (B, C, M); base.py:949-1010."""
        B, C = self.n_batchs, self.n_coils
        x = np.asarray(x, dtype=np.complex128)
        out = np.empty((B, C, self.M), dtype=np.complex128)
        if self.smaps is not None:
            x = x.reshape(B, *self.shape)
            for b in range(B):
                for c in range(C):
                    out[b, c] = self._t2(self.smaps[c] * x[b])
        else:
            x = x.reshape(B, C, *self.shape)
            for b in range(B):
                for c in range(C):
                    out[b, c] = self._t2(x[b, c])
        return out / self.norm

    def adj(self, y, use_density=True):
        """(B, C, M) -> (B, 1|C, *N); base.py:1015-1073."""
        B, C = self.n_batchs, self.n_coils
        y = np.asarray(y, dtype=np.complex128).reshape(B, C, self.M)
        if use_density and self.density is not None:
            y = y * self.density
        if self.smaps is not None:
            out = np.zeros((B, 1, *self.shape), dtype=np.complex128)
            for b in range(B):
                for c in range(C):
                    out[b, 0] += np.conj(self.smaps[c]) * self._t1(y[b, c])
        else:
            out = np.empty((B, C, *self.shape), dtype=np.complex128)
            for b in range(B):
                for c in range(C):
                    out[b, c] = self._t1(y[b, c])
        return out / self.norm

    def dc(self, x, y):
        """A^H(Ax - y) with density once (base.py:1094-1139)."""
        return self.adj(self.op(x) - np.asarray(y).reshape(self.n_batchs, self.n_coils, self.M))

    def gram(self, x):
        return self.adj(self.op(x))


class EsOperator(NDFTOperator):
    """The same operator semantics with the FP64 CPU ES-kernel NUFFT of
    ``oracle/esnufft.py`` (eps 1e-6, about 1e-6 from the exact NDFT) in
    place of the exact sum, for sizes where the NDFT would take hours."""

    def __init__(self, samples, shape, n_coils=1, n_batchs=1, smaps=None, density=None,
                 eps=1e-6, nthreads=None):
        super().__init__(samples, shape, n_coils=n_coils, n_batchs=n_batchs, smaps=smaps,
                         density=density)
        from . import esnufft

        self._es = esnufft.EsNufft(self.samples * (2 * np.pi), self.shape, eps=eps,
                                   dtype=np.float64, nthreads=nthreads)

    def _t2(self, x):
        return self._es.type2(np.asarray(x, dtype=np.complex128).reshape(self.shape))

    def _t1(self, c):
        return self._es.type1(np.asarray(c, dtype=np.complex128).reshape(-1))


def power_method(max_iter, gram, x):
    """base.py:1155-1221 with numpy norms; returns (norm, x)."""
    x = np.array(x, dtype=np.complex128)
    x_norm = np.linalg.norm(x)
    x = x / x_norm
    x_new_norm = x_norm
    for _ in range(max_iter):
        x_new = gram(x)
        x_new_norm = np.linalg.norm(x_new)
        x_new = x_new / x_new_norm
        if abs(x_norm - x_new_norm) < 1e-6:
            break
        x_norm = x_new_norm
        x = x_new
    return x_new_norm, x_new


def cg(op: NDFTOperator, y, L, max_iter=10, tol=1e-4, damp=0.0, x0=None):
    """optim.py:801-902 (density handling of 838-842) in complex128."""
    y = np.asarray(y, dtype=np.complex128).reshape(op.n_batchs, op.n_coils, op.M)
    img_shape = (op.n_batchs, 1 if op.smaps is not None else op.n_coils, *op.shape)
    x_init = None
    old_density = None
    if op.density is not None:
        xi = op.adj(y)
        yy = op.op(xi)
        x_init = xi * np.linalg.norm(y) / np.linalg.norm(yy)
        old_density = op.density
        op.density = None
    try:
        image = np.zeros(img_shape, dtype=np.complex128) if x_init is None else x_init.reshape(img_shape)
        velocity = np.zeros_like(image)

        def grad_of(img):
            g = op.dc(img, y).reshape(img_shape)
            if damp:
                g = g + damp * (img - (x0 if x0 is not None else 0))
            return g

        grad = grad_of(image)
        velocity = tol * velocity + grad / L
        image = image - velocity
        for _ in range(max_iter):
            grad_new = grad_of(image)
            if np.linalg.norm(grad_new) <= tol:
                break
            beta = np.dot(grad_new.ravel(), (grad_new - grad).ravel()) / np.dot(grad.ravel(), grad.ravel())
            beta = max(0, beta)
            velocity = grad_new + beta * velocity
            image = image - velocity / L
            grad = grad_new
        return image
    finally:
        if old_density is not None:
            op.density = old_density
