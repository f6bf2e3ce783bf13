"""Toeplitz embedding of the Gram operator in FP64 — TEST INFRASTRUCTURE ONLY.

Restates, with numpy and the exact NDFT of ``oracle/ndft.py``, the
construction that ``gbn_toep_create`` / ``gbn_toep_apply`` run on the GPU and
that mri-nufft's ``compute_toeplitz_kernel`` / ``apply_toeplitz_kernel``
(``src/mrinufft/operators/toeplitz.py:35-96, 193-269``) compute by another
route (modulated adjoints on the N grid): A^H W A x is the linear
convolution of x with psf(m) = sum_j w_j exp(+i k_j . m), |m_d| < N_d, a
circular convolution on a grid of P_d >= 2 N_d - 1 cells.  Imported only by
tests.
"""

from __future__ import annotations

import numpy as np

from . import ndft


def toeplitz_kernel(samples, shape, weights=None, grid=None):
    """Real kernel spectrum on the circulant grid (default 2N), scaled by
    1/norm_factor^2 as the reference's kernel."""
    shape = tuple(int(s) for s in shape)
    s = ndft.proper_trajectory_unit(samples)
    M = s.shape[0]
    w = np.ones(M) if weights is None else np.asarray(weights, dtype=np.float64)
    two = tuple(2 * n for n in shape)
    psf = ndft.ndft_type1(s, w.astype(np.complex128), two)  # mode m at index m + N
    P = two if grid is None else tuple(grid)
    placed = np.zeros(P, dtype=np.complex128)
    idx = []
    src = []
    for N, p in zip(shape, P):
        m = np.arange(-(N - 1), N)
        idx.append(np.mod(m, p))
        src.append(m + N)
    placed[np.ix_(*idx)] = psf[np.ix_(*src)]
    return np.fft.fftn(placed).real / ndft.norm_factor(shape) ** 2


def apply_toeplitz(x, kernel):
    """Zero-pad x (mode n at index n mod P), multiply its FFT by the kernel,
    inverse FFT, crop."""
    shape = x.shape
    P = kernel.shape
    pad = np.zeros(P, dtype=np.complex128)
    idx = [np.mod(np.arange(N) - N // 2, p) for N, p in zip(shape, P)]
    pad[np.ix_(*idx)] = x
    out = np.fft.ifftn(np.fft.fftn(pad) * kernel)
    return out[np.ix_(*idx)]
