"""Stacked NUFFT in FP64 — TEST INFRASTRUCTURE ONLY.

Restates mri-nufft's ``MRIStackedNUFFT`` (``src/mrinufft/operators/stacked.py:
178-330``) on the exact NDFT of ``oracle/ndft.py``: per coil, a centred
orthonormal DFT along the last axis divided by sqrt(2), then the normalised
2D NDFT of each kept plane; the adjoint in reverse.  Imported only by tests.
"""

from __future__ import annotations

import numpy as np

from . import ndft


def _fftz(x):
    return np.fft.fftshift(np.fft.fft(np.fft.ifftshift(x, axes=-1), axis=-1, norm="ortho"),
                           axes=-1) / np.sqrt(2)


def _ifftz(x):
    return np.fft.fftshift(np.fft.ifft(np.fft.ifftshift(x, axes=-1), axis=-1, norm="ortho"),
                           axes=-1) / np.sqrt(2)


def stacked_op(samples2d, shape, z_index, x, smaps=None, n_coils=1, n_batchs=1):
    """(B, *shape) with maps or (B, C, *shape) -> (B, C, NZ * NS)."""
    s = ndft.proper_trajectory_unit(samples2d)
    sh2 = tuple(shape[:2])
    nrm = ndft.norm_factor(sh2)
    C = n_coils if smaps is None else smaps.shape[0]
    B = n_batchs
    x = np.asarray(x, dtype=np.complex128)
    xs = x.reshape(B, *shape) if smaps is not None else x.reshape(B, C, *shape)
    out = np.empty((B, C, len(z_index), s.shape[0]), dtype=np.complex128)
    for b in range(B):
        for c in range(C):
            img = xs[b] * smaps[c] if smaps is not None else xs[b, c]
            z = _fftz(img)
            for k, zi in enumerate(z_index):
                out[b, c, k] = ndft.ndft_type2(s, z[..., zi], sh2) / nrm
    return out.reshape(B, C, -1)


def stacked_adj(samples2d, shape, z_index, y, smaps=None, n_coils=1, n_batchs=1):
    """(B, C, NZ * NS) -> (B, *shape) with maps or (B, C, *shape)."""
    s = ndft.proper_trajectory_unit(samples2d)
    sh2 = tuple(shape[:2])
    nrm = ndft.norm_factor(sh2)
    C = n_coils if smaps is None else smaps.shape[0]
    B = n_batchs
    y = np.asarray(y, dtype=np.complex128).reshape(B, C, len(z_index), s.shape[0])
    imgs = np.zeros((B, C, *shape), dtype=np.complex128)
    for b in range(B):
        for c in range(C):
            for k, zi in enumerate(z_index):
                imgs[b, c][..., zi] = ndft.ndft_type1(s, y[b, c, k], sh2) / nrm
    imgs = _ifftz(imgs)
    if smaps is None:
        return imgs
    return np.sum(imgs * np.conj(smaps)[None], axis=1)
