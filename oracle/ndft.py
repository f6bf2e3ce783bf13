"""FP64 direct NDFT oracle — TEST INFRASTRUCTURE ONLY.

This module is the checker for the GB300 NUFFT backend. Only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of ``bench.py`` may
import it; the product path never does.

It restates mri-nufft's exact non-uniform DFT
(``src/mrinufft/operators/interfaces/nudft_numpy.py:12-81``):

* type 2 (``op``):  ``y_j = sum_n x_n exp(-2 i pi k_j . n)``
* type 1 (``adj``): ``x_n = sum_j c_j exp(+2 i pi k_j . n)``

with ``k`` in "unit" normalisation ([-0.5, 0.5)) and ``n`` on the centred grid
``linspace(-N/2, N/2 - 1, N)`` per axis, column ``d`` of the samples pairing
with image axis ``d`` (C order).  The reference loops over pixels (type 2) or
samples (type 1); here the sum is factorised per axis
(``exp(-2i pi sum_d k_d n_d) = prod_d exp(-2i pi k_d n_d)``) and evaluated
as a chain of complex128 matrix products, which is the same sum in exact
arithmetic and far faster.  Parity with ``MRInumpy`` is pinned by the golden
fixtures in ``tests/golden``.
"""

from __future__ import annotations

import numpy as np


def proper_trajectory_unit(samples):
    """Flatten to (M, d) float64 in [-0.5, 0.5).

    Restates ``src/mrinufft/_utils.py:58-100`` for ``normalize="unit"``:
    samples whose max |k| exceeds 0.5 + 1e-4 are assumed to be in radians and
    divided by 2 pi; values >= 0.5 are wrapped to [-0.5, 0.5).
    """
    s = np.asarray(samples, dtype=np.float64)
    s = s.reshape(-1, s.shape[-1])
    m = np.max(np.abs(s)) if s.size else 0.0
    if m - 1e-4 > 0.5:
        s = s / (2 * np.pi)
    if m >= 0.5:
        s = (s + 0.5) % 1 - 0.5
    return s


def proper_trajectory_pi(samples):
    """Flatten to (M, d) in radians, restating ``_utils.py:58-100`` ("pi")."""
    s = np.asarray(samples)
    s = s.reshape(-1, s.shape[-1])
    m = np.max(np.abs(s)) if s.size else 0.0
    if m - 1e-4 < 0.5:
        s = s * 2 * np.pi
    return s


def _axis_phases(k_axis, n_axis, sign):
    # (M, N) complex128 table exp(sign * 2 i pi k n)
    return np.exp(sign * 2j * np.pi * np.outer(k_axis, n_axis))


def _grid_axes(shape, grid="ndft"):
    """Per-axis image coordinates.

    ``"ndft"`` is the reference NDFT's ``linspace(-N/2, N/2 - 1, N)``
    (``nudft_numpy.py:38``), half-integer for odd N; ``"finufft"`` is the
    integer mode range ``-(N//2) .. N - N//2 - 1`` that the finufft backend
    uses.  Both agree for even N.
    """
    if grid == "ndft":
        return [np.linspace(-s / 2, s / 2 - 1, s) for s in shape]
    return [np.arange(-(s // 2), s - s // 2, dtype=np.float64) for s in shape]


def ndft_type2(samples, image, shape, chunk=2048, grid="ndft"):
    """Exact forward NDFT of one image; samples in "unit" normalisation.

    Returns complex128 of shape (M,).  Restates
    ``nudft_numpy.py:58-69`` (``implicit_type2_ndft``).
    """
    k = np.asarray(samples, dtype=np.float64).reshape(-1, len(shape))
    x = np.asarray(image, dtype=np.complex128).reshape(shape)
    axes = _grid_axes(shape, grid)
    M = k.shape[0]
    out = np.empty(M, dtype=np.complex128)
    d = len(shape)
    for s0 in range(0, M, chunk):
        kk = k[s0 : s0 + chunk]
        e = [_axis_phases(kk[:, a], axes[a], -1.0) for a in range(d)]
        if d == 1:
            out[s0 : s0 + chunk] = e[0] @ x
        elif d == 2:
            # t[j, n0] = sum_n1 x[n0, n1] e1[j, n1]
            t = e[1] @ x.T
            out[s0 : s0 + chunk] = np.sum(e[0] * t, axis=1)
        else:
            # t[j, n0, n1] = sum_n2 x[n0, n1, n2] e2[j, n2]
            t = np.einsum("abc,jc->jab", x, e[2], optimize=True)
            t = np.einsum("jab,jb->ja", t, e[1], optimize=True)
            out[s0 : s0 + chunk] = np.sum(e[0] * t, axis=1)
    return out


def ndft_type1(samples, coeffs, shape, chunk=4096, grid="ndft"):
    """Exact adjoint NDFT of one k-space vector; samples in "unit" normalisation.

    Returns complex128 of ``shape``.  Restates ``nudft_numpy.py:72-81``
    (``implicit_type1_ndft``).
    """
    k = np.asarray(samples, dtype=np.float64).reshape(-1, len(shape))
    c = np.asarray(coeffs, dtype=np.complex128).reshape(-1)
    axes = _grid_axes(shape, grid)
    d = len(shape)
    out = np.zeros(shape, dtype=np.complex128)
    for s0 in range(0, k.shape[0], chunk):
        kk = k[s0 : s0 + chunk]
        cc = c[s0 : s0 + chunk]
        e = [_axis_phases(kk[:, a], axes[a], +1.0) for a in range(d)]
        if d == 1:
            out += (cc[:, None] * e[0]).sum(0)
        elif d == 2:
            out += (e[0] * cc[:, None]).T @ e[1]
        else:
            t = e[0] * cc[:, None]  # (j, n0)
            # out[n0, n1, n2] = sum_j t[j,n0] e1[j,n1] e2[j,n2]
            t01 = np.einsum("ja,jb->jab", t, e[1], optimize=True)
            out += np.einsum("jab,jc->abc", t01, e[2], optimize=True)
    return out


def ndft_type2_rows(samples, image, shape, rows, grid="ndft"):
    """Exact forward NDFT evaluated only at the sample indices ``rows``."""
    k = np.asarray(samples, dtype=np.float64).reshape(-1, len(shape))
    return ndft_type2(k[rows], image, shape, grid=grid)


def ndft_type1_voxels(samples, coeffs, shape, voxels, chunk=8192, grid="ndft"):
    """Exact adjoint NDFT evaluated only at the flat voxel indices ``voxels``."""
    k = np.asarray(samples, dtype=np.float64).reshape(-1, len(shape))
    c = np.asarray(coeffs, dtype=np.complex128).reshape(-1)
    axes = _grid_axes(shape, grid)
    idx = np.unravel_index(np.asarray(voxels), shape)
    pos = np.stack([axes[a][idx[a]] for a in range(len(shape))], axis=1)  # (V, d)
    out = np.zeros(len(voxels), dtype=np.complex128)
    for s0 in range(0, k.shape[0], chunk):
        ph = np.exp(2j * np.pi * (k[s0 : s0 + chunk] @ pos.T))  # (j, V)
        out += c[s0 : s0 + chunk] @ ph
    return out


def ndft_type1_grid(samples, coeffs, shape, axis_idx, chunk=16384, grid="ndft"):
    """Exact adjoint NDFT at the product set of per-axis image indices
    ``axis_idx`` (one integer array per axis), e.g. 16 seeded indices per
    axis of a 3D image for 4096 voxels.  The phase factorises per axis, so
    the sum is a chain of small matrix products per chunk of samples.
    ``coeffs`` is (M,) or (C, M) (several k-space vectors share the phase
    tables).  Returns complex128 of shape ``[C] + [len(i) for i in axis_idx]``."""
    k = np.asarray(samples, dtype=np.float64).reshape(-1, len(shape))
    c = np.asarray(coeffs, dtype=np.complex128)
    single = c.ndim == 1
    c = c.reshape(-1, k.shape[0])
    C = c.shape[0]
    axes = _grid_axes(shape, grid)
    pos = [axes[a][np.asarray(axis_idx[a])] for a in range(len(shape))]
    d = len(shape)
    sizes = tuple(len(p) for p in pos)
    out = np.zeros((C, *sizes), dtype=np.complex128)
    for s0 in range(0, k.shape[0], chunk):
        kk = k[s0 : s0 + chunk]
        e = [_axis_phases(kk[:, a], pos[a], +1.0) for a in range(d)]
        for q in range(C):
            t = e[0] * c[q, s0 : s0 + chunk, None]  # (j, n0)
            if d == 2:
                out[q] += t.T @ e[1]
            else:
                t01 = (t[:, :, None] * e[1][:, None, :]).reshape(t.shape[0], -1)  # (j, n0 n1)
                out[q] += (t01.T @ e[2]).reshape(sizes)
    return out[0] if single else out


def norm_factor(shape):
    """``sqrt(prod(N) * 2**d)``, restating ``operators/base.py:837-850``."""
    return float(np.sqrt(np.prod(shape) * (2 ** len(shape))))
