"""Coil sensitivity estimation from the k-space centre, on the GB300 library.

Restates mri-nufft's ``low_frequency`` method (``src/mrinufft/extras/
smaps.py:85-306``): the samples inside a window around the k-space centre
(ellipse, rectangle, Hann / Hamming, or a callable) keep their values, a
calibrationless operator with one "coil" per channel reconstructs them by
LSQR (the device solver of :mod:`mrinufft_gb300.optim`), and the images are
normalised by their root sum of squares.  Masking by the convex hull of an
Otsu threshold and Gaussian smoothing use scikit-image, as in the reference,
and are available only when it is installed.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _array
from ._traj import proper_trajectory


def _window(loc: torch.Tensor, threshold, window_fun) -> torch.Tensor:
    """Per-sample weights of the k-space centre window (smaps.py:135-170)."""
    d = loc.shape[1]
    thr = torch.as_tensor(np.broadcast_to(np.asarray(threshold, dtype=np.float64), (d,)).copy(),
                          dtype=loc.dtype, device=loc.device)
    if callable(window_fun):
        return _array.to_tensor(window_fun(loc), loc.device, torch.float32).reshape(-1)
    if window_fun == "rect":
        return ((loc.abs() - thr) <= 0).all(dim=1).to(torch.float32)
    if window_fun in ("hann", "hanning", "hamming"):
        radius = torch.linalg.norm(loc, dim=1)
        a0 = 0.5 if window_fun in ("hann", "hanning") else 0.53836
        return (a0 + (1 - a0) * torch.cos(np.pi * radius / thr[0])).to(torch.float32)
    if window_fun == "ellipse":
        return ((loc ** 2 / thr ** 2).sum(dim=1) <= 1).to(torch.float32)
    raise ValueError("Unsupported window function.")


def low_frequency(traj, shape, kspace_data, backend="gb300", threshold=0.1, density=None,
                  max_iter=10, window_fun="ellipse", blurr_factor=0.0, mask=False, device=None):
    """Sensitivity maps (n_coils, *shape) from the k-space centre; returned in
    the array type of ``kspace_data``."""
    from .operator import MRIGB300

    like = _array.interface_of(kspace_data)
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    shape = tuple(int(s) for s in shape)
    loc = _array.to_tensor(proper_trajectory(traj, normalize="unit"), dev, torch.float32)
    loc = loc.reshape(-1, len(shape))
    y = _array.to_tensor(kspace_data, dev, torch.complex64)
    y = y.reshape(-1, loc.shape[0])
    C = y.shape[0]
    y = y * _window(loc, threshold, window_fun)
    op = MRIGB300(loc, shape, n_coils=C, squeeze_dims=True, device=dev.index)
    maps = _array.to_tensor(op.pinv_solver(y, max_iter=max_iter), dev, torch.complex64)
    maps = maps.reshape(C, *shape)
    sos = torch.linalg.vector_norm(maps, dim=0)
    if isinstance(mask, (np.ndarray, torch.Tensor)):
        maps = maps * _array.to_tensor(mask, dev, torch.float32)
    elif isinstance(mask, bool) and mask:
        from skimage.filters import threshold_otsu  # type: ignore
        from skimage.morphology import convex_hull_image  # type: ignore

        s = sos.cpu().numpy()
        hull = convex_hull_image(s > threshold_otsu(s))
        maps = maps * torch.from_numpy(hull.astype(np.float32)).to(dev)
    if np.sum(blurr_factor) > 0:
        from skimage.filters import gaussian  # type: ignore

        if isinstance(blurr_factor, (float, int)):
            blurr_factor = (blurr_factor,) * len(shape)
        m = maps.cpu().numpy()
        m = gaussian(np.abs(m), sigma=(0,) + tuple(blurr_factor)) * np.exp(1j * np.angle(m))
        maps = torch.from_numpy(m.astype(np.complex64)).to(dev)
    any_mask = bool(mask.any()) if isinstance(mask, torch.Tensor) else bool(np.any(mask))
    if any_mask or np.sum(blurr_factor) > 0:
        sos = torch.linalg.vector_norm(maps, dim=0) + 1e-10
    return _array.from_tensor(maps / sos, like)


METHODS = {"low_frequency": low_frequency}
