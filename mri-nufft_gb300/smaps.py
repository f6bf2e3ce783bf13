"""Coil sensitivity estimation from the k-space centre, on the GB300 library.

Restates mri-nufft's ``low_frequency`` method (``src/mrinufft/extras/
smaps.py:85-306``) and its ESPIRiT (``smaps.py:315-471``, at the end of this
module).  low_frequency: the samples inside a window around the k-space centre
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


def _cfft(x: torch.Tensor, dims=3, inverse=False) -> torch.Tensor:
    """Centred orthonormal FFT over the last ``dims`` axes
    (``extras/cartesian.py:6-59``: ifftshift, fftn / ifftn, fftshift).  The
    reference's callers keep its default ``dims=3``, which for a 2D coil
    stack (C, X, Y) also transforms the coil axis; so does this restatement."""
    axes = tuple(range(-min(dims, x.ndim), 0))
    y = torch.fft.ifftshift(x, dim=axes)
    y = (torch.fft.ifftn if inverse else torch.fft.fftn)(y, dim=axes, norm="ortho")
    return torch.fft.fftshift(y, dim=axes)


def _crop_or_pad(x: torch.Tensor, target) -> torch.Tensor:
    """Centred crop / zero pad to ``target`` (smaps.py:178-216)."""
    slices, pads = [], []
    for s_, t in zip(x.shape, target):
        diff = t - s_
        before = max(diff, 0) // 2
        pads.append((before, max(diff, 0) - before))
        c0 = max(-diff, 0) // 2
        slices.append(slice(c0, c0 + min(s_, t)))
    x = x[tuple(slices)]
    if any(p != (0, 0) for p in pads):
        flat = [v for p in reversed(pads) for v in p]
        x = torch.nn.functional.pad(x, flat)
    return x


def cartesian_espirit(kspace, shape, calib_width=24, kernel_width=6, thresh=0.02, crop=0.95,
                      decim=1, device=None, kernel_chunk=16):
    """ESPIRiT maps from Cartesian k-space (n_coils, *kspace_shape), on the
    device (``extras/smaps.py:367-471``): the calibration region's Hankel
    block matrix (sliding kernel windows), its SVD (in complex128) and the
    right singular vectors above ``thresh`` times the largest; the image-space
    covariance sum_k v_k v_k^H of the zero-padded, inverse-transformed
    kernels per voxel; its leading eigenvector per voxel by 100 power
    iterations (``operators/base.py:1155-1221`` with a per-voxel norm and the
    reference's global stopping test); phase relative to coil 0; voxels whose
    eigenvalue is not above ``crop`` set to zero.

    The reference's last step multiplies by an eigenvalue array that does
    not broadcast against the maps when ``decim == 1`` and raises; here the
    mask is applied per voxel, as its ``decim > 1`` branch does.  ``decim > 1``
    (phase unwrapping by scikit-image) is not restated."""
    if decim > 1:
        raise NotImplementedError("decim > 1 needs scikit-image's phase unwrapping")
    like = _array.interface_of(kspace)
    maps, eig = espirit_eigen(kspace, calib_width, kernel_width, thresh, device, kernel_chunk)
    return _array.from_tensor(maps * (eig > crop), like)


def espirit_eigen(kspace, calib_width=24, kernel_width=6, thresh=0.02, device=None, kernel_chunk=16):
    """The unmasked ESPIRiT maps (phase relative to coil 0) and the leading
    eigenvalue per voxel, as device tensors (see :func:`cartesian_espirit`)."""
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    k = _array.to_tensor(kspace, dev, torch.complex64)
    C = k.shape[0]
    d = k.ndim - 1
    cw = (calib_width,) * d if isinstance(calib_width, int) else tuple(calib_width)
    kw = (kernel_width,) * d if isinstance(kernel_width, int) else tuple(kernel_width)
    calib = _crop_or_pad(k, (C, *cw))
    for a, w in enumerate(kw):
        calib = calib.unfold(1 + a, w, 1)  # (C, n..., k...) as sliding_window_view
    nk = int(np.prod(kw))
    calib = calib.reshape(C, -1, nk).permute(1, 0, 2).reshape(-1, C * nk)
    _, S, VH = torch.linalg.svd(calib.to(torch.complex128), full_matrices=False)
    VH = VH[S > thresh * S.max()].to(torch.complex64)
    kernels = VH.reshape(VH.shape[0], C, *kw)
    spatial = tuple(k.shape[1:])
    nvox = int(np.prod(spatial))
    aha = torch.zeros((nvox, C, C), dtype=torch.complex64, device=dev)
    for k0 in range(0, kernels.shape[0], kernel_chunk):
        kc = kernels[k0:k0 + kernel_chunk]
        imgs = torch.stack([_cfft(_crop_or_pad(kk, k.shape), inverse=True) for kk in kc])
        v = imgs.reshape(kc.shape[0], C, nvox).permute(2, 1, 0)  # (vox, C, kernels)
        aha += v @ v.conj().transpose(1, 2)
    aha *= float(nvox) / float(np.prod(kw))
    # per-voxel power method from ones (base.py:1155-1221)
    x = torch.ones((nvox, C, 1), dtype=torch.complex64, device=dev)
    x_norm = torch.linalg.vector_norm(x, dim=1, keepdim=True)
    x = x / x_norm
    x_new, x_new_norm = x, x_norm
    for _ in range(100):
        x_new = aha @ x
        x_new_norm = torch.linalg.vector_norm(x_new, dim=1, keepdim=True)
        x_new = x_new / x_new_norm
        if float(torch.linalg.vector_norm(x_norm - x_new_norm)) < 1e-6:
            break
        x_norm = x_new_norm
        x = x_new
    maps = x_new[..., 0].transpose(0, 1).reshape(C, *spatial)
    eig = x_new_norm.reshape(spatial).real
    maps = maps * (maps[0] / maps[0].abs()).conj()
    return maps, eig


def espirit(traj, shape, kspace_data, backend="gb300", density=None, max_iter=10, calib_width=24,
            kernel_width=6, thresh=0.02, crop=0.95, decim=1, device=None):
    """ESPIRiT on non-Cartesian data (``extras/smaps.py:315-364``): the samples
    inside the rectangle |k_d| <= calib_width / shape_d (unit normalisation)
    keep their values, a calibrationless operator reconstructs the centre by
    LSQR on the device, its centred FFT (the reference's default over the
    last three axes) is the Cartesian calibration data of
    :func:`cartesian_espirit`."""
    from .operator import MRIGB300

    like = _array.interface_of(kspace_data)
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    shape = tuple(int(s_) for s_ in shape)
    loc = _array.to_tensor(proper_trajectory(traj, normalize="unit"), dev, torch.float32)
    loc = loc.reshape(-1, len(shape))
    y = _array.to_tensor(kspace_data, dev, torch.complex64).reshape(-1, loc.shape[0])
    C = y.shape[0]
    cw = np.broadcast_to(np.asarray(calib_width, dtype=np.float64), (len(shape),))
    thr = torch.as_tensor(cw / np.asarray(shape, dtype=np.float64), dtype=loc.dtype, device=dev)
    keep = ((loc.abs() - thr) <= 0).all(dim=1)
    op = MRIGB300(loc[keep], shape, n_coils=C, squeeze_dims=True, device=dev.index)
    img = _array.to_tensor(op.pinv_solver(y[:, keep].contiguous(), max_iter=max_iter), dev,
                           torch.complex64).reshape(C, *shape)
    central = _cfft(img)
    maps = cartesian_espirit(central, shape, calib_width, kernel_width, thresh, crop, decim,
                             device=dev.index)
    return _array.from_tensor(maps, like)


METHODS = {"low_frequency": low_frequency, "espirit": espirit}
