"""Off-resonance corrected NUFFT on the GB300 library.

Restates mri-nufft's ``MRIFourierCorrected``
(``src/mrinufft/operators/off_resonance.py:24-444``): with time interpolators
B (NK x L) and spatial interpolators C (L x image) from a factorisation of
exp(field_map * t),

    y = sum_l B_l * A(C_l x),        A^H y = sum_l conj(C_l) A^H(conj(B_l) y).

The L interpolators run as extra "coils" of the plain operator: one
``gbn_op`` / ``gbn_adj`` call over L * C transforms whose coil maps are the
products C_l s_c (calibrationless: C_l per coil image), plus one
``gbn_orc_reduce`` / ``gbn_orc_expand`` pass for the B weights.  The
factorisations ("svd", "mti") restate ``src/mrinufft/extras/field_map.py``
(176-513) on the host; mri-nufft's own methods are used when it is
installed and a method is named that is not restated here.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _array, _lib
from .plan import _ptr


def get_complex_fieldmap_rad(b0_map, r2star_map=None):
    """Complex field map in rad/s: 2j pi b0 (+ R2*), field_map.py:176-212."""
    b0 = np.asarray(b0_map)
    if np.iscomplexobj(b0):
        return b0
    fm = np.complex64(2j * np.pi) * b0.astype(np.float32, copy=False)
    if r2star_map is not None:
        fm = fm + np.asarray(r2star_map, dtype=np.float32)
    return fm


def _create_histogram(field_map, mask, n_bins=1024):
    """Histogram of the (masked) complex field map (field_map.py:215-258)."""
    masked = field_map[mask] if mask is not None else field_map.ravel()
    if isinstance(n_bins, int):
        dR = np.max(masked.real) - np.min(masked.real)
        dI = np.max(masked.imag) - np.min(masked.imag)
        if dI == 0:
            n_bins = (n_bins, 1)
        elif dR == 0:
            n_bins = (1, n_bins)
        else:
            nr = np.maximum(1, int(np.around(n_bins * dR / dI)))
            n_bins = (int(nr), int(np.around(n_bins / nr)))
    z = np.ascontiguousarray(masked.astype(np.complex64)).view(np.float32).reshape(-1, 2)
    counts, edges = np.histogramdd(z, bins=n_bins)
    centers = [e[1:] - (e[1] - e[0]) / 2 for e in edges]
    return counts, np.add.outer(centers[0], 1j * centers[1]).astype(np.complex64)


def _full_c(field_map, c_small, n_bins):
    """Spatial interpolators at every voxel from their histogram-bin values
    (field_map.py:303-359)."""
    fr, fi = field_map.real.ravel(), field_map.imag.ravel()
    minr, maxr, mini, maxi = fr.min(), fr.max(), fi.min(), fi.max()
    dr, di = (maxr - minr) / n_bins[0], (maxi - mini) / n_bins[1]
    idxr = np.zeros(fr.shape, dtype=int)
    idxi = np.zeros(fi.shape, dtype=int)
    if dr != 0:
        idxr = np.clip(np.around((fr - minr) / dr).astype(int), 0, n_bins[0] - 1)
    if di != 0:
        idxi = np.clip(np.around((fi - mini) / di).astype(int), 0, n_bins[1] - 1)
    c_sr = c_small.reshape(-1, *n_bins)
    return np.ascontiguousarray(c_sr[:, idxr, idxi].reshape(-1, *field_map.shape))


def compute_svd_coefficients(field_map, readout_time, mask, L=-1, n_bins=1024):
    """B, C by a truncated SVD of the histogram-weighted phase matrix, C by
    least squares (field_map.py:381-439; full SVD here)."""
    field_map = get_complex_fieldmap_rad(field_map)
    h_k, w_k = _create_histogram(field_map, mask, n_bins)
    shape_h = h_k.shape
    w_k, h_k = w_k.ravel(), h_k.ravel()
    t = np.asarray(readout_time).ravel()
    E = np.exp(np.outer(t, w_k))
    Ew = np.sqrt(h_k) * E
    if L == -1:
        L = max(1, int(np.ceil(abs(w_k[-1] - w_k[0]) * np.max(t) / 2 * np.pi)))
    u, _, _ = np.linalg.svd(Ew, full_matrices=False)
    B = u[:, :L]
    C, _, _, _ = np.linalg.lstsq(B, E, rcond=None)
    return B, _full_c(field_map, C, shape_h), E


def compute_mti_coefficients(field_map, readout_time, mask, L=-1, n_bins=1024):
    """Mixed time interpolation: C = exp(t_l w), B by least squares
    (field_map.py:442-500)."""
    field_map = get_complex_fieldmap_rad(field_map)
    h_k, w_k = _create_histogram(field_map, mask, n_bins)
    shape_h = h_k.shape
    h_k, w_k = h_k.ravel(), w_k.ravel()
    t = np.asarray(readout_time).ravel()
    if L == -1:
        L = max(1, int(np.ceil(2 * abs(w_k[-1] - w_k[0]) * np.max(t) / np.pi)))
    t_l = np.linspace(np.min(t), np.max(t), L, dtype=np.float32)
    C = np.exp(np.outer(t_l, w_k))
    E = np.exp(np.outer(t, w_k))
    B, _, _, _ = np.linalg.lstsq((np.sqrt(h_k) * C).T, (np.sqrt(h_k) * E).T, rcond=None)
    return B.T, _full_c(field_map, C, shape_h), E


FACTORISATIONS = {"svd": compute_svd_coefficients, "mti": compute_mti_coefficients}


class MRIFourierCorrectedGB300:
    """Off-resonance corrected operator around an ``MRIGB300``.

    Arguments follow ``MRIFourierCorrected(fourier_op, b0_map, readout_time,
    r2star_map, mask, interpolator)``; ``interpolator`` is "svd", "mti", a
    ``{"name": ..., **kwargs}`` dict or a ``(B, C)`` tuple.
    """

    def __init__(self, fourier_op, b0_map=None, readout_time=None, r2star_map=None, mask=None,
                 interpolator="svd"):
        self._fourier_op = fourier_op
        self.squeeze_dims = fourier_op.squeeze_dims
        self._fourier_op.squeeze_dims = False
        if b0_map is None and readout_time is None and not isinstance(interpolator, tuple):
            raise ValueError("b0_map  and readout_time required for off-resonance correction.")
        self.lib = _lib.load()
        fm = None if b0_map is None else get_complex_fieldmap_rad(b0_map, r2star_map)
        self.compute_interpolator(interpolator, fm, readout_time, mask)

    def __getattr__(self, name):
        return getattr(self._fourier_op, name)

    # ------------------------------------------------------------ interpolators
    def compute_interpolator(self, interpolators, field_map, readout_time, mask):
        """Set the time (B) and space (C) interpolators (off_resonance.py:109-197)."""
        op = self._fourier_op
        M = op.n_samples
        if field_map is not None and tuple(field_map.shape) != tuple(op.shape):
            # resize to the image grid (linear for the map, nearest for the mask)
            from scipy.ndimage import zoom

            f = tuple(np.array(op.shape) / np.array(field_map.shape))
            field_map = zoom(field_map, zoom=f, order=1)
            if mask is not None:
                mask = zoom(np.asarray(mask), zoom=f, order=0)
        self._field_map, self.mask, self.readout_time = field_map, mask, readout_time
        self.interpolator_method = interpolators
        self._t_dev = None
        if isinstance(interpolators, tuple):
            B, C = (np.asarray(_array.to_tensor(a, torch.device("cpu"), torch.complex64))
                    for a in interpolators)
            if M % B.shape[0]:
                raise ValueError("Time interpolator should divide or equal size of the samples.")
        else:
            t = np.asarray(readout_time).ravel()
            if M % t.size:
                raise ValueError("readout_time should divide or equal the size of the samples.")
            if np.all(field_map == 0) or np.all(t == 0):
                B = np.ones((t.size, 1), np.complex64)
                C = np.ones((1, *op.shape), np.complex64)
            else:
                kwargs = {}
                if isinstance(interpolators, dict):
                    kwargs = dict(interpolators)
                    interpolators = kwargs.pop("name")
                if isinstance(interpolators, str):
                    fn = FACTORISATIONS.get(interpolators)
                    if fn is None:
                        from mrinufft.extras import get_orc_factorization  # type: ignore

                        fn = get_orc_factorization(interpolators)
                else:
                    fn = interpolators
                B, C, _ = fn(field_map=field_map, readout_time=t, mask=mask, **kwargs)
                B, C = np.asarray(B), np.asarray(C)
        self.n_shots = M // B.shape[0]
        dev = op.device
        self.B = torch.from_numpy(np.ascontiguousarray(B, dtype=np.complex64)).to(dev)
        self.C = torch.from_numpy(np.ascontiguousarray(C, dtype=np.complex64)).to(dev).reshape(-1, *op.shape)
        self._maps = None

    def update_field_map(self, new_field_map):
        """Recompute the interpolators for a new complex field map with the
        same method, readout time and mask (off_resonance.py:199-206)."""
        if isinstance(new_field_map, torch.Tensor):
            new_field_map = new_field_map.detach().cpu().numpy()
        self.compute_interpolator(self.interpolator_method, np.asarray(new_field_map),
                                  self.readout_time, self.mask)

    @property
    def field_map(self):
        """The complex field map (rad/s) the interpolators were computed from."""
        return self._field_map

    @field_map.setter
    def field_map(self, new_field_map):
        self.update_field_map(new_field_map)

    @property
    def full_readout_time(self):
        """``repeat(readout_time, n_shots)`` as off_resonance.py:218-222."""
        return np.repeat(np.asarray(self.readout_time), self.n_shots)

    def _sample_times(self):
        """(M,) float32 device tensor: the readout time of every sample in the
        layout ``op`` weights by ``B`` (sample m at time index m mod NK)."""
        if self.readout_time is None:
            raise ValueError("the operator has no readout time")
        if self._t_dev is None:
            t = np.asarray(self.readout_time, dtype=np.float32).ravel()
            self._t_dev = torch.from_numpy(np.tile(t, self.n_shots)).to(self._fourier_op.device)
        return self._t_dev

    autograd_available = True

    def make_autograd(self, *, wrt_data=True, wrt_traj=False, wrt_field_map=False,
                      paired_batch=False):
        """Differentiable wrapper (off_resonance.py:397-444)."""
        from .autodiff import MRINufftAutoGrad

        return MRINufftAutoGrad(self, wrt_data=wrt_data, wrt_traj=wrt_traj,
                                wrt_field_map=wrt_field_map, paired_batch=paired_batch)

    @property
    def n_interpolators(self):
        return self.B.shape[1]

    @property
    def n_samples_per_shot(self):
        return self.B.shape[0]

    def _effective_maps(self):
        """C_l s_c for every (l, c), interpolator major (SENSE), or C_l."""
        op = self._fourier_op
        if op._smaps is None:
            return self.C
        if self._maps is None or self._maps.shape[0] != self.C.shape[0] * op._smaps.shape[0]:
            self._maps = (self.C[:, None] * op._smaps[None]).reshape(-1, *op.shape).contiguous()
        return self._maps

    def _st(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self._fourier_op.device).cuda_stream)

    # -------------------------------------------------------------- operators
    def _op_device(self, x):
        op = self._fourier_op
        B, C, M, L = op.n_batchs, op.n_coils, op.n_samples, self.n_interpolators
        maps = self._effective_maps()
        sense = op._smaps is not None
        nb, cc = (B, C) if sense else (B * C, 1)
        x = x.reshape((B, *op.shape) if sense else (B * C, *op.shape))
        yl = torch.empty((nb, L * cc, M), dtype=torch.complex64, device=op.device)
        op._plan.op(x, maps, yl, nb, L * cc, op.inv_norm_factor, isign=op._isign)
        y = torch.empty((B, C, M), dtype=torch.complex64, device=op.device)
        _lib.check(self.lib.gbn_orc_reduce(_ptr(yl), _ptr(self.B), _ptr(y), nb, L, cc, M,
                                           self.n_samples_per_shot, self._st()), "gbn_orc_reduce")
        return y

    def _adj_device(self, y):
        op = self._fourier_op
        B, C, M, L = op.n_batchs, op.n_coils, op.n_samples, self.n_interpolators
        maps = self._effective_maps()
        sense = op._smaps is not None
        nb, cc = (B, C) if sense else (B * C, 1)
        y = y.reshape(nb, cc, M)
        yl = torch.empty((nb, L * cc, M), dtype=torch.complex64, device=op.device)
        _lib.check(self.lib.gbn_orc_expand(_ptr(y), _ptr(self.B), _ptr(yl), nb, L, cc, M,
                                           self.n_samples_per_shot, self._st()), "gbn_orc_expand")
        out = torch.empty((B, 1, *op.shape) if sense else (B, C, *op.shape), dtype=torch.complex64,
                          device=op.device)
        op._plan.adj(yl, op._density, maps, out, nb, L * cc, op.inv_norm_factor, isign=-op._isign)
        return out

    def _grad_field_map(self, img, k, adjoint):
        """Gradient of a real loss with respect to the complex field map.

        For ``y = E(f) x`` with ``E_mn = A_mn exp(f_n t_m)`` (holomorphic in f)
        the cotangent ``dy`` gives ``conj(x) * E^H(t dy)``; for the adjoint
        ``x = E(f)^H y`` (anti-holomorphic in f) the cotangent ``dx`` gives
        ``conj(dx) * E^H(t y)`` (autodiff.py:44-56, 89-100; the forward case
        conjugates the image, which is the exact derivative).  E^H is the
        corrected adjoint; the sum runs over batch items and, without maps,
        coils.  ``img`` is ``x`` (forward) or ``dx`` (adjoint), ``k`` is
        ``dy`` (forward) or ``y`` (adjoint).
        """
        op = self._fourier_op
        B, C, M = op.n_batchs, op.n_coils, op.n_samples
        k = k.reshape(B, C, M) * self._sample_times()
        g = self._adj_device(k)
        img = img.reshape(g.shape)
        return (torch.conj(img) * g).sum(dim=(0, 1)).reshape(op.shape)

    def _grad_traj(self, img, k, adjoint):
        """Trajectory gradient of the corrected forward (``adjoint=False``:
        ``img`` = x, ``k`` = dy) or adjoint (``img`` = dx, ``k`` = y)
        operator: the plain kernel-derivative interpolation over the L * C
        effective maps ``C_l s_c`` with ``conj(B_l) k`` as the k-space input,
        which is the exact derivative of ``sum_l B_l A(C_l s x)`` and of its
        adjoint."""
        op = self._fourier_op
        B, C, M, L = op.n_batchs, op.n_coils, op.n_samples, self.n_interpolators
        maps = self._effective_maps()
        sense = op._smaps is not None
        nb, cc = (B, C) if sense else (B * C, 1)
        img = img.reshape(nb, *op.shape)
        kl = torch.empty((nb, L * cc, M), dtype=torch.complex64, device=op.device)
        _lib.check(self.lib.gbn_orc_expand(_ptr(k.reshape(nb, cc, M).contiguous()), _ptr(self.B),
                                           _ptr(kl), nb, L, cc, M, self.n_samples_per_shot,
                                           self._st()), "gbn_orc_expand")
        grad = torch.empty((M, len(op.shape)), dtype=torch.float32, device=op.device)
        fn = op.plan.grad_traj_adj if adjoint else op.plan.grad_traj_op
        fn(img.contiguous(), maps, kl, grad, nb, L * cc, op.inv_norm_factor)
        return grad

    def _squeeze(self, arr):
        if self.squeeze_dims:
            if arr.ndim > 1 and arr.shape[1] == 1:
                arr = arr.squeeze(1)
            if arr.ndim > 0 and arr.shape[0] == 1:
                arr = arr.squeeze(0)
        return arr

    def op(self, data, *args):
        """Forward operator with the off-resonance effect (off_resonance.py:233-282)."""
        like = _array.interface_of(data)
        x = _array.to_tensor(data, self._fourier_op.device, torch.complex64)
        return _array.from_tensor(self._squeeze(self._op_device(x)), like)

    def adj_op(self, coeffs, *args):
        """Adjoint operator with the off-resonance effect (off_resonance.py:284-332)."""
        like = _array.interface_of(coeffs)
        y = _array.to_tensor(coeffs, self._fourier_op.device, torch.complex64)
        return _array.from_tensor(self._squeeze(self._adj_device(y)), like)

    def data_consistency(self, image_data, obs_data):
        like = _array.interface_of(image_data)
        op = self._fourier_op
        x = _array.to_tensor(image_data, op.device, torch.complex64)
        y = _array.to_tensor(obs_data, op.device, torch.complex64).reshape(op.n_batchs, op.n_coils, -1)
        return _array.from_tensor(self._squeeze(self._adj_device(self._op_device(x) - y)), like)

    def get_lipschitz_cst(self, max_iter=10, **kwargs):
        """Power method on the corrected operator with one coil and no maps
        (off_resonance.py:340-388), FP64 norms on the device."""
        from .plan import norm2_f64

        op = self._fourier_op
        smaps, C, B = op._smaps, op._n_coils, op._n_batchs
        op._smaps, op._n_coils, op._n_batchs = None, 1, 1
        self._maps = None
        try:
            x = 1j * np.random.random(op.shape).astype(np.complex64)
            x += np.random.random(op.shape).astype(np.complex64)
            x = torch.from_numpy(x).to(op.device).reshape(1, *op.shape)
            x_norm = float(norm2_f64(x).sqrt())
            x = x / x_norm
            x_new_norm = x_norm
            for _ in range(max_iter):
                x_new = self._adj_device(self._op_device(x)).reshape(1, *op.shape)
                x_new_norm = float(norm2_f64(x_new).sqrt())
                x_new = x_new / x_new_norm
                if abs(x_norm - x_new_norm) < 1e-6:
                    break
                x_norm = x_new_norm
                x = x_new
            return x_new_norm
        finally:
            op._smaps, op._n_coils, op._n_batchs = smaps, C, B
            self._maps = None

    def _op(self, image, coeffs):
        return self._fourier_op._op(image, coeffs)

    def _adj_op(self, coeffs, image):
        return self._fourier_op._adj_op(coeffs, image)
