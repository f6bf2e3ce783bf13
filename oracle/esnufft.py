"""CPU ES-kernel NUFFT (C spreader + scipy FFT) — TEST INFRASTRUCTURE ONLY.

A restatement of the finufft algorithm that mri-nufft's CPU backend calls
(``src/mrinufft/operators/interfaces/finufft.py:23-80``, pipe 195-245):

* type 2: pad x_n / phihat(n) into the fine grid, forward FFT, interpolate;
* type 1: spread, inverse FFT, crop and divide by phihat(n);
* pipe:   spread / interpolate on the N grid (no FFT, no deapodisation).

Used as the checker of the GPU pipe density and as the timed CPU baseline
(``float32`` variant with OpenMP threads and ``scipy.fft`` workers).
"""

from __future__ import annotations

import ctypes
import math
import os

import numpy as np
import scipy.fft

from . import build as _build

_lib = None


def _load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(str(_build.build()))
        for sfx, real in (("_d", ctypes.c_double), ("_f", ctypes.c_float)):
            rp = ctypes.POINTER(real)
            for name in ("es_interp", "es_spread"):
                fn = getattr(lib, name + sfx)
                fn.restype = None
                fn.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int64), ctypes.c_int64,
                               rp, rp, rp, rp, rp, ctypes.c_int, ctypes.c_double, ctypes.c_int]
        _lib = lib
    return _lib


def kernel_params(eps, sigma=2.0):
    """Published ES rules (see the module docstring of ``esnufft.c``)."""
    if sigma == 2.0:
        w = math.ceil(-math.log10(eps / 10.0))
    else:
        w = math.ceil(-math.log(eps) / (math.pi * math.sqrt(1.0 - 1.0 / sigma)))
    w = max(2, min(16, w))
    if sigma == 2.0:
        beta = {2: 2.20, 3: 2.26, 4: 2.38}.get(w, 2.30) * w
    else:
        beta = 0.97 * math.pi * w * (1.0 - 1.0 / (2.0 * sigma))
    return w, beta


def _smooth_even(n):
    n += n % 2
    while True:
        r = n
        for p in (2, 3, 5):
            while r % p == 0:
                r //= p
        if r == 1:
            return n
        n += 2


def phihat(N, nf, w, beta):
    """phihat(k) = int phi(x) cos(2 pi k x / nf) dx for modes k = i - N//2 (FP64)."""
    x, wt = np.polynomial.legendre.leggauss(2 * w + 48)
    h = 0.5 * w
    xs = h * x
    f = np.exp(beta * (np.sqrt(np.maximum(1 - (xs / h) ** 2, 0)) - 1)) * h * wt
    k = np.arange(N) - N // 2
    return np.cos(2 * np.pi * np.outer(k, xs) / nf) @ f


class EsNufft:
    """Type-1 / type-2 NUFFT of one image shape on the CPU."""

    def __init__(self, samples_pi, shape, eps=1e-6, upsampfac=2.0, dtype=np.float64,
                 nthreads=None, spread_only=False):
        self.shape = tuple(int(s) for s in shape)
        self.d = len(self.shape)
        self.w, self.beta = kernel_params(eps, upsampfac)
        if spread_only:
            self.nf = self.shape
        else:
            self.nf = tuple(_smooth_even(max(math.ceil(upsampfac * n), 2 * self.w)) for n in self.shape)
        self.real = np.dtype(dtype)
        self.cpx = np.dtype(np.complex128 if self.real == np.float64 else np.complex64)
        self.sfx = "_d" if self.real == np.float64 else "_f"
        self.nthreads = nthreads or os.cpu_count() or 1
        k = np.asarray(samples_pi, dtype=self.real).reshape(-1, self.d)
        self.cols = [np.ascontiguousarray(k[:, i]) for i in range(self.d)]
        while len(self.cols) < 3:
            self.cols.append(self.cols[0])
        self.M = k.shape[0]
        if not spread_only:
            ph = [phihat(n, f, self.w, self.beta) for n, f in zip(self.shape, self.nf)]
            dec = ph[0]
            for p in ph[1:]:
                dec = np.multiply.outer(dec, p)
            self.inv_phihat = (1.0 / dec).astype(self.real)

    def _ptr(self, a):
        return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double if self.real == np.float64 else ctypes.c_float))

    def interp(self, grid):
        grid = np.ascontiguousarray(grid, dtype=self.cpx)
        y = np.empty(self.M, dtype=self.cpx)
        lib = _load()
        nf = (ctypes.c_int64 * 3)(*(list(self.nf) + [1] * (3 - self.d)))
        getattr(lib, "es_interp" + self.sfx)(
            self.d, nf, self.M, self._ptr(self.cols[0]), self._ptr(self.cols[1]),
            self._ptr(self.cols[2]), self._ptr(grid.view(self.real)), self._ptr(y.view(self.real)),
            self.w, self.beta, self.nthreads)
        return y

    def spread(self, c):
        c = np.ascontiguousarray(c, dtype=self.cpx)
        grid = np.zeros(self.nf, dtype=self.cpx)
        lib = _load()
        nf = (ctypes.c_int64 * 3)(*(list(self.nf) + [1] * (3 - self.d)))
        getattr(lib, "es_spread" + self.sfx)(
            self.d, nf, self.M, self._ptr(self.cols[0]), self._ptr(self.cols[1]),
            self._ptr(self.cols[2]), self._ptr(c.view(self.real)), self._ptr(grid.view(self.real)),
            self.w, self.beta, self.nthreads)
        return grid

    def _fine_index(self):
        return tuple(np.arange(n) - n // 2 for n in self.shape)

    def type2(self, x, isign=-1):
        """y_j = sum_n x_n exp(isign i k_j . n)."""
        fine = np.zeros(self.nf, dtype=self.cpx)
        idx = np.ix_(*[np.mod(m, f) for m, f in zip(self._fine_index(), self.nf)])
        fine[idx] = np.asarray(x, dtype=self.cpx) * self.inv_phihat
        if isign < 0:
            fine = scipy.fft.fftn(fine, workers=self.nthreads, overwrite_x=True)
        else:
            fine = scipy.fft.ifftn(fine, workers=self.nthreads, overwrite_x=True, norm="forward")
        return self.interp(fine)

    def type1(self, c, isign=1):
        """x_n = sum_j c_j exp(isign i k_j . n)."""
        fine = self.spread(c)
        if isign > 0:
            fine = scipy.fft.ifftn(fine, workers=self.nthreads, overwrite_x=True, norm="forward")
        else:
            fine = scipy.fft.fftn(fine, workers=self.nthreads, overwrite_x=True)
        idx = np.ix_(*[np.mod(m, f) for m, f in zip(self._fine_index(), self.nf)])
        return (fine[idx] * self.inv_phihat).astype(self.cpx)


def pipe(samples_pi, shape, max_iter=10, osf=2.0, normalize=True, eps=1e-6, nthreads=None):
    """Pipe density (finufft.py:195-245) on the CPU, FP64."""
    grid = EsNufft(samples_pi, shape, eps=eps, upsampfac=osf, spread_only=True, nthreads=nthreads)
    nrm = np.sqrt(np.prod(shape) * 2 ** len(shape))
    w = np.ones(grid.M, dtype=np.complex128)
    for _ in range(max_iter):
        v = grid.interp(grid.spread(w)) / (nrm * nrm)
        w = w / np.abs(v)
    if normalize:
        full = EsNufft(samples_pi, shape, eps=eps, nthreads=nthreads)
        y = full.type2(np.ones(shape)) / nrm
        recon = full.type1(w * y) / nrm
        w = w / np.mean(np.abs(recon))
    return np.abs(w)
