"""Generate ``espirit_golden.npz`` from mri-nufft's own ESPIRiT code (run
where the reference sources are importable; not used at test time)::

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_espirit_golden.py <mri-nufft src>

The reference's ``cartesian_espirit`` (``extras/smaps.py:367-471``) raises
at its last masking step whenever ``decim == 1`` (its default): it multiplies
the (n_coils, *shape) maps in place by the power method's eigenvalue array
of shape (*shape[::-1], 1, 1), which does not broadcast (numpy:
"operands could not be broadcast together"); ``decim > 1`` needs
scikit-image, which is not installed.  The fixtures therefore run the
reference's steps one by one with its own functions (``_crop_or_pad``,
``_unfold_blocks``, ``fft`` / ``ifft`` of ``extras/cartesian.py``,
``power_method`` of ``operators/base.py``, ``_extract_kspace_center`` and an
``MRInumpy`` LSQR for the non-Cartesian front end of ``espirit``,
smaps.py:315-364, run in the backend's precision: float32 samples and
complex64 k-space) and apply the final mask per voxel, the broadcast-correct
form that the reference's ``decim > 1`` branch uses.  Stored per case: the
inputs, the maps before the mask, the eigenvalue per voxel and the masked
maps.  Both the 2D k-space FFT of ``espirit`` and the kernel iFFTs use the
reference's default ``dims=3``, which in 2D also transforms the coil axis;
the fixtures keep that behaviour.
"""

from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
from _refsrc import reference_src  # noqa: E402

HERE = Path(__file__).resolve().parent


def main(ref_src):
    os.environ.setdefault("PYTHONDONTWRITEBYTECODE", "1")
    sys.dont_write_bytecode = True
    sys.path.insert(0, ref_src)
    from mrinufft.extras.cartesian import fft, ifft
    from mrinufft.extras.smaps import _crop_or_pad, _extract_kspace_center, _unfold_blocks
    from mrinufft.operators.base import power_method
    from mrinufft.operators.interfaces.nudft_numpy import MRInumpy

    def espirit_steps(kspace, shape, calib_width, kernel_width, thresh, crop):
        # extras/smaps.py:393-463 with the reference's own helpers
        if isinstance(calib_width, int):
            calib_width = (calib_width,) * (kspace.ndim - 1)
        if isinstance(kernel_width, int):
            kernel_width = (kernel_width,) * (kspace.ndim - 1)
        n_coils = kspace.shape[0]
        calib = _crop_or_pad(kspace, (n_coils, *calib_width))
        calib = _unfold_blocks(calib, kernel_width)
        calib = calib.reshape(calib.shape[0], -1, np.prod(kernel_width))
        calib = calib.transpose(1, 0, 2).reshape(-1, calib.shape[0] * np.prod(kernel_width))
        _, S, VH = np.linalg.svd(calib, full_matrices=False)
        margin = float(np.min(np.abs(S / S.max() - thresh)))
        VH = VH[S > thresh * S.max(), :]
        kernels = VH.reshape((len(VH), n_coils, *kernel_width))
        AHA = np.zeros(kspace.shape[1:][::-1] + (n_coils, n_coils), dtype=kspace.dtype)
        for kernel in kernels:
            img_kernel = ifft(_crop_or_pad(kernel, kspace.shape))
            aH = np.expand_dims(img_kernel.T, axis=-1)
            a = np.conj(aH.swapaxes(-1, -2))
            AHA += aH @ a
        AHA *= np.prod(kspace.shape[1:]) / np.prod(kernel_width)
        Smaps = np.ones(kspace.shape[::-1] + (1,), dtype=kspace.dtype)
        max_eig, Smaps = power_method(
            operator=AHA.__matmul__, max_iter=100,
            norm_func=lambda x: np.sum(np.abs(x) ** 2, axis=-2, keepdims=True) ** 0.5, x=Smaps)
        Smaps = Smaps.T[0]
        Smaps *= np.conj(Smaps[0] / np.abs(Smaps[0]))
        eig = max_eig.T[0, 0]
        return Smaps, eig, Smaps * (eig > crop), len(VH), margin

    def phantom(rng, shape):
        g = np.meshgrid(*[np.linspace(-1, 1, n) for n in shape], indexing="ij")
        r2 = sum(x ** 2 for x in g)
        img = (r2 < 0.7).astype(np.complex128) * (1 + 0.3 * g[0])
        return img + 0.02 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))

    def maps(rng, shape, C):
        g = np.meshgrid(*[np.linspace(-1, 1, n) for n in shape], indexing="ij")
        out = []
        for c in range(C):
            ctr = rng.uniform(-0.8, 0.8, len(shape))
            d2 = sum((x - cc) ** 2 for x, cc in zip(g, ctr))
            out.append(np.exp(-d2 / 0.8) * np.exp(1j * (rng.uniform(0, 2 * np.pi) + sum(
                0.5 * rng.uniform(-1, 1) * x for x in g))))
        out = np.array(out)
        return out / np.sqrt(np.sum(np.abs(out) ** 2, axis=0))

    out = {}
    cases = {
        "cart2d": ((48, 48), 6, 24, 6),
        "cart3d": ((20, 18, 16), 5, 10, 4),
    }
    for i, (name, (shape, C, cw, kw)) in enumerate(cases.items()):
        rng = np.random.default_rng(30 + i)
        s = maps(rng, shape, C)
        ksp = fft(s * phantom(rng, shape), dims=len(shape))
        ksp = ksp.astype(np.complex64)
        sm, eig, masked, nk, margin = espirit_steps(ksp, shape, cw, kw, 0.02, 0.95)
        out[f"{name}__kspace"] = ksp
        out[f"{name}__shape"] = np.array(shape)
        out[f"{name}__calib_width"] = np.array(cw)
        out[f"{name}__kernel_width"] = np.array(kw)
        out[f"{name}__maps"] = sm
        out[f"{name}__eig"] = eig
        out[f"{name}__masked"] = masked
        print(name, "kernels", nk, "threshold margin", margin,
              "eig margin", float(np.min(np.abs(eig - 0.95))))

    # non-Cartesian front end of espirit (smaps.py:340-364) on a radial trajectory
    rng = np.random.default_rng(40)
    shape, C = (40, 40), 4
    nc, ns = 48, 40
    seg = np.linspace(0, 0.5, ns)
    ang = 2 * np.pi * np.arange(nc) / nc
    traj = np.stack([np.outer(np.cos(ang), seg), np.outer(np.sin(ang), seg)], -1).reshape(-1, 2)
    s = maps(rng, shape, C)
    img = phantom(rng, shape)
    y = MRInumpy(traj, shape, n_coils=C, smaps=s).op(img)
    y = y + 0.001 * (rng.standard_normal(y.shape) + 1j * rng.standard_normal(y.shape))
    cw, kw = 16, 5
    # the front end in the backend's precision (float32 samples, complex64
    # data): the reference's LSQR itself moves by 5e-3 between complex64 and
    # complex128 on this system after 10 iterations
    y = y.astype(np.complex64)
    k_space, samples, _ = _extract_kspace_center(
        kspace_data=y, kspace_loc=traj.astype(np.float32),
        threshold=tuple(float(v) for v in cw / np.asarray(shape)), density=None, window_fun="rect")
    nufft = MRInumpy(samples, shape, n_coils=k_space.shape[-2])
    nufft.squeeze_dims = True
    img_c = nufft.pinv_solver(k_space, max_iter=10)
    central = fft(img_c)
    sm, eig, masked, nk, margin = espirit_steps(central.astype(np.complex64), shape, cw, kw, 0.02, 0.95)
    out["radial__samples"] = traj.astype(np.float32)
    out["radial__kspace"] = y
    out["radial__shape"] = np.array(shape)
    out["radial__calib_width"] = np.array(cw)
    out["radial__kernel_width"] = np.array(kw)
    out["radial__center_img"] = np.asarray(img_c)
    out["radial__central"] = central
    out["radial__maps"] = sm
    out["radial__eig"] = eig
    out["radial__masked"] = masked
    print("radial kernels", nk, "threshold margin", margin, "eig margin", float(np.min(np.abs(eig - 0.95))))
    np.savez_compressed(HERE / "espirit_golden.npz", **out)
    print("wrote", HERE / "espirit_golden.npz")


if __name__ == "__main__":
    main(reference_src())
