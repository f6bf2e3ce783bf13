"""Generate the golden stacked-NUFFT fixtures from the mri-nufft reference itself.

Run in a container where the reference sources are present::

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_stacked_golden.py <mri-nufft src>

It imports ``mrinufft`` from the given source tree and runs the reference's
``MRIStackedNUFFT`` (``operators/stacked.py``) with its FP64 NDFT backend
``MRInumpy`` (float64 samples, complex128 outputs) as the 2D operator, on
small seeded cases: SENSE with a subset of planes, calibrationless with two
batches and an odd number of planes, and a 3D stacked trajectory whose planes
are recovered by ``traj3d2stacked``.  Stored per case: the 2D samples, shape,
z_index, coil maps (if any), an image, its forward transform, a k-space array
and its adjoint.
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
    from mrinufft.operators.interfaces.nudft_numpy import MRInumpy
    from mrinufft.operators.stacked import MRIStackedNUFFT, stacked2traj3d, traj3d2stacked

    out = {}

    def cplx(rng, shape):
        return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)

    specs = {
        "stack_sense": ((16, 12, 10), 200, 3, 1, np.array([0, 2, 3, 5, 7, 9]), True),
        "stack_calib": ((12, 14, 9), 150, 2, 2, None, False),
    }
    for name, (shape, M, C, B, zi, sense, ) in specs.items():
        rng = np.random.default_rng(len(name))
        s2 = rng.uniform(-0.5, 0.5, (M, 2))
        z_index = np.arange(shape[-1]) if zi is None else zi
        back = MRInumpy(s2, shape[:2], n_coils=C * len(z_index))
        back.squeeze_dims = True
        smaps = cplx(rng, (C, *shape)) if sense else None
        op = MRIStackedNUFFT(s2, shape, backend=back, smaps=smaps, z_index=z_index, n_coils=C,
                             n_batchs=B)
        x = cplx(rng, (B, *shape) if sense else (B, C, *shape))
        y = cplx(rng, (B, C, len(z_index) * M))
        out[f"{name}__samples"] = s2
        out[f"{name}__shape"] = np.array(shape)
        out[f"{name}__z_index"] = z_index
        out[f"{name}__n_coils"] = np.array(C)
        out[f"{name}__n_batchs"] = np.array(B)
        if sense:
            out[f"{name}__smaps"] = smaps
        out[f"{name}__img"] = x
        out[f"{name}__op"] = op.op(x)
        out[f"{name}__ksp"] = y
        out[f"{name}__adj"] = op.adj_op(y)

    # 3D stacked trajectory -> planes (reference helper)
    rng = np.random.default_rng(7)
    s2 = rng.uniform(-0.5, 0.5, (100, 2))
    zi = np.array([1, 4, 5, 8])
    s3 = stacked2traj3d(s2, zi, 10)
    t2, z2 = traj3d2stacked(s3, 10)
    out["traj3d__samples3d"] = s3
    out["traj3d__samples2d"] = t2
    out["traj3d__z_index"] = z2
    np.savez_compressed(HERE / "stacked_golden.npz", **out)
    print("wrote", HERE / "stacked_golden.npz", sorted(out))


if __name__ == "__main__":
    main(reference_src())
