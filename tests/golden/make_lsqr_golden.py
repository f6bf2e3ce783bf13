"""Generate golden LSQR reconstructions from the mri-nufft reference itself.

Run in a container where the reference sources are present::

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_lsqr_golden.py <mri-nufft src>

It imports ``mrinufft`` from the given source tree and runs the reference's
``lsqr`` (``extras/optim.py``) for 10 iterations on its FP64 NDFT backend
``MRInumpy`` (float64 samples, complex128): a SENSE case, a damped case
with a prior x0, and a calibrationless two-batch case.  Stored per case: the
operator inputs, the k-space data and the reconstruction.
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
    from mrinufft.extras.optim import lsqr
    from mrinufft.operators.interfaces.nudft_numpy import MRInumpy

    def cplx(rng, shape):
        return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)

    out = {}
    specs = {
        "lsqr_sense": ((24, 20), 600, 2, 1, True, 0.0),
        "lsqr_damp": ((20, 16), 500, 2, 1, True, 0.5),
        "lsqr_calib": ((16, 18), 400, 2, 2, False, 0.0),
    }
    for name, (shape, M, C, B, sense, damp) in specs.items():
        rng = np.random.default_rng(len(name) + 11)
        s = rng.uniform(-0.5, 0.5, (M, 2))
        smaps = cplx(rng, (C, *shape)) if sense else None
        op = MRInumpy(s, shape, n_coils=C, smaps=smaps)
        op.n_batchs = B
        op.squeeze_dims = False
        y = cplx(rng, (B, C, M))
        x0 = cplx(rng, (B, 1 if sense else C, *shape)) if damp else None
        x = lsqr(op, y, damp=damp, x0=x0, max_iter=10, progressbar=False)
        out[f"{name}__samples"] = s
        out[f"{name}__shape"] = np.array(shape)
        out[f"{name}__n_coils"] = np.array(C)
        out[f"{name}__n_batchs"] = np.array(B)
        out[f"{name}__damp"] = np.array(damp)
        if sense:
            out[f"{name}__smaps"] = smaps
        if x0 is not None:
            out[f"{name}__x0"] = x0
        out[f"{name}__ksp"] = y
        out[f"{name}__x"] = np.asarray(x)
    np.savez_compressed(HERE / "lsqr_golden.npz", **out)
    print("wrote", HERE / "lsqr_golden.npz", sorted(out))


if __name__ == "__main__":
    main(reference_src())
