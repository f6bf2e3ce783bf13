"""Generate the golden Toeplitz fixtures from the mri-nufft reference itself.

Run in a container where the reference sources are present::

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_toeplitz_golden.py <mri-nufft src>

It imports ``mrinufft`` from the given source tree and, on the reference's FP64
NDFT backend ``MRInumpy`` (``operators/interfaces/nudft_numpy.py``, float64
samples, complex128 outputs), runs the reference's own Toeplitz code
(``operators/toeplitz.py``: ``compute_toeplitz_kernel`` with explicit weights,
``apply_toeplitz_kernel``) on small seeded 2D and 3D cases.  Stored per case:
samples, shape, weights (ones when the case has none), the real kernel
spectrum on the 2N grid, an input image and its Gram product.
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
    from mrinufft.operators.toeplitz import apply_toeplitz_kernel, compute_toeplitz_kernel

    specs = {
        "toep2D_w": ((16, 20), 300, True, 1),
        "toep2D": ((16, 16), 250, False, 2),
        "toep3D_w": ((8, 10, 12), 400, True, 3),
    }
    out = {}
    for name, (shape, M, weighted, seed) in specs.items():
        rng = np.random.default_rng(seed)
        s = rng.uniform(-0.5, 0.5, (M, len(shape)))
        w = rng.uniform(0.5, 1.5, M) if weighted else np.ones(M)
        op = MRInumpy(s, shape)
        kernel = compute_toeplitz_kernel(op, w.astype(np.complex128))
        x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        gram = apply_toeplitz_kernel(x, kernel)
        out[f"{name}__samples"] = s
        out[f"{name}__shape"] = np.array(shape)
        out[f"{name}__weights"] = w
        out[f"{name}__kernel"] = kernel
        out[f"{name}__img"] = x
        out[f"{name}__gram"] = gram
    np.savez_compressed(HERE / "toeplitz_golden.npz", **out)
    print("wrote", HERE / "toeplitz_golden.npz", sorted(out))


if __name__ == "__main__":
    main(reference_src())
