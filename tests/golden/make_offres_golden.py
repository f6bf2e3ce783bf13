"""Generate the golden off-resonance fixtures from the mri-nufft reference itself.

Run in a container where the reference sources are present::

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_offres_golden.py <mri-nufft src>

It imports ``mrinufft`` from the given source tree and runs the reference's
``MRIFourierCorrected`` (``operators/off_resonance.py``) around its FP64 NDFT
backend ``MRInumpy`` on small seeded cases: explicit (B, C) interpolators
(set as the operator's attributes) with SENSE maps, the "svd" factorisation without maps, and the "mti"
factorisation in 3D.  Stored per case: samples, shape, maps, field map,
readout time, the interpolators the reference used, an image, its forward
transform, a k-space array and its adjoint.
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
    from mrinufft.operators.off_resonance import MRIFourierCorrected

    def cplx(rng, shape):
        return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)

    specs = {
        "orc_tuple": ((16, 12), 2, True, "tuple"),
        "orc_svd": ((16, 12), 2, False, "svd"),
        "orc_mti3d": ((8, 10, 6), 2, True, "mti"),
    }
    out = {}
    for name, (shape, C, sense, method) in specs.items():
        rng = np.random.default_rng(len(name) + 3)
        NK, NS = 40, 6
        s = rng.uniform(-0.5, 0.5, (NS * NK, len(shape)))
        smaps = cplx(rng, (C, *shape)) if sense else None
        op = MRInumpy(s, shape, n_coils=C, smaps=smaps)
        op.squeeze_dims = False
        b0 = rng.uniform(-60.0, 60.0, shape)
        t = np.linspace(0.0, 6e-3, NK)
        cor = MRIFourierCorrected(op, b0_map=b0, readout_time=t,
                                  interpolator="svd" if method == "tuple" else method)
        if method == "tuple":
            # explicit interpolators set on the operator (its tuple argument
            # does not survive the array-module decorator in this version)
            L = 4
            cor.B, cor.C = cplx(rng, (NK, L)), cplx(rng, (L, *shape))
        x = cplx(rng, (1, 1, *shape) if sense else (1, C, *shape))
        y = cplx(rng, (1, C, NS * NK))
        out[f"{name}__samples"] = s
        out[f"{name}__shape"] = np.array(shape)
        if sense:
            out[f"{name}__smaps"] = smaps
        out[f"{name}__n_coils"] = np.array(C)
        out[f"{name}__b0"] = b0
        out[f"{name}__t"] = t
        out[f"{name}__B"] = np.asarray(cor.B)
        out[f"{name}__C"] = np.asarray(cor.C[:] if hasattr(cor.C, "__getitem__") else cor.C)
        out[f"{name}__img"] = x
        out[f"{name}__op"] = cor.op(x)
        out[f"{name}__ksp"] = y
        out[f"{name}__adj"] = cor.adj_op(y)
    np.savez_compressed(HERE / "offres_golden.npz", **out)
    print("wrote", HERE / "offres_golden.npz", sorted(out))


if __name__ == "__main__":
    main(reference_src())
