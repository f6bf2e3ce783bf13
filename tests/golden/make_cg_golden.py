"""Generate golden CG reconstructions and Lipschitz estimates from the
mri-nufft reference itself (run where the reference sources are importable;
not used at test time)::

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_cg_golden.py <mri-nufft src>

Every case runs on the reference's FP64 NDFT backend ``MRInumpy`` (float64
samples, complex128).  The Lipschitz estimate is the reference's GPU-backend
procedure (``interfaces/cufinufft.py:1239-1279``: single coil, no maps, the
seeded start vector ``1j * U + U`` from numpy's global generator, then the
reference's own ``power_method``, ``operators/base.py:1155-1221``), which is
the procedure the GB300 backend mirrors; ``MRInumpy.get_lipschitz_cst`` is
bound to it for these runs.  CG is the reference's ``cg``
(``extras/optim.py:801-902``, 10 iterations) with that estimate, started
after ``np.random.seed(seed)``.  Stored per case: the operator inputs, the
seed, the k-space data, the estimate and the reconstruction.
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
    from mrinufft.extras.optim import cg
    from mrinufft.operators.base import power_method
    from mrinufft.operators.interfaces.nudft_numpy import MRInumpy

    def lipschitz_gpu_backend(self, max_iter=10, **kwargs):
        n_coils, n_batchs, smaps, sq = self.n_coils, self.n_batchs, self.smaps, self.squeeze_dims
        self.smaps = None
        self.n_coils = 1
        self.n_batchs = 1
        self.squeeze_dims = True
        x = 1j * np.random.random(self.shape).astype(self.cpx_dtype, copy=False)
        x += np.random.random(self.shape).astype(self.cpx_dtype, copy=False)
        L, _ = power_method(max_iter, self, norm_func=lambda v: np.linalg.norm(v.flatten()), x=x)
        self.n_coils, self.n_batchs, self.smaps, self.squeeze_dims = n_coils, n_batchs, smaps, sq
        return L

    MRInumpy.get_lipschitz_cst = lipschitz_gpu_backend

    def cplx(rng, shape):
        return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)

    out = {}
    # name: shape, M, coils, batches, sense, density, damp, x0
    specs = {
        "cg_sense": ((24, 20), 600, 2, 1, True, False, 0.0, False),
        "cg_density": ((20, 24), 700, 3, 1, True, True, 0.0, False),
        "cg_damp": ((16, 20), 500, 2, 1, True, False, 0.25, True),
        "cg_calib": ((18, 16), 450, 2, 2, False, False, 0.0, False),
        "cg_3d": ((10, 12, 8), 900, 2, 1, True, True, 0.0, False),
    }
    for i, (name, (shape, M, C, B, sense, dens, damp, with_x0)) in enumerate(specs.items()):
        rng = np.random.default_rng(100 + i)
        s = rng.uniform(-0.5, 0.5, (M, len(shape)))
        smaps = cplx(rng, (C, *shape)) if sense else None
        if sense:
            smaps /= np.sqrt(np.sum(np.abs(smaps) ** 2, axis=0))
        density = 0.05 + np.linalg.norm(s, axis=-1) if dens else None
        op = MRInumpy(s, shape, n_coils=C, smaps=smaps)
        if density is not None:
            op.density = density  # the base class setter (base.py:770-784)
        op.n_batchs = B
        op.squeeze_dims = False
        x_true = cplx(rng, (B, 1 if sense else C, *shape))
        y = op.op(x_true) + 0.05 * cplx(rng, (B, C, M))
        x0 = cplx(rng, (B, 1 if sense else C, *shape)) if with_x0 else None
        seed = 1000 + i
        np.random.seed(seed)
        L = op.get_lipschitz_cst(max_iter=10)
        np.random.seed(seed)
        x = cg(op, y, damp=damp, x0=x0, max_iter=10, progressbar=False)
        out[f"{name}__samples"] = s
        out[f"{name}__shape"] = np.array(shape)
        out[f"{name}__n_coils"] = np.array(C)
        out[f"{name}__n_batchs"] = np.array(B)
        out[f"{name}__damp"] = np.array(damp)
        out[f"{name}__seed"] = np.array(seed)
        if sense:
            out[f"{name}__smaps"] = smaps
        if density is not None:
            out[f"{name}__density"] = density
        if x0 is not None:
            out[f"{name}__x0"] = x0
        out[f"{name}__ksp"] = y
        out[f"{name}__lipschitz"] = np.array(float(L))
        out[f"{name}__x"] = np.asarray(x)
    np.savez_compressed(HERE / "cg_golden.npz", **out)
    print("wrote", HERE / "cg_golden.npz", sorted(k for k in out if k.endswith("lipschitz")),
          [float(out[k]) for k in sorted(out) if k.endswith("lipschitz")])


if __name__ == "__main__":
    main(reference_src())
