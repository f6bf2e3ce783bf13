"""Generate the golden NDFT fixtures from the mri-nufft reference itself.

Run in a container where the reference sources are present::

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py <mri-nufft src>

It imports ``mrinufft`` from the given source tree, builds the reference's own
test trajectories (``tests/case_trajectories.py`` cases random2D, grid2D,
grid3D, radial2D, a small random3D) and runs the reference FP64 NDFT backend
``MRInumpy`` (``operators/interfaces/nudft_numpy.py``) with float64 samples, so
that every output is complex128.  Inputs are seeded.  The fixtures pin the
oracle in ``oracle/ndft.py`` (CPU tests) and the CUDA backend (GPU tests).
"""

from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
from _refsrc import reference_src  # noqa: E402

HERE = Path(__file__).resolve().parent


def _rng(seed):
    return np.random.default_rng(seed)


def _cplx(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(
        np.complex128
    )


def main(ref_src):
    os.environ.setdefault("PYTHONDONTWRITEBYTECODE", "1")
    sys.dont_write_bytecode = True
    sys.path.insert(0, ref_src)
    import scipy as sp
    from mrinufft._utils import proper_trajectory
    from mrinufft.operators.interfaces.nudft_numpy import MRInumpy
    from mrinufft.trajectories import initialize_2D_radial

    cases = {}

    # tests/case_trajectories.py: case_random2D (M=1000, N=64, seed 0)
    np.random.seed(0)
    s = sp.stats.truncnorm(-3, 3, loc=0, scale=0.16).rvs(size=1000 * 2)
    cases["random2D"] = (s.reshape(1000, 2), (64, 128))
    # case_random3D shrunk (M=2000, N=16 -> (16, 32, 26)), same generator
    np.random.seed(0)
    s = sp.stats.truncnorm(-3, 3, loc=0, scale=0.16).rvs(size=2000 * 3)
    cases["random3D"] = (s.reshape(2000, 3), (16, 32, 26))
    # case_grid2D / case_grid3D (N=16): Cartesian fftfreq grids
    f = sp.fft.fftfreq(16)
    cases["grid2D"] = (np.stack(np.meshgrid(f, f), axis=-1).reshape(-1, 2), (16, 16))
    cases["grid3D"] = (
        np.stack(np.meshgrid(f, f, f), axis=-1).reshape(-1, 3),
        (16, 16, 16),
    )
    # case_radial2D (Nc=10, Ns=500, N=64)
    cases["radial2D"] = (initialize_2D_radial(10, 500).reshape(-1, 2), (64, 64))

    out = {}
    for i, (name, (samples, shape)) in enumerate(cases.items()):
        samples = np.asarray(samples, dtype=np.float64)
        rng = _rng(100 + i)
        img = _cplx(rng, shape)
        ksp = _cplx(rng, (samples.shape[0],))
        op = MRInumpy(samples, shape)
        y = np.asarray(op.op(img)).reshape(-1)
        x = np.asarray(op.adj_op(ksp)).reshape(shape)
        out[f"{name}__samples"] = samples
        out[f"{name}__shape"] = np.array(shape)
        out[f"{name}__img"] = img
        out[f"{name}__ksp"] = ksp
        out[f"{name}__op"] = y
        out[f"{name}__adj"] = x
        assert y.dtype == np.complex128 and x.dtype == np.complex128

    # SENSE and calibrationless multi-coil, batched: operator-level semantics
    # (operators/base.py:949-1139), still on the FP64 NDFT.
    rng = _rng(7)
    np.random.seed(1)
    samples = sp.stats.truncnorm(-3, 3, loc=0, scale=0.16).rvs(size=400 * 2)
    samples = samples.reshape(400, 2).astype(np.float64)
    shape = (24, 32)
    C, B = 3, 2
    smaps = _cplx(rng, (C, *shape)) * 0.5
    img = _cplx(rng, (B, 1, *shape))
    ksp = _cplx(rng, (B, C, 400))
    op = MRInumpy(samples, shape, n_coils=C, smaps=smaps)
    op.n_batchs = B
    out["sense__samples"] = samples
    out["sense__shape"] = np.array(shape)
    out["sense__smaps"] = smaps
    out["sense__img"] = img
    out["sense__ksp"] = ksp
    out["sense__op"] = np.asarray(op.op(img))
    out["sense__adj"] = np.asarray(op.adj_op(ksp))
    out["sense__dc"] = np.asarray(op.data_consistency(img, ksp))
    imgc = _cplx(rng, (B, C, *shape))
    opc = MRInumpy(samples, shape, n_coils=C)
    opc.n_batchs = B
    out["calib__img"] = imgc
    out["calib__op"] = np.asarray(opc.op(imgc))
    out["calib__adj"] = np.asarray(opc.adj_op(ksp))
    out["calib__dc"] = np.asarray(opc.data_consistency(imgc, ksp))

    # proper_trajectory semantics (_utils.py:58-100)
    t_unit = np.array([[-0.5, 0.25], [0.4999, -0.1]], dtype=np.float64)
    t_pi = t_unit * 2 * np.pi
    out["proper__unit_in"] = t_unit
    out["proper__unit_to_pi"] = np.asarray(proper_trajectory(t_unit, "pi"))
    out["proper__pi_to_unit"] = np.asarray(proper_trajectory(t_pi, "unit"))
    t_wrap = np.array([[0.5, -0.5], [0.75, 0.1]])
    out["proper__wrap_in"] = t_wrap
    out["proper__wrap_unit"] = np.asarray(proper_trajectory(t_wrap, "unit"))

    np.savez_compressed(HERE / "ndft_golden.npz", **out)
    print("wrote", HERE / "ndft_golden.npz", sum(v.nbytes for v in out.values()), "B")


if __name__ == "__main__":
    main(reference_src())
