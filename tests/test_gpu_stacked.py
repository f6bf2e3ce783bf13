"""Stacked NUFFT on the GPU against the reference's own ``MRIStackedNUFFT``
(golden fixtures from ``tests/golden/make_stacked_golden.py``, FP64 NDFT
backend) and the FP64 oracle.

Tolerance: relative l2 <= 1e-4 (eps = 1e-6 2D transforms, float32 z-FFT).
"""

from pathlib import Path

import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import stacked as ostacked

pytestmark = pytest.mark.gpu

TOL = 1e-4
GOLD = Path(__file__).resolve().parent / "golden" / "stacked_golden.npz"


@pytest.mark.parametrize("name", ["stack_sense", "stack_calib"])
def test_op_adj_match_reference(gpu_pkg, name):
    g = np.load(GOLD)
    shape = tuple(int(v) for v in g[f"{name}__shape"])
    smaps = g[f"{name}__smaps"].astype(np.complex64) if f"{name}__smaps" in g else None
    C, B = int(g[f"{name}__n_coils"]), int(g[f"{name}__n_batchs"])
    op = gpu_pkg.MRIStackedGB300(g[f"{name}__samples"].astype(np.float32), shape, smaps=smaps,
                                 n_coils=C, n_batchs=B, z_index=g[f"{name}__z_index"])
    y = op.op(g[f"{name}__img"].astype(np.complex64))
    assert y.shape == g[f"{name}__op"].shape
    assert rel_l2(y, g[f"{name}__op"]) < TOL
    x = op.adj_op(g[f"{name}__ksp"].astype(np.complex64))
    assert x.shape == g[f"{name}__adj"].shape
    assert rel_l2(x, g[f"{name}__adj"]) < TOL


def test_3d_trajectory_density_and_dc(gpu_pkg):
    # a 3D stacked trajectory with z_index="auto", density weights of the 2D
    # trajectory, data consistency, adjointness
    from mrinufft_gb300.stacked import stacked2traj3d

    rng = np.random.default_rng(31)
    shape, C = (24, 20, 16), 2
    s2 = rng.uniform(-0.5, 0.5, (700, 2)).astype(np.float32)
    zi = np.array([0, 3, 7, 8, 9, 15])
    s3 = stacked2traj3d(s2, zi, shape[-1])
    d = rng.uniform(0.5, 1.5, s2.shape[0]).astype(np.float32)
    smaps = (rng.standard_normal((C, *shape)) + 1j * rng.standard_normal((C, *shape))).astype(np.complex64)
    op = gpu_pkg.MRIStackedGB300(s3, shape, smaps=smaps, n_coils=C, density=d)
    np.testing.assert_array_equal(op.z_index, zi)
    x = (rng.standard_normal((1, *shape)) + 1j * rng.standard_normal((1, *shape))).astype(np.complex64)
    y = (rng.standard_normal((1, C, op.n_samples)) + 1j * rng.standard_normal((1, C, op.n_samples))).astype(np.complex64)
    ref_op = ostacked.stacked_op(s2, shape, zi, x, smaps=smaps)
    assert rel_l2(op.op(x), ref_op) < TOL
    yd = (y.reshape(1, C, len(zi), -1) * d).reshape(y.shape)
    assert rel_l2(op.adj_op(y), ostacked.stacked_adj(s2, shape, zi, yd, smaps=smaps)) < TOL
    r = (ref_op - y.reshape(ref_op.shape)).reshape(1, C, len(zi), -1) * d
    ref_dc = ostacked.stacked_adj(s2, shape, zi, r.reshape(1, C, -1), smaps=smaps)
    assert rel_l2(op.data_consistency(x, y), ref_dc) < TOL
    # adjointness without density
    op2 = gpu_pkg.MRIStackedGB300(s3, shape, smaps=smaps, n_coils=C)
    lhs = np.vdot(op2.op(x).astype(np.complex128), y)
    rhs = np.vdot(x.astype(np.complex128), op2.adj_op(y))
    assert abs(lhs - rhs) / abs(rhs) < 5e-5


def test_torch_device_arrays(gpu_pkg):
    rng = np.random.default_rng(32)
    shape = (16, 16, 8)
    s2 = rng.uniform(-0.5, 0.5, (300, 2)).astype(np.float32)
    op = gpu_pkg.MRIStackedGB300(s2, shape, n_coils=2, z_index=None)
    x = torch.randn((1, 2, *shape), dtype=torch.complex64, device="cuda")
    y = op.op(x)
    assert isinstance(y, torch.Tensor) and y.is_cuda and tuple(y.shape) == (1, 2, 8 * 300)
    ref = ostacked.stacked_op(s2, shape, np.arange(8), x.cpu().numpy(), n_coils=2)
    assert rel_l2(y.cpu().numpy(), ref) < TOL
