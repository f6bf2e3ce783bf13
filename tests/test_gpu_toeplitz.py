"""Toeplitz Gram operator on the GPU against the reference's own Toeplitz code
(golden fixtures from ``tests/golden/make_toeplitz_golden.py``) and the FP64
NDFT oracle.

Tolerance: relative l2 <= 1e-4 (eps = 1e-6 transforms build the kernel; the
Gram product itself is FFT-exact up to float32 rounding).
"""

from pathlib import Path

import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import toeplitz
from oracle.operator import NDFTOperator

pytestmark = pytest.mark.gpu

TOL = 1e-4
GOLD = Path(__file__).resolve().parent / "golden" / "toeplitz_golden.npz"


@pytest.mark.parametrize("name", ["toep2D_w", "toep2D", "toep3D_w"])
def test_kernel_and_gram_match_reference(gpu_pkg, name):
    g = np.load(GOLD)
    s = g[f"{name}__samples"].astype(np.float32)
    shape = tuple(int(v) for v in g[f"{name}__shape"])
    w = g[f"{name}__weights"].astype(np.float32)
    dens = None if name == "toep2D" else w
    op = gpu_pkg.MRIGB300(s, shape, density=dens)
    k = op.compute_toeplitz_kernel()
    assert k.shape == g[f"{name}__kernel"].shape
    assert rel_l2(k, g[f"{name}__kernel"]) < TOL
    x = g[f"{name}__img"].astype(np.complex64)
    assert rel_l2(op.gram_op(x), g[f"{name}__gram"]) < TOL


@pytest.mark.parametrize("shape", [(24, 20, 18), (15, 17)])
def test_sense_batches_density_vs_ndft(gpu_pkg, shape):
    # SENSE with 2 batches and 3 coils, density; odd sizes use a circulant
    # grid larger than 2N (the reference only supports even sizes)
    rng = np.random.default_rng(21)
    M, B, C = 3000, 2, 3
    s = rng.uniform(-0.5, 0.5, (M, len(shape))).astype(np.float32)
    d = rng.uniform(0.2, 2.0, M).astype(np.float32)
    smaps = (rng.standard_normal((C, *shape)) + 1j * rng.standard_normal((C, *shape))).astype(np.complex64)
    x = (rng.standard_normal((B, *shape)) + 1j * rng.standard_normal((B, *shape))).astype(np.complex64)
    op = gpu_pkg.MRIGB300(s, shape, n_coils=C, n_batchs=B, smaps=smaps, density=d, squeeze_dims=False)
    g = op.gram_op(x)
    grid = "finufft" if any(n % 2 for n in shape) else "ndft"
    ref = NDFTOperator(s, shape, n_coils=C, n_batchs=B, smaps=smaps, density=d, grid=grid)
    assert rel_l2(g, ref.adj(ref.op(x.reshape(B, 1, *shape)))) < TOL
    assert rel_l2(g, op.gram_op(x, toeplitz=False)) < TOL


def test_calibrationless_and_sample_update(gpu_pkg):
    rng = np.random.default_rng(22)
    shape, M, C = (32, 28), 4000, 2
    s = rng.uniform(-0.5, 0.5, (M, 2)).astype(np.float32)
    x = (rng.standard_normal((C, *shape)) + 1j * rng.standard_normal((C, *shape))).astype(np.complex64)
    op = gpu_pkg.MRIGB300(s, shape, n_coils=C, squeeze_dims=False)
    assert rel_l2(op.gram_op(x), op.gram_op(x, toeplitz=False)) < TOL
    # a new trajectory invalidates the kernel
    s2 = rng.uniform(-0.5, 0.5, (M, 2)).astype(np.float32)
    op.update_samples(s2)
    ref = NDFTOperator(s2, shape, n_coils=C)
    assert rel_l2(op.gram_op(x), ref.adj(ref.op(x.reshape(1, C, *shape)))) < TOL
    # the kernel of the oracle's construction on the new trajectory (2N = 56
    # is not 2-3-5 smooth along axis 1: the circulant grid is 64 x 60)
    k = op.compute_toeplitz_kernel()
    assert k.shape == (64, 60)
    assert rel_l2(k, toeplitz.toeplitz_kernel(s2, shape, grid=k.shape)) < TOL


def test_torch_inputs_stay_on_device(gpu_pkg):
    rng = np.random.default_rng(23)
    shape = (16, 16, 16)
    s = rng.uniform(-0.5, 0.5, (2000, 3)).astype(np.float32)
    op = gpu_pkg.MRIGB300(s, shape)
    x = torch.randn(shape, dtype=torch.complex64, device="cuda")
    g = op.gram_op(x)
    assert isinstance(g, torch.Tensor) and g.is_cuda
    assert rel_l2(g.cpu().numpy(), op.gram_op(x.cpu().numpy(), toeplitz=False)) < TOL
