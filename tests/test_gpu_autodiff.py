"""Gradients of the differentiable operator.

* data gradients against the FP64 NDFT (relative l2 <= 1e-4);
* trajectory gradients against FP64 central finite differences of the exact
  NDFT loss (h = 1e-4 rad) on a subset of samples (relative l2 <= 1e-3 over
  the subset), and against the reference's autodiff formula
  ``sum -i conj(dy) op(x n_d)`` (autodiff.py:22-41) evaluated on the NDFT.
"""

import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import ndft
from oracle.operator import NDFTOperator

pytestmark = pytest.mark.gpu


def _problem(seed=0, shape=(24, 20), coils=2, nc=6, ns=128):
    from mrinufft_gb300 import workloads

    rng = np.random.default_rng(seed)
    traj = workloads.spiral_2d(nc, ns, power=2).reshape(-1, 2)
    traj = (traj + 1e-3 * rng.standard_normal(traj.shape)).astype(np.float32)
    smaps = (rng.standard_normal((coils, *shape)) + 1j * rng.standard_normal((coils, *shape))).astype(np.complex64)
    x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    y = (rng.standard_normal((coils, traj.shape[0])) + 1j * rng.standard_normal((coils, traj.shape[0]))).astype(np.complex64)
    return traj, shape, smaps, x, y


def _ndft_loss(k_pi, shape, smaps, x, y):
    op = NDFTOperator(k_pi / (2 * np.pi), shape, smaps=smaps.astype(np.complex128))
    r = op.op(x.astype(np.complex128)).reshape(y.shape) - y
    return float(np.sum(np.abs(r) ** 2))


def test_op_data_gradient(gpu_pkg):
    traj, shape, smaps, x, y = _problem()
    nufft = gpu_pkg.MRIGB300(traj, shape, n_coils=2, smaps=smaps, squeeze_dims=False)
    ad = nufft.make_autograd(wrt_data=True)
    xt = torch.from_numpy(x).cuda().reshape(1, 1, *shape).requires_grad_(True)
    yt = torch.from_numpy(y).cuda().reshape(1, 2, -1)
    loss = torch.sum(torch.abs(ad.op(xt) - yt) ** 2)
    loss.backward()
    ref = NDFTOperator(traj, shape, smaps=smaps)
    g_ref = 2 * ref.adj(ref.op(x) - y.reshape(1, 2, -1))
    assert rel_l2(xt.grad.cpu().numpy(), g_ref) < 1e-4


def test_adj_data_gradient(gpu_pkg):
    traj, shape, smaps, x, y = _problem(1)
    nufft = gpu_pkg.MRIGB300(traj, shape, n_coils=2, smaps=smaps, squeeze_dims=False)
    ad = nufft.make_autograd(wrt_data=True)
    yt = torch.from_numpy(y).cuda().reshape(1, 2, -1).requires_grad_(True)
    xt = torch.from_numpy(x).cuda().reshape(1, 1, *shape)
    loss = torch.sum(torch.abs(ad.adj_op(yt) - xt) ** 2)
    loss.backward()
    ref = NDFTOperator(traj, shape, smaps=smaps)
    g_ref = 2 * ref.op(ref.adj(y.reshape(1, 2, -1)) - x.reshape(1, 1, *shape))
    assert rel_l2(yt.grad.cpu().numpy(), g_ref) < 1e-4


def test_op_trajectory_gradient_fd(gpu_pkg):
    traj, shape, smaps, x, y = _problem(2)
    nufft = gpu_pkg.MRIGB300(traj, shape, n_coils=2, smaps=smaps, squeeze_dims=False)
    ad = nufft.make_autograd(wrt_data=False, wrt_traj=True)
    xt = torch.from_numpy(x).cuda().reshape(1, 1, *shape)
    yt = torch.from_numpy(y).cuda().reshape(1, 2, -1)
    loss = torch.sum(torch.abs(ad.op(xt) - yt) ** 2)
    loss.backward()
    g = ad.samples.grad.cpu().numpy().astype(np.float64)
    k = nufft.samples.astype(np.float64)  # radians
    idx = np.random.default_rng(0).choice(k.shape[0], 12, replace=False)
    h = 1e-4
    fd = np.zeros((len(idx), 2))
    for a, j in enumerate(idx):
        for d in range(2):
            kp, km = k.copy(), k.copy()
            kp[j, d] += h
            km[j, d] -= h
            fd[a, d] = (_ndft_loss(kp, shape, smaps, x, y) - _ndft_loss(km, shape, smaps, x, y)) / (2 * h)
    assert rel_l2(g[idx], fd) < 1e-3
    # the reference formula: grad = Re(sum_c -i conj(dy) op(x n_d)), dy = 2 (Ax - y)
    ref = NDFTOperator(k / (2 * np.pi), shape, smaps=smaps)
    dy = 2 * (ref.op(x) - y.reshape(1, 2, -1))
    axes = [np.arange(n) - n // 2 for n in shape]
    grid = np.meshgrid(*axes, indexing="ij")
    g_ref = np.stack([np.real(np.sum(-1j * np.conj(dy) * ref.op(x * grid[d]), axis=(0, 1)))
                      for d in range(2)], axis=1)
    assert rel_l2(g, g_ref) < 1e-3


def test_adj_trajectory_gradient_fd(gpu_pkg):
    traj, shape, smaps, x, y = _problem(3)
    nufft = gpu_pkg.MRIGB300(traj, shape, n_coils=2, smaps=smaps, squeeze_dims=False)
    ad = nufft.make_autograd(wrt_data=False, wrt_traj=True)
    yt = torch.from_numpy(y).cuda().reshape(1, 2, -1)
    xt = torch.from_numpy(x).cuda().reshape(1, 1, *shape)
    loss = torch.sum(torch.abs(ad.adj_op(yt) - xt) ** 2)
    loss.backward()
    g = ad.samples.grad.cpu().numpy().astype(np.float64)
    k = nufft.samples.astype(np.float64)

    def loss_np(kk):
        op = NDFTOperator(kk / (2 * np.pi), shape, smaps=smaps)
        r = op.adj(y.reshape(1, 2, -1)) - x.reshape(1, 1, *shape)
        return float(np.sum(np.abs(r) ** 2))

    idx = np.random.default_rng(1).choice(k.shape[0], 12, replace=False)
    h = 1e-4
    fd = np.zeros((len(idx), 2))
    for a, j in enumerate(idx):
        for d in range(2):
            kp, km = k.copy(), k.copy()
            kp[j, d] += h
            km[j, d] -= h
            fd[a, d] = (loss_np(kp) - loss_np(km)) / (2 * h)
    assert rel_l2(g[idx], fd) < 1e-3


def test_trajectory_gradient_3d(gpu_pkg):
    from mrinufft_gb300 import workloads

    rng = np.random.default_rng(4)
    shape = (12, 14, 10)
    traj = (workloads.kooshball_3d(64, 16).reshape(-1, 3) + 1e-3 * rng.standard_normal((1024, 3))).astype(np.float32)
    x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    y = (rng.standard_normal(traj.shape[0]) + 1j * rng.standard_normal(traj.shape[0])).astype(np.complex64)
    nufft = gpu_pkg.MRIGB300(traj, shape, squeeze_dims=False)
    ad = nufft.make_autograd(wrt_data=False, wrt_traj=True)
    xt = torch.from_numpy(x).cuda().reshape(1, 1, *shape)
    loss = torch.sum(torch.abs(ad.op(xt) - torch.from_numpy(y).cuda().reshape(1, 1, -1)) ** 2)
    loss.backward()
    g = ad.samples.grad.cpu().numpy().astype(np.float64)
    k = nufft.samples.astype(np.float64)
    ref = NDFTOperator(k / (2 * np.pi), shape)
    dy = 2 * (ref.op(x) - y.reshape(1, 1, -1))
    axes = [np.arange(n) - n // 2 for n in shape]
    grid = np.meshgrid(*axes, indexing="ij")
    g_ref = np.stack([np.real(np.sum(-1j * np.conj(dy) * ref.op(x * grid[d]), axis=(0, 1)))
                      for d in range(3)], axis=1)
    assert rel_l2(g, g_ref) < 1e-3


def test_squeeze_dims_rejected(gpu_pkg):
    traj, shape, smaps, x, y = _problem()
    nufft = gpu_pkg.MRIGB300(traj, shape, squeeze_dims=True)
    with pytest.raises(ValueError):
        nufft.make_autograd()
