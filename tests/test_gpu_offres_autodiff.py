"""Gradients of the off-resonance corrected operator (``MRINufftAutoGrad``
around ``MRIFourierCorrectedGB300``), against torch autograd of dense FP64
models on the CPU.

* Field-map gradients, forward and adjoint: against the exact model
  ``E = A * exp(t f^T)`` (relative l2 <= 1e-2: the SVD interpolators quantise
  the field map into 1024 histogram bins, about 1e-3 of phase) and against
  the factorised model ``sum_l diag(B_l) A diag(C_l)`` built from the
  operator's own interpolators (relative l2 <= 1e-4).
* Data and trajectory gradients: against the factorised model (relative
  l2 <= 1e-4 for data, <= 1e-3 for the trajectory).

Readout: six spiral shots of 128 samples with one readout-time vector of
128 entries, so sample m has time index m mod 128.
"""

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu

SHAPE = (24, 20)


def _problem(seed, sense):
    from mrinufft_gb300 import workloads

    rng = np.random.default_rng(seed)
    traj = workloads.spiral_2d(6, 128, power=2).reshape(-1, 2)
    traj = (traj + 1e-3 * rng.standard_normal(traj.shape)).astype(np.float32)
    C, B = 2, (1 if sense else 2)
    smaps = None
    if sense:
        smaps = (rng.standard_normal((C, *SHAPE)) + 1j * rng.standard_normal((C, *SHAPE))).astype(np.complex64)
    b0 = rng.uniform(-30, 30, SHAPE).astype(np.float32)
    t = np.linspace(0, 5e-3, 128, dtype=np.float32)
    nx = B if sense else B * C
    x = (rng.standard_normal((nx, *SHAPE)) + 1j * rng.standard_normal((nx, *SHAPE))).astype(np.complex64)
    y = (rng.standard_normal((B, C, traj.shape[0])) + 1j * rng.standard_normal((B, C, traj.shape[0]))).astype(np.complex64)
    return traj, smaps, b0, t, x, y, B, C


def _make(gpu_pkg, traj, smaps, b0, t, B, C):
    op = gpu_pkg.MRIGB300(traj, SHAPE, n_coils=C, n_batchs=B, smaps=smaps, squeeze_dims=False)
    return op.with_off_resonance_correction(t, b0_map=b0, interpolator={"name": "svd", "L": 8})


def _dense_A(k_rad):
    """(M, N) FP64 type-2 NDFT matrix on the reference's grid, normalised."""
    axes = [torch.linspace(-s / 2, s / 2 - 1, s, dtype=torch.float64) for s in SHAPE]
    grid = torch.stack(torch.meshgrid(*axes, indexing="ij"), -1).reshape(-1, len(SHAPE))
    norm = np.sqrt(np.prod(SHAPE) * 2 ** len(SHAPE))
    return torch.exp(-1j * (k_rad @ grid.T)) / norm


def _maps(smaps, C):
    if smaps is None:
        return None
    return torch.from_numpy(smaps.astype(np.complex128)).reshape(C, -1)


def _forward(E, maps, x, B, C):
    """(B, C, M) from (B, N) images with maps or (B*C, N) without."""
    if maps is not None:
        return torch.stack([(E @ (maps * x[b]).T).T for b in range(B)])
    return (E @ x.reshape(B * C, -1).T).T.reshape(B, C, -1)


def _adjoint(E, maps, y, B, C):
    """(B, 1 or C, N) from (B, C, M)."""
    z = (E.conj().T @ y.reshape(B * C, -1).T).T.reshape(B, C, -1)
    if maps is not None:
        return (maps.conj() * z).sum(1, keepdim=True)
    return z


def _exact_E(k_rad, f, tt):
    return _dense_A(k_rad) * torch.exp(tt[:, None] * f.reshape(1, -1))


def _factorised_E(k_rad, cor):
    Bt = cor.B.cpu().to(torch.complex128)          # (NK, L)
    Cs = cor.C.cpu().to(torch.complex128).reshape(Bt.shape[1], -1)
    Bfull = Bt.repeat(cor.n_shots, 1)              # sample m -> row m mod NK
    A = _dense_A(k_rad)
    return sum(Bfull[:, l:l + 1] * A * Cs[l][None, :] for l in range(Bt.shape[1]))


@pytest.mark.parametrize("sense", [True, False])
def test_field_map_gradient_forward(gpu_pkg, sense):
    traj, smaps, b0, t, x, y, B, C = _problem(50 + sense, sense)
    cor = _make(gpu_pkg, traj, smaps, b0, t, B, C)
    ad = cor.make_autograd(wrt_data=False, wrt_field_map=True)
    xt = torch.from_numpy(x).cuda().reshape(*((B, 1) if sense else (B, C)), *SHAPE)
    yt = torch.from_numpy(y).cuda()
    loss = torch.sum(torch.abs(ad.op(xt) - yt) ** 2)
    loss.backward()
    g = ad.field_map.grad.cpu().numpy()
    assert g.shape == SHAPE

    k = torch.from_numpy(cor.samples.astype(np.float64))
    tt = torch.from_numpy(np.tile(t.astype(np.float64), cor.n_shots))
    maps = _maps(smaps, C)
    x64 = torch.from_numpy(x.astype(np.complex128)).reshape(x.shape[0], -1)
    y64 = torch.from_numpy(y.astype(np.complex128))
    # exact exponential model
    f = torch.from_numpy(np.asarray(cor.field_map).astype(np.complex128)).reshape(-1).requires_grad_(True)
    ref_loss = torch.sum(torch.abs(_forward(_exact_E(k, f, tt), maps, x64, B, C) - y64) ** 2)
    ref_loss.backward()
    assert rel_l2(g, f.grad.reshape(SHAPE).numpy()) < 1e-2
    # closed form on the factorised model: conj(x) E^H(t dy), summed over b, c
    Ef = _factorised_E(k, cor)
    dy = 2 * (_forward(Ef, maps, x64, B, C) - y64)
    gx = _adjoint(Ef, maps, dy * tt, B, C)
    closed = (x64.reshape(gx.shape).conj() * gx).sum((0, 1)).reshape(SHAPE).numpy()
    assert rel_l2(g, closed) < 1e-4


@pytest.mark.parametrize("sense", [True, False])
def test_field_map_gradient_adjoint(gpu_pkg, sense):
    traj, smaps, b0, t, x, y, B, C = _problem(60 + sense, sense)
    cor = _make(gpu_pkg, traj, smaps, b0, t, B, C)
    ad = cor.make_autograd(wrt_data=True, wrt_field_map=True)
    yt = torch.from_numpy(y).cuda().requires_grad_(True)
    xt = torch.from_numpy(x).cuda().reshape(*((B, 1) if sense else (B, C)), *SHAPE)
    loss = torch.sum(torch.abs(ad.adj_op(yt) - xt) ** 2)
    loss.backward()
    g = ad.field_map.grad.cpu().numpy()

    k = torch.from_numpy(cor.samples.astype(np.float64))
    tt = torch.from_numpy(np.tile(t.astype(np.float64), cor.n_shots))
    maps = _maps(smaps, C)
    x64 = torch.from_numpy(x.astype(np.complex128)).reshape((B, 1, -1) if sense else (B, C, -1))
    y64 = torch.from_numpy(y.astype(np.complex128))
    f = torch.from_numpy(np.asarray(cor.field_map).astype(np.complex128)).reshape(-1).requires_grad_(True)
    ref_loss = torch.sum(torch.abs(_adjoint(_exact_E(k, f, tt), maps, y64, B, C) - x64) ** 2)
    ref_loss.backward()
    assert rel_l2(g, f.grad.reshape(SHAPE).numpy()) < 1e-2
    # data gradient on the factorised model: 2 E (E^H y - x)
    Ef = _factorised_E(k, cor)
    r = _adjoint(Ef, maps, y64, B, C) - x64
    gy = 2 * _forward(Ef, maps, r.reshape(r.shape[0] * r.shape[1], -1) if not sense else r[:, 0], B, C)
    assert rel_l2(yt.grad.cpu().numpy(), gy.numpy()) < 1e-4


@pytest.mark.parametrize("adjoint", [False, True])
def test_trajectory_gradient_corrected(gpu_pkg, adjoint):
    traj, smaps, b0, t, x, y, B, C = _problem(70 + adjoint, True)
    cor = _make(gpu_pkg, traj, smaps, b0, t, B, C)
    ad = cor.make_autograd(wrt_data=False, wrt_traj=True)
    xt = torch.from_numpy(x).cuda().reshape(B, 1, *SHAPE)
    yt = torch.from_numpy(y).cuda()
    if adjoint:
        loss = torch.sum(torch.abs(ad.adj_op(yt) - xt) ** 2)
    else:
        loss = torch.sum(torch.abs(ad.op(xt) - yt) ** 2)
    loss.backward()
    g = ad.samples.grad.cpu().numpy()

    k = torch.from_numpy(cor.samples.astype(np.float64)).requires_grad_(True)
    maps = _maps(smaps, C)
    x64 = torch.from_numpy(x.astype(np.complex128)).reshape(B, -1)
    y64 = torch.from_numpy(y.astype(np.complex128))
    Ef = _factorised_E(k, cor)
    if adjoint:
        ref_loss = torch.sum(torch.abs(_adjoint(Ef, maps, y64, B, C) - x64[:, None]) ** 2)
    else:
        ref_loss = torch.sum(torch.abs(_forward(Ef, maps, x64, B, C) - y64) ** 2)
    ref_loss.backward()
    assert rel_l2(g, k.grad.numpy()) < 1e-3


def test_field_map_update_and_errors(gpu_pkg):
    traj, smaps, b0, t, x, y, B, C = _problem(80, True)
    cor = _make(gpu_pkg, traj, smaps, b0, t, B, C)
    np.testing.assert_allclose(cor.full_readout_time, np.repeat(t, cor.n_shots))
    ad = cor.make_autograd(wrt_field_map=True)
    # a new field map recomputes the interpolators: the operator then matches
    # the factorised model of the new map
    new = torch.from_numpy(np.asarray(cor.field_map) * 0.5)
    ad.field_map = new
    assert ad.field_map is new
    k = torch.from_numpy(cor.samples.astype(np.float64))
    Ef = _factorised_E(k, cor)
    x64 = torch.from_numpy(x.astype(np.complex128)).reshape(B, -1)
    ref = _forward(Ef, _maps(smaps, C), x64, B, C).numpy()
    out = cor.op(x.reshape(B, 1, *SHAPE))
    assert rel_l2(out, ref) < 1e-4
    # the plain operator takes no field map
    plain = gpu_pkg.MRIGB300(traj, SHAPE, n_coils=C, smaps=smaps, squeeze_dims=False).make_autograd()
    with pytest.raises(ValueError):
        plain.op(torch.from_numpy(x).cuda().reshape(B, 1, *SHAPE), field_map=new)
    with pytest.raises(ValueError):
        _ = plain.field_map
