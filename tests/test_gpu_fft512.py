"""The fused pruned transforms of 512 x 512 fine grids (2D).

2D plans whose fine grid is 512 on both axes run pad + transform and
transform + crop as two line-transform passes each (the default);
GBN_FUSED_FFT=0 keeps the pad pass, cuFFT and the crop pass.  Both paths
agree to relative l2 <= 1e-5 on op, adj, data consistency, the Toeplitz Gram
operator, the +1 exponent and the trajectory gradient, for 256 x 256 (modes
known at compile time) and 255 x 254 (odd / even sizes, integer modes
-(N//2) .. N - N//2 - 1), SENSE and calibrationless, two batch items, and
two coil passes; the fused path matches the FP64 NDFT oracle (relative l2
<= 1e-4) on row and voxel subsets, and at oversampling 2.5 and 1.25 it is as
accurate as the cuFFT path against the oracle.
"""

import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import ndft

pytestmark = pytest.mark.gpu

SAME = 1e-5
TOL = 1e-4


def _problem(shape, C, M, seed, B=1):
    rng = np.random.default_rng(seed)
    k = np.concatenate([rng.uniform(-0.5, 0.5, (M // 2, 2)),
                        np.clip(rng.normal(0, 0.07, (M - M // 2, 2)), -0.5, 0.4999)]).astype(np.float32)
    cpx = lambda *s: (rng.standard_normal(s) + 1j * rng.standard_normal(s)).astype(np.complex64)
    return k, cpx(C, *shape), cpx(B, 1, *shape), cpx(B, C, *shape), cpx(B, C, M), \
        rng.uniform(0.5, 1.5, M).astype(np.float32)


def _pair(gpu_pkg, monkeypatch, *args, **kw):
    ops = []
    for env in ("1", "0"):
        monkeypatch.setenv("GBN_FUSED_FFT", env)
        ops.append(gpu_pkg.MRIGB300(*args, squeeze_dims=False, **kw))
    monkeypatch.delenv("GBN_FUSED_FFT")
    return ops


@pytest.mark.parametrize("shape", [(256, 256), (255, 254)])
@pytest.mark.parametrize("sense", [True, False])
@pytest.mark.parametrize("B", [1, 2])
def test_fused_equals_cufft_path(gpu_pkg, monkeypatch, shape, sense, B):
    C, M = 5, 40000
    k, smaps, xs, xc, y, dens = _problem(shape, C, M, seed=sum(shape) + sense + 7 * B, B=B)
    # a fine-grid budget of 4 grids: passes of 4 coils and a last one of 1
    fused, plain = _pair(gpu_pkg, monkeypatch, k, shape, n_coils=C, n_batchs=B,
                         smaps=smaps if sense else None, density=dens,
                         fine_budget_bytes=4 * 512 * 512 * 8)
    assert fused.plan.info()["nf"] == (512, 512)
    x = xs if sense else xc
    assert rel_l2(fused.op(x), plain.op(x)) < SAME
    assert rel_l2(fused.adj_op(y), plain.adj_op(y)) < SAME
    assert rel_l2(fused.data_consistency(x, y), plain.data_consistency(x, y)) < SAME
    if sense:
        assert rel_l2(fused.gram_op(x), plain.gram_op(x)) < SAME


@pytest.mark.parametrize("shape", [(256, 256), (255, 254)])
def test_fused_against_ndft(gpu_pkg, shape):
    C, M = 5, 30000
    k, smaps, x, _, y, _ = _problem(shape, C, M, seed=3)
    op = gpu_pkg.MRIGB300(k, shape, n_coils=C, smaps=smaps, squeeze_dims=False)
    yk = op.op(x)[0]
    ku = ndft.proper_trajectory_unit(k)
    nf = ndft.norm_factor(shape)
    rng = np.random.default_rng(1)
    rows = np.sort(rng.choice(M, 2048, replace=False))
    for c in (0, 4):
        ref = ndft.ndft_type2(ku[rows], x[0, 0].astype(np.complex128) * smaps[c], shape,
                              grid="finufft") / nf
        assert rel_l2(yk[c, rows], ref) < TOL, c
    z = op.adj_op(y)[0, 0]
    idx = [np.sort(rng.choice(n, 48, replace=False)) for n in shape]
    t1 = ndft.ndft_type1_grid(ku, y[0].astype(np.complex128), shape, idx, grid="finufft") / nf
    sub = np.ix_(*idx)
    ref = sum(np.conj(smaps[c][sub]) * t1[c] for c in range(C))
    assert rel_l2(z[sub], ref) < TOL


def test_fused_plus_sign_and_trajectory_gradient(gpu_pkg, monkeypatch):
    shape, C, M = (256, 256), 2, 20000
    k, smaps, x, _, y, _ = _problem(shape, C, M, seed=11)
    res = []
    for env in ("1", "0"):
        monkeypatch.setenv("GBN_FUSED_FFT", env)
        op = gpu_pkg.MRIGB300(k, shape, n_coils=C, smaps=smaps, squeeze_dims=False)
        xt = torch.from_numpy(x).cuda()
        out = torch.empty((1, C, M), dtype=torch.complex64, device="cuda")
        op.plan.op(xt, op._smaps, out, 1, C, 1.0, isign=+1)
        yt = torch.from_numpy(y).cuda()
        img = torch.empty((1, 1, *shape), dtype=torch.complex64, device="cuda")
        op.plan.adj(yt, None, op._smaps, img, 1, C, 1.0, isign=-1)
        ad = op.make_autograd(wrt_data=False, wrt_traj=True)
        loss = torch.sum(torch.abs(ad.op(xt) - yt) ** 2)
        loss.backward()
        res.append((out.cpu().numpy(), img.cpu().numpy(), ad.samples.grad.cpu().numpy()))
    monkeypatch.delenv("GBN_FUSED_FFT")
    for a, b in zip(*res):
        assert rel_l2(a, b) < SAME
    ku = ndft.proper_trajectory_unit(k)
    rows = np.arange(0, M, 13)
    ref = np.conj(ndft.ndft_type2(ku[rows], np.conj(x[0, 0].astype(np.complex128) * smaps[1]), shape))
    assert rel_l2(res[0][0][0, 1, rows], ref) < TOL


@pytest.mark.parametrize("shape,osf", [((204, 203), 2.5), ((409, 408), 1.25)])
def test_fused_other_oversampling(gpu_pkg, monkeypatch, shape, osf):
    C, M = 3, 20000
    k, smaps, x, _, y, _ = _problem(shape, C, M, seed=int(osf * 100))
    ops = _pair(gpu_pkg, monkeypatch, k, shape, n_coils=C, smaps=smaps, upsampfac=osf)
    assert ops[0].plan.info()["nf"] == (512, 512)
    ku = ndft.proper_trajectory_unit(k)
    nrm = ndft.norm_factor(shape)
    rng = np.random.default_rng(5)
    rows = np.sort(rng.choice(M, 1024, replace=False))
    ref = ndft.ndft_type2(ku[rows], x[0, 0].astype(np.complex128) * smaps[1], shape, grid="finufft") / nrm
    err_op = [rel_l2(o.op(x)[0, 1, rows], ref) for o in ops]
    idx = [np.sort(rng.choice(n, 32, replace=False)) for n in shape]
    t1 = ndft.ndft_type1_grid(ku, y[0].astype(np.complex128), shape, idx, grid="finufft") / nrm
    sub = np.ix_(*idx)
    ref_adj = sum(np.conj(smaps[c][sub]) * t1[c] for c in range(C))
    err_adj = [rel_l2(o.adj_op(y)[0, 0][sub], ref_adj) for o in ops]
    for fused, plain in (err_op, err_adj):
        assert fused <= 1.5 * plain + 1e-6, (fused, plain)
        assert fused < (TOL if osf == 2.5 else 1e-3), fused


def test_fused_many_coils(gpu_pkg, monkeypatch):
    """24 coils in one pass (one launch per pass direction over all coils)."""
    shape, C, M = (256, 256), 24, 20000
    k, smaps, xs, xc, y, dens = _problem(shape, C, M, seed=40)
    fused, plain = _pair(gpu_pkg, monkeypatch, k, shape, n_coils=C, smaps=smaps, density=dens)
    assert rel_l2(fused.op(xs), plain.op(xs)) < SAME
    assert rel_l2(fused.adj_op(y), plain.adj_op(y)) < SAME
    assert rel_l2(fused.gram_op(xs), plain.gram_op(xs)) < SAME
