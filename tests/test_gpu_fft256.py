"""The fused pruned transforms of 256^3 fine grids.

Plans whose fine grid is 256 on every axis run pad + transform and transform
+ crop as three line-transform passes each (the default); GBN_FUSED_FFT=0
keeps the pad pass, cuFFT and the crop pass.  Both paths compute the same
sums in FP32, so op, adj, data consistency, the Toeplitz Gram operator and
the trajectory gradient of the two agree to relative l2 <= 1e-5; the fused
path also matches the FP64 NDFT oracle (relative l2 <= 1e-4) on row and
voxel subsets, for an even 128^3 image and for odd / even 127 x 126 x 128
(whose modes sit asymmetrically on the 256-point axes; integer modes
-(N//2) .. N - N//2 - 1, the oracle's "finufft" grid), SENSE and
calibrationless, with two coil passes (5 coils, 4 per pass), and for the +1
exponent sign; at oversampling 2.5 and 1.25 (101-204 modes on the 256-point
axes) it is as accurate as the cuFFT path against the oracle.
"""

import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import ndft

pytestmark = pytest.mark.gpu

SAME = 1e-5
TOL = 1e-4


def _problem(shape, C, M, seed):
    rng = np.random.default_rng(seed)
    k = np.concatenate([rng.uniform(-0.5, 0.5, (M // 2, 3)),
                        np.clip(rng.normal(0, 0.07, (M - M // 2, 3)), -0.5, 0.4999)]).astype(np.float32)
    cpx = lambda *s: (rng.standard_normal(s) + 1j * rng.standard_normal(s)).astype(np.complex64)
    return k, cpx(C, *shape), cpx(1, *shape), cpx(1, C, M), rng.uniform(0.5, 1.5, M).astype(np.float32)


def _ops(gpu_pkg, monkeypatch, k, shape, C, smaps, dens):
    out = []
    for env in ("1", "0"):
        monkeypatch.setenv("GBN_FUSED_FFT", env)
        out.append(gpu_pkg.MRIGB300(k, shape, n_coils=C, smaps=smaps, density=dens, squeeze_dims=False))
    monkeypatch.delenv("GBN_FUSED_FFT")
    return out


@pytest.mark.parametrize("shape", [(128, 128, 128), (127, 126, 128)])
@pytest.mark.parametrize("sense", [True, False])
def test_fused_equals_cufft_path(gpu_pkg, monkeypatch, shape, sense):
    C, M = 5, 40000
    k, smaps, x1, y, dens = _problem(shape, C, M, seed=sum(shape) + sense)
    fused, plain = _ops(gpu_pkg, monkeypatch, k, shape, C, smaps if sense else None, dens)
    assert fused.plan.info()["nf"] == (256, 256, 256)
    x = x1 if sense else np.repeat(x1, C, axis=0)[None]
    assert rel_l2(fused.op(x), plain.op(x)) < SAME
    assert rel_l2(fused.adj_op(y), plain.adj_op(y)) < SAME
    assert rel_l2(fused.data_consistency(x, y), plain.data_consistency(x, y)) < SAME
    if sense:
        assert rel_l2(fused.gram_op(x), plain.gram_op(x)) < SAME


@pytest.mark.parametrize("shape", [(128, 128, 128), (127, 126, 128)])
def test_fused_against_ndft(gpu_pkg, shape):
    C, M = 5, 30000
    k, smaps, x, y, dens = _problem(shape, C, M, seed=7)
    op = gpu_pkg.MRIGB300(k, shape, n_coils=C, smaps=smaps, squeeze_dims=False)
    yk = op.op(x)[0]
    ku = ndft.proper_trajectory_unit(k)
    nf = ndft.norm_factor(shape)
    rng = np.random.default_rng(1)
    rows = np.sort(rng.choice(M, 1024, replace=False))
    for c in (0, 4):
        ref = ndft.ndft_type2(ku[rows], x[0].astype(np.complex128) * smaps[c], shape,
                              grid="finufft") / nf
        assert rel_l2(yk[c, rows], ref) < TOL, c
    z = op.adj_op(y)[0, 0]
    idx = [np.sort(rng.choice(n, 12, replace=False)) for n in shape]
    t1 = ndft.ndft_type1_grid(ku, y[0].astype(np.complex128), shape, idx, grid="finufft") / nf
    sub = np.ix_(*idx)
    ref = sum(np.conj(smaps[c][sub]) * t1[c] for c in range(C))
    assert rel_l2(z[sub], ref) < TOL


def test_fused_plus_sign_and_trajectory_gradient(gpu_pkg, monkeypatch):
    """The +1 exponent (conjugated line transforms) through the plan, and the
    trajectory gradient (its pad runs with conjugated inputs)."""
    shape, C, M = (128, 128, 128), 2, 20000
    k, smaps, x, y, _ = _problem(shape, C, M, seed=11)
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
        loss = torch.sum(torch.abs(ad.op(xt.reshape(1, 1, *shape)) - yt) ** 2)
        loss.backward()
        res.append((out.cpu().numpy(), img.cpu().numpy(), ad.samples.grad.cpu().numpy()))
    monkeypatch.delenv("GBN_FUSED_FFT")
    for a, b in zip(*res):
        assert rel_l2(a, b) < SAME
    # the +1 sign against the oracle on a row subset
    ku = ndft.proper_trajectory_unit(k)
    rows = np.arange(0, M, 37)
    ref = np.conj(ndft.ndft_type2(ku[rows], np.conj(x[0].astype(np.complex128) * smaps[1]), shape))
    assert rel_l2(res[0][0][0, 1, rows], ref) < TOL


@pytest.mark.parametrize("shape,osf", [((102, 101, 102), 2.5), ((204, 203, 204), 1.25)])
def test_fused_other_oversampling(gpu_pkg, monkeypatch, shape, osf):
    """Other oversampling factors that land on 256-point fine axes: 101-102
    modes per axis at 2.5 (kernel width 6) and 203-204 at 1.25 (width 10),
    where a pruned line reads most of its entries.  At 1.25 the
    deapodisation factors at the band edge are large, so the FP32 rounding
    of either transform is amplified and the two paths differ by about 1e-4;
    the criterion is the FP64 oracle: on row and voxel subsets the fused
    path is as accurate as the cuFFT path (and within 1e-4 at 2.5)."""
    C, M = 3, 20000
    k, smaps, x, y, _ = _problem(shape, C, M, seed=int(osf * 100))
    ops = []
    for env in ("1", "0"):
        monkeypatch.setenv("GBN_FUSED_FFT", env)
        ops.append(gpu_pkg.MRIGB300(k, shape, n_coils=C, smaps=smaps, upsampfac=osf, squeeze_dims=False))
    monkeypatch.delenv("GBN_FUSED_FFT")
    assert ops[0].plan.info()["nf"] == (256, 256, 256)
    ku = ndft.proper_trajectory_unit(k)
    nrm = ndft.norm_factor(shape)
    rng = np.random.default_rng(5)
    rows = np.sort(rng.choice(M, 256, replace=False))
    ref = ndft.ndft_type2(ku[rows], x[0].astype(np.complex128) * smaps[1], shape, grid="finufft") / nrm
    err_op = [rel_l2(o.op(x)[0, 1, rows], ref) for o in ops]
    idx = [np.sort(rng.choice(n, 8, replace=False)) for n in shape]
    t1 = ndft.ndft_type1_grid(ku, y[0].astype(np.complex128), shape, idx, grid="finufft") / nrm
    sub = np.ix_(*idx)
    ref_adj = sum(np.conj(smaps[c][sub]) * t1[c] for c in range(C))
    err_adj = [rel_l2(o.adj_op(y)[0, 0][sub], ref_adj) for o in ops]
    for fused, plain in (err_op, err_adj):
        assert fused <= 1.5 * plain + 1e-6, (fused, plain)
        assert fused < (TOL if osf == 2.5 else 1e-3), fused


@pytest.mark.parametrize("sense", [True, False])
def test_fused_several_batches(gpu_pkg, monkeypatch, sense):
    """n_batchs = 2: the passes loop over batch items (SENSE: one image per
    item, its crop restarts the coil sum); op, adjoint, data consistency and
    the Toeplitz Gram against the cuFFT path."""
    shape, C, B, M = (128, 128, 128), 3, 2, 20000
    rng = np.random.default_rng(21 + sense)
    k, smaps, _, _, dens = _problem(shape, C, M, seed=31 + sense)
    cpx = lambda *s: (rng.standard_normal(s) + 1j * rng.standard_normal(s)).astype(np.complex64)
    x = cpx(B, 1, *shape) if sense else cpx(B, C, *shape)
    y = cpx(B, C, M)
    ops = []
    for env in ("1", "0"):
        monkeypatch.setenv("GBN_FUSED_FFT", env)
        ops.append(gpu_pkg.MRIGB300(k, shape, n_coils=C, n_batchs=B, smaps=smaps if sense else None,
                                    density=dens, squeeze_dims=False))
    monkeypatch.delenv("GBN_FUSED_FFT")
    assert rel_l2(ops[0].op(x), ops[1].op(x)) < SAME
    assert rel_l2(ops[0].adj_op(y), ops[1].adj_op(y)) < SAME
    assert rel_l2(ops[0].data_consistency(x, y), ops[1].data_consistency(x, y)) < SAME
    if sense:
        assert rel_l2(ops[0].gram_op(x), ops[1].gram_op(x)) < SAME
