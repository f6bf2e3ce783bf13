"""The benchmark configurations at their full sizes against the FP64 oracle.

* 2D single coil: radial 100 x 500 (50 000 samples), 256^2; op and adj on
  every sample and voxel against the exact NDFT;
* 3D multi-coil: kooshball 4096 x 512 (2 097 152 samples), 128^3, 16 coils,
  pipe density; op on 4096 seeded rows of 4 seeded coils, the
  density-compensated SENSE adjoint of those 4 coils on a seeded 16^3
  product set of voxels (4096);
* 32 uneven 2D SENSE instances through the batched form with the autotuner's
  choices; op on 2048 seeded rows of up to 4 coils and the adjoint of up to 4
  coils on a 64 x 64 product set of voxels, per instance; and a 3D batch
  whose interpolation the autotuner must take from the warp-cooperative
  direct kernel;
* differentiable 256^2, 8 coils, Galilean spiral 64 x 2048 (131 072
  samples): image and k-space data gradients on voxel / row subsets against
  the NDFT, trajectory gradients on 32 seeded samples against FP64 central
  differences (h = 1e-4 rad) of the exact loss;
* served requests of each template of the mixed stream (2D 256^2 radial
  256 x 512, 2D 384^2 spiral 32 x 4096, 3D 128^3 kooshball 2048 x 512) against
  the oracle's CG on the FP64 ES-kernel NUFFT (about 1e-6 from the exact sum;
  the exact NDFT would take hours at these sizes), same Lipschitz start
  vector.

Tolerance: relative l2 <= 1e-4 everywhere (the accuracy bar at eps = 1e-6),
1e-3 for the finite-difference trajectory gradients (the difference quotient
itself carries about 1e-6 relative truncation and cancellation error per
sample, and the comparison is over 32 samples only).
"""

import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import ndft

pytestmark = pytest.mark.gpu

TOL = 1e-4


def test_config1_full(gpu_pkg):
    from mrinufft_gb300 import workloads

    traj, shape, img = workloads.config1()
    op = gpu_pkg.MRIGB300(traj, shape, squeeze_dims=False)
    y = op.op(img).reshape(-1)
    nf = ndft.norm_factor(shape)
    k = ndft.proper_trajectory_unit(traj)
    assert rel_l2(y, ndft.ndft_type2(k, img, shape) / nf) < TOL
    x = op.adj_op(y).reshape(shape)
    assert rel_l2(x, ndft.ndft_type1(k, y, shape) / nf) < TOL


def test_config2_subsets(gpu_pkg):
    from mrinufft_gb300 import workloads

    traj, shape, img, smaps = workloads.config2()
    M, C = traj.shape[0], smaps.shape[0]
    dens = gpu_pkg.MRIGB300.pipe(traj, shape, max_iter=10)
    op = gpu_pkg.MRIGB300(traj, shape, n_coils=C, smaps=smaps, density=dens, squeeze_dims=False)
    x = torch.from_numpy(img).cuda().reshape(1, *shape)
    y = op._op_device(x)
    rng = np.random.default_rng(2)
    coils = np.sort(rng.choice(C, 4, replace=False))
    rows = np.sort(rng.choice(M, 4096, replace=False))
    k = ndft.proper_trajectory_unit(traj)
    nf = ndft.norm_factor(shape)
    yh = y[0].cpu().numpy()
    for c in coils:
        ref = ndft.ndft_type2(k[rows], img.astype(np.complex128) * smaps[c], shape) / nf
        assert rel_l2(yh[c, rows], ref) < TOL, c
    # SENSE adjoint of the 4 coils' k-space (others zero), density compensated
    yk = torch.zeros_like(y)
    yk[0, coils] = y[0, coils]
    z = op._adj_device(yk)[0, 0].cpu().numpy()
    idx = [np.sort(rng.choice(n, 16, replace=False)) for n in shape]
    d = dens.astype(np.float64)
    t1 = ndft.ndft_type1_grid(k, yh[coils].astype(np.complex128) * d, shape, idx) / nf
    sub = np.ix_(*idx)
    ref = sum(np.conj(smaps[c][sub]) * t1[q] for q, c in enumerate(coils))
    assert rel_l2(z[sub], ref) < TOL


def _check_instance(inst, y, x_adj, y_in, rng):
    """op rows of up to 4 coils; SENSE adjoint of the adjoint input y_in
    (nonzero on up to 4 coils) on a 64 x 64 voxel product set."""
    shape, smaps = inst["shape"], inst["smaps"]
    C = smaps.shape[0]
    k = ndft.proper_trajectory_unit(inst["samples"])
    nf = ndft.norm_factor(shape)
    img = inst["image"].astype(np.complex128)
    coils = np.sort(rng.choice(C, min(C, 4), replace=False))
    rows = np.sort(rng.choice(k.shape[0], min(k.shape[0], 2048), replace=False))
    for c in coils:
        ref = ndft.ndft_type2(k[rows], img * smaps[c], shape) / nf
        assert rel_l2(y[c, rows], ref) < TOL
    idx = [np.sort(rng.choice(n, 64, replace=False)) for n in shape]
    nz = np.nonzero(np.any(y_in != 0, axis=1))[0]
    t1 = ndft.ndft_type1_grid(k, y_in[nz].astype(np.complex128), shape, idx) / nf
    sub = np.ix_(*idx)
    ref = sum(np.conj(smaps[c][sub]) * t1[q] for q, c in enumerate(nz))
    assert rel_l2(x_adj.reshape(shape)[sub], ref) < TOL


def test_config3_batched_instances(gpu_pkg, tmp_path):
    from mrinufft_gb300 import workloads
    from mrinufft_gb300.autotune import Autotuner
    from mrinufft_gb300.batched import BatchedNufft

    insts = workloads.config3(32, seed=0)
    bat = BatchedNufft(insts, tuner=Autotuner(cache_path=tmp_path / "tune.json"))
    bat.set_images([i["image"] for i in insts])
    ys = [t.cpu().numpy() for t in bat.op()]
    rng = np.random.default_rng(3)
    y_in = []
    for inst, y in zip(insts, ys):
        C = inst["smaps"].shape[0]
        keep = np.zeros(C, bool)
        keep[rng.choice(C, min(C, 4), replace=False)] = True
        y_in.append(np.where(keep[:, None], y, 0).astype(np.complex64))
    bat.set_kspace(y_in)
    xs = [t.cpu().numpy() for t in bat.adj()]
    for inst, y, x, yi in zip(insts, ys, xs, y_in):
        _check_instance(inst, y, x, yi, rng)


def test_batched_3d_warp_direct_interp(gpu_pkg, tmp_path):
    """A 3D batch tuned over the warp-cooperative direct interpolation only,
    so that every instance runs it, against the NDFT."""
    from mrinufft_gb300 import workloads
    from mrinufft_gb300.autotune import Autotuner
    from mrinufft_gb300.batched import BatchedNufft

    rng = np.random.default_rng(5)
    insts = []
    for N, C, (nc, ns) in [(24, 2, (96, 24)), (20, 3, (64, 32)), (28, 1, (128, 20))]:
        shape = (N,) * 3
        insts.append({"samples": workloads.kooshball_3d(nc, ns).reshape(-1, 3).astype(np.float32),
                      "shape": shape, "smaps": workloads.coil_maps(shape, C, seed=N),
                      "image": workloads.phantom(shape, seed=N)})
    tuner = Autotuner(cache_path=tmp_path / "t.json", interp_methods=("warp_direct",))
    bat = BatchedNufft(insts, tuner=tuner)
    assert all(c["interp"] == "warp_direct" for c in tuner.cache.values())
    bat.set_images([i["image"] for i in insts])
    ys = [t.cpu().numpy() for t in bat.op()]
    xs = [t.cpu().numpy() for t in bat.adj()]
    for inst, y, x in zip(insts, ys, xs):
        shape, smaps = inst["shape"], inst["smaps"]
        k = ndft.proper_trajectory_unit(inst["samples"])
        nf = ndft.norm_factor(shape)
        for c in range(smaps.shape[0]):
            ref = ndft.ndft_type2(k, inst["image"].astype(np.complex128) * smaps[c], shape) / nf
            assert rel_l2(y[c], ref) < TOL
        ref = sum(np.conj(smaps[c]) * ndft.ndft_type1(k, y[c], shape) for c in range(smaps.shape[0])) / nf
        assert rel_l2(x.reshape(shape), ref) < TOL


def test_config4_gradients(gpu_pkg):
    from mrinufft_gb300 import workloads

    shape, C = (256, 256), 8
    traj = workloads.spiral_2d(64, 2048, power=2).reshape(-1, 2).astype(np.float32)
    M = traj.shape[0]
    smaps = workloads.coil_maps(shape, C, seed=4)
    img = workloads.phantom(shape, seed=4)
    rng = np.random.default_rng(4)
    pert = traj + 1e-3 * rng.standard_normal(traj.shape).astype(np.float32)
    y = gpu_pkg.MRIGB300(pert, shape, n_coils=C, smaps=smaps, squeeze_dims=False).op(img)
    y = np.asarray(y).reshape(C, M)
    nufft = gpu_pkg.MRIGB300(traj, shape, n_coils=C, smaps=smaps, squeeze_dims=False)
    ad = nufft.make_autograd(wrt_data=True, wrt_traj=True)
    x = torch.from_numpy(img).cuda().reshape(1, 1, *shape).requires_grad_(True)
    yt = torch.from_numpy(y).cuda().reshape(1, C, M)
    loss = torch.sum(torch.abs(ad.op(x) - yt) ** 2)
    loss.backward()
    gx = x.grad.cpu().numpy().reshape(shape)
    gk = ad.samples.grad.cpu().numpy().astype(np.float64)

    k_pi = nufft.samples.astype(np.float64)  # radians, as the gradient is taken
    k = k_pi / (2 * np.pi)
    nf = ndft.norm_factor(shape)
    xs = img.astype(np.complex128)
    # residual A x - y on every sample (exact), then the image gradient
    # 2 A^H (A x - y) on a 64 x 64 voxel product set
    r = np.stack([ndft.ndft_type2(k, xs * smaps[c], shape) / nf for c in range(C)]) - y
    idx = [np.sort(rng.choice(n, 64, replace=False)) for n in shape]
    t1 = ndft.ndft_type1_grid(k, r, shape, idx) / nf
    sub = np.ix_(*idx)
    g_ref = 2 * sum(np.conj(smaps[c][sub]) * t1[c] for c in range(C))
    assert rel_l2(gx[sub], g_ref) < TOL

    # trajectory gradient: the loss depends on k_j only through row j
    sel = np.sort(rng.choice(M, 32, replace=False))
    h = 1e-4

    def row_loss(kj, j):
        u = (kj / (2 * np.pi))[None]
        v = np.array([ndft.ndft_type2(u, xs * smaps[c], shape)[0] for c in range(C)]) / nf
        return float(np.sum(np.abs(v - y[:, j]) ** 2))

    fd = np.zeros((len(sel), 2))
    for a, j in enumerate(sel):
        for d in range(2):
            kp, km = k_pi[j].copy(), k_pi[j].copy()
            kp[d] += h
            km[d] -= h
            fd[a, d] = (row_loss(kp, j) - row_loss(km, j)) / (2 * h)
    assert rel_l2(gk[sel], fd) < 1e-3

    # k-space data gradient of a loss on the adjoint: 2 A (A^H y - x0)
    ya = torch.from_numpy(y).cuda().reshape(1, C, M).requires_grad_(True)
    x0 = torch.from_numpy(img).cuda().reshape(1, 1, *shape)
    loss2 = torch.sum(torch.abs(ad.adj_op(ya) - x0) ** 2)
    loss2.backward()
    gy = ya.grad.cpu().numpy().reshape(C, M)
    z = sum(np.conj(smaps[c]) * ndft.ndft_type1(k, y[c], shape) for c in range(C)) / nf - xs
    rows = np.sort(rng.choice(M, 2048, replace=False))
    for c in rng.choice(C, 3, replace=False):
        ref = 2 * ndft.ndft_type2(k[rows], z * smaps[c], shape) / nf
        assert rel_l2(gy[c, rows], ref) < TOL


@pytest.mark.parametrize("index", [0, 3, 4, 5])
def test_served_templates_against_oracle_cg(gpu_pkg, index):
    """One served request of template ``index`` of the mixed stream (a8, a32,
    b16, c8) against the oracle's CG (10 iterations, step 1/L from the same
    seeded start vector) on the FP64 ES-kernel NUFFT."""
    from mrinufft_gb300 import workloads
    from mrinufft_gb300.serving import ReconRequest, ReconServer, start_vector
    from oracle import operator as oop

    key, _, kind, shape, C = workloads.SERVE_MIX[index]
    traj, smaps, img = workloads.serve_template(index)
    rng = np.random.default_rng(60 + index)
    op = gpu_pkg.MRIGB300(traj, shape, n_coils=C, smaps=smaps, squeeze_dims=False)
    y = np.asarray(op.op(img)).reshape(C, -1)
    y = (y + 0.01 * (rng.standard_normal(y.shape) + 1j * rng.standard_normal(y.shape))).astype(np.complex64)
    req = ReconRequest(rid=0, samples=traj, shape=shape, kspace=y, smaps=smaps, seed=11 + index)
    ReconServer(max_active=4).run([req], realtime=False)
    x = req.result.cpu().numpy().reshape(shape)

    ref = oop.EsOperator(traj.astype(np.float64), shape, smaps=smaps)
    single = oop.EsOperator(traj.astype(np.float64), shape)
    L, _ = oop.power_method(10, single.gram, start_vector(shape, 11 + index).reshape(1, 1, *shape))
    assert abs(float(req.lipschitz.cpu()) - L) / L < TOL
    x_ref = oop.cg(ref, y.reshape(1, C, -1), L, max_iter=10)
    assert rel_l2(x, x_ref.reshape(shape)) < TOL
