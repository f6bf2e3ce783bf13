"""Served form: results are the same alone and in a mix, and equal the plain
operator's CG; admission respects the HBM budget.

Tolerances: alone vs in the mix, relative l2 <= 1e-5 (same kernels, only the
order of floating-point atomics differs); served vs ``MRIGB300.pinv_solver``
with the same power-method start vector, relative l2 <= 1e-4.
"""

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _requests(rng, first_id=0):
    from mrinufft_gb300 import workloads
    from mrinufft_gb300.serving import ReconRequest

    reqs = []
    specs = [
        ("radial", (48, 48), 4, None),
        ("spiral", (40, 40), 3, None),
        ("koosh", (20, 20, 20), 2, None),
        ("radial", (48, 48), 4, "density"),
        ("random", (32, 36), 2, None),
    ]
    for i, (kind, shape, C, dens) in enumerate(specs):
        if kind == "radial":
            traj = workloads.radial_2d(32, 96).reshape(-1, 2)
        elif kind == "spiral":
            traj = workloads.spiral_2d(8, 300, power=2).reshape(-1, 2)
        elif kind == "koosh":
            traj = workloads.kooshball_3d(96, 32).reshape(-1, 3)
        else:
            traj = rng.uniform(-0.5, 0.5, (2500, 2))
        traj = traj.astype(np.float32)
        M = traj.shape[0]
        smaps = workloads.coil_maps(shape, C, seed=i)
        x = workloads.phantom(shape, seed=i)
        from oracle.operator import NDFTOperator

        y = NDFTOperator(traj, shape, smaps=smaps).op(x).reshape(C, M).astype(np.complex64)
        y += (0.01 * (rng.standard_normal(y.shape) + 1j * rng.standard_normal(y.shape))).astype(np.complex64)
        d = None
        if dens:
            d = rng.uniform(0.5, 1.5, M).astype(np.float32)
        reqs.append(ReconRequest(rid=first_id + i, samples=traj, shape=shape, kspace=y, smaps=smaps,
                                 density=d, seed=100 + i, traj_key=f"{kind}{shape}"))
    return reqs


def _copy(r, rid=None):
    from mrinufft_gb300.serving import ReconRequest

    return ReconRequest(rid=r.rid if rid is None else rid, samples=r.samples, shape=r.shape,
                        kspace=r.kspace, smaps=r.smaps, density=r.density, seed=r.seed,
                        traj_key=r.traj_key)


def test_alone_equals_mix_equals_plain(gpu_pkg):
    from mrinufft_gb300.serving import ReconServer

    rng = np.random.default_rng(0)
    reqs = _requests(rng)
    alone = {}
    for r in reqs:
        srv = ReconServer(max_active=4)
        out = srv.run([_copy(r)], realtime=False)
        alone[r.rid] = out[0].result.cpu().numpy()
    srv = ReconServer(max_active=8)
    mix = [_copy(r) for r in reqs] + [_copy(r, rid=100 + r.rid) for r in reqs]
    done = srv.run(mix, realtime=False)
    assert len(done) == len(mix)
    for r in done:
        assert rel_l2(r.result.cpu().numpy(), alone[r.rid % 100]) < 1e-5
    for r in reqs:
        op = gpu_pkg.MRIGB300(r.samples, r.shape, n_coils=r.n_coils, smaps=r.smaps,
                              density=r.density)
        np.random.seed(r.seed)
        x = op.pinv_solver(r.kspace, optim="cg", max_iter=10)
        assert rel_l2(alone[r.rid], x) < 1e-4


def test_budget_limits_concurrency(gpu_pkg):
    from mrinufft_gb300.serving import ReconServer, request_bytes

    rng = np.random.default_rng(1)
    reqs = _requests(rng)[:2] * 3
    reqs = [_copy(r, rid=i) for i, r in enumerate(reqs)]
    one = max(request_bytes(r.shape, r.kspace.shape[1], r.n_coils) for r in reqs)
    srv = ReconServer(hbm_budget_bytes=1.5 * one, max_active=8)
    peak = 0
    pending = list(reqs)
    for r in pending:
        srv.submit(r)
    while not srv.idle():
        srv.tick()
        peak = max(peak, len(srv.active) + len(srv.finishing))
        assert srv.used <= 1.5 * one or len(srv.active) + len(srv.finishing) == 1
    torch.cuda.synchronize()
    assert len(srv.done) == len(reqs)
    assert peak <= 2
