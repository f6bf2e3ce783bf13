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


@pytest.mark.parametrize("gram", ["toeplitz", "nufft"])
def test_alone_equals_plain_both_grams(gpu_pkg, gram):
    """Both served iteration forms equal the plain per-call CG (the NUFFT
    form exactly the same arithmetic; the Toeplitz form through its own
    option of the plain solver too)."""
    from mrinufft_gb300.serving import ReconServer

    rng = np.random.default_rng(3)
    reqs = _requests(rng)
    srv = ReconServer(max_active=8, gram=gram)
    done = {r.rid: r for r in srv.run([_copy(r) for r in reqs], realtime=False)}
    for r in reqs:
        op = gpu_pkg.MRIGB300(r.samples, r.shape, n_coils=r.n_coils, smaps=r.smaps,
                              density=r.density)
        np.random.seed(r.seed)
        x = op.pinv_solver(r.kspace, optim="cg", max_iter=10, toeplitz=gram == "toeplitz")
        assert rel_l2(done[r.rid].result.cpu().numpy(), x) < 1e-4


def test_budget_limits_concurrency(gpu_pkg):
    from mrinufft_gb300.serving import ReconServer, plan_set_bytes, solve_bytes

    rng = np.random.default_rng(1)
    reqs = _requests(rng)[:2] * 3
    reqs = [_copy(r, rid=i) for i, r in enumerate(reqs)]
    one = max(plan_set_bytes(r.shape, r.kspace.shape[1], r.n_coils)
              + solve_bytes(r.shape, r.kspace.shape[1], r.n_coils) for r in reqs)
    budget = 2.5 * one
    srv = ReconServer(hbm_budget_bytes=budget, max_active=8)
    srv.prewarm(reqs)
    assert srv.ledger.total <= budget
    peak = 0
    for r in reqs:
        srv.submit(r)
    while not srv.idle():
        srv.tick()
        peak = max(peak, len(srv.active) + len(srv.finishing))
        assert srv.ledger.total <= budget
    torch.cuda.synchronize()
    assert len(srv.done) == len(reqs)
    assert peak <= 2
    assert srv.ledger.peak <= budget


def test_plan_set_estimate_bounds_library_bytes(gpu_pkg):
    """The ledger's per-trajectory charge is at least what the library
    allocates for the plan and its Toeplitz embedding."""
    from mrinufft_gb300.plan import NufftPlan, ToeplitzKernel
    from mrinufft_gb300.serving import plan_set_bytes

    rng = np.random.default_rng(2)
    for r in _requests(rng):
        k = torch.from_numpy(np.asarray(r.samples, np.float32) * np.float32(2 * np.pi)).cuda()
        plan = NufftPlan(tuple(r.shape), eps=1e-6, ntrans=r.n_coils)
        plan.setpts(k)
        toep = ToeplitzKernel(plan, None)
        inner = toep.inner_device_bytes()
        assert plan.device_bytes + inner <= plan_set_bytes(r.shape, k.shape[0], r.n_coils)
        del toep, plan
