"""Lipschitz constant, CG solver and pipe density against their CPU oracles.

Tolerances: the power-method eigenvalue within 1e-3 relative of the FP64
oracle run from the same start vector; CG images (10 iterations, nonlinear in
the data through beta) within 1e-3 relative l2 of the FP64 oracle with the
same step; pipe weights within 1e-3 relative l2 of the FP64 CPU pipe.
"""

import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import esnufft
from oracle import operator as oop

pytestmark = pytest.mark.gpu


def _case(seed=0, shape=(48, 40), M=4000, coils=3, sense=True):
    rng = np.random.default_rng(seed)
    s = np.clip(rng.normal(0, 0.16, (M, 2)), -0.499, 0.499).astype(np.float32)
    smaps = None
    if sense:
        smaps = (rng.standard_normal((coils, *shape)) + 1j * rng.standard_normal((coils, *shape)))
        smaps = (smaps / np.sqrt(np.sum(np.abs(smaps) ** 2, 0))).astype(np.complex64)
    return rng, s, shape, smaps


def _start_vector(shape):
    x = 1j * np.random.random(shape).astype(np.complex64)
    x += np.random.random(shape).astype(np.complex64)
    return x


def test_lipschitz_matches_oracle(gpu_pkg):
    rng, s, shape, smaps = _case()
    op = gpu_pkg.MRIGB300(s, shape, n_coils=3, smaps=smaps)
    np.random.seed(42)
    L = op.get_lipschitz_cst(max_iter=10)
    np.random.seed(42)
    x0 = _start_vector(shape)
    ref = oop.NDFTOperator(s, shape)  # single coil, no maps (base.py:647-665)
    L_ref, _ = oop.power_method(10, ref.gram, x0.reshape(1, 1, *shape))
    assert abs(L - L_ref) / L_ref < 1e-3
    # test_interfaces.py:161-176: L bounds ||A^H A||
    img = lambda: (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    Ls = []
    single = gpu_pkg.MRIGB300(s, shape)
    for _ in range(5):
        a, b = img(), img()
        Ls.append(np.linalg.norm(single.gram_op(b) - single.gram_op(a)) / np.linalg.norm(b - a))
    assert np.mean(Ls) < 1.1 * L


@pytest.mark.parametrize("density", [False, True])
def test_cg_matches_oracle(gpu_pkg, density):
    rng, s, shape, smaps = _case(seed=1)
    x_true = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    ref = oop.NDFTOperator(s, shape, smaps=smaps)
    y = ref.op(x_true).astype(np.complex64)
    op = gpu_pkg.MRIGB300(s, shape, n_coils=3, smaps=smaps, density=density)
    np.random.seed(3)
    x = op.pinv_solver(y, optim="cg", max_iter=10)
    np.random.seed(3)
    x0 = _start_vector(shape)
    L_ref, _ = oop.power_method(10, oop.NDFTOperator(
        s, shape, density=None if op.density is None else op.density.cpu().numpy()).gram,
        x0.reshape(1, 1, *shape))
    if density:
        ref.density = op.density.cpu().numpy().astype(np.float64)
    x_ref = oop.cg(ref, y, L_ref, max_iter=10)
    assert x.shape == shape
    assert rel_l2(x, x_ref) < 1e-3
    # the reconstruction moves towards the truth
    assert rel_l2(x, x_true) < 1.0


def _radial_nyquist_2d():
    from mrinufft_gb300 import workloads

    return workloads.radial_2d(128, 16).reshape(-1, 2), (32, 32)


def test_pipe_matches_cpu_oracle(gpu_pkg):
    traj, shape = _radial_nyquist_2d()
    w = gpu_pkg.MRIGB300.pipe(traj.astype(np.float32), shape, max_iter=10, osf=2)
    w_ref = esnufft.pipe(traj.astype(np.float32).astype(np.float64) * 2 * np.pi, shape, max_iter=10,
                         osf=2.0)
    assert isinstance(w, np.ndarray) and w.shape == (traj.shape[0],)
    assert np.all(w > 0)
    assert rel_l2(w, w_ref) < 1e-3


def _assert_correlate(a, b, slope=1.0, slope_err=None, r_err=None):
    # tests/helpers/asserts.py:50-70 of the reference
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    r = np.corrcoef(a, b)[0, 1]
    sl = np.cov(a, b)[0, 1] / np.var(a)
    if r_err is not None:
        assert abs(r - 1) <= r_err, r
    if slope_err is not None:
        assert abs(abs(sl) - slope) <= slope_err, sl


@pytest.mark.parametrize("osf", [1.5, 2])
def test_pipe_correlates_with_radius(gpu_pkg, osf):
    # test_density_for_op.py:20-57 with the finufft tolerances
    from mrinufft_gb300 import workloads

    # case_nyquist_radial3D of the reference: the 128 x 16 radial disc passed
    # through trajectories.tools.rotate with no tilt, i.e. the disc (z = 0)
    # repeated 128 times
    disc = workloads.radial_2d(128, 16)
    disc3 = np.concatenate([disc, np.zeros((*disc.shape[:2], 1))], axis=-1)
    for traj, shape in [_radial_nyquist_2d(),
                        (np.tile(disc3.reshape(-1, 3), (128, 1)), (32, 32, 32))]:
        res = gpu_pkg.MRIGB300.pipe(traj.astype(np.float32), shape, max_iter=10, osf=osf)
        dist = np.linalg.norm(traj, axis=-1)
        res = res / np.mean(res)
        dist = dist / np.mean(dist)
        r_err = (0.1 if osf == 2 else 0.2) * 3
        slope_err = 0.1 * 4 if osf == 2 else None
        _assert_correlate(res, dist, slope=1, slope_err=slope_err, r_err=r_err)


def test_density_true_uses_pipe(gpu_pkg):
    traj, shape = _radial_nyquist_2d()
    op = gpu_pkg.MRIGB300(traj.astype(np.float32), shape, density=True)
    w = gpu_pkg.MRIGB300.pipe(traj.astype(np.float32), shape)
    np.testing.assert_allclose(op.density.cpu().numpy(), w, rtol=1e-5)


@pytest.mark.parametrize("name", ["lsqr_sense", "lsqr_damp", "lsqr_calib"])
def test_lsqr_matches_reference(gpu_pkg, name):
    # tests/golden/lsqr_golden.npz: the reference's lsqr (10 iterations) on its
    # FP64 NDFT backend; pinv_solver's default optimizer
    from pathlib import Path

    g = np.load(Path(__file__).resolve().parent / "golden" / "lsqr_golden.npz")
    shape = tuple(int(v) for v in g[f"{name}__shape"])
    smaps = g[f"{name}__smaps"].astype(np.complex64) if f"{name}__smaps" in g else None
    C, B = int(g[f"{name}__n_coils"]), int(g[f"{name}__n_batchs"])
    op = gpu_pkg.MRIGB300(g[f"{name}__samples"].astype(np.float32), shape, n_coils=C, n_batchs=B,
                          smaps=smaps, squeeze_dims=False)
    kw = {"damp": float(g[f"{name}__damp"]), "max_iter": 10}
    if f"{name}__x0" in g:
        kw["x0"] = g[f"{name}__x0"].astype(np.complex64)
    x = op.pinv_solver(g[f"{name}__ksp"].astype(np.complex64), **kw)
    assert rel_l2(x, g[f"{name}__x"]) < 1e-4


CG_CASES = ["cg_sense", "cg_density", "cg_damp", "cg_calib", "cg_3d"]


def _cg_golden():
    from pathlib import Path

    return np.load(Path(__file__).resolve().parent / "golden" / "cg_golden.npz")


def _cg_operator(gpu_pkg, g, name):
    shape = tuple(int(v) for v in g[f"{name}__shape"])
    smaps = g[f"{name}__smaps"].astype(np.complex64) if f"{name}__smaps" in g else None
    dens = g[f"{name}__density"].astype(np.float32) if f"{name}__density" in g else False
    C, B = int(g[f"{name}__n_coils"]), int(g[f"{name}__n_batchs"])
    return gpu_pkg.MRIGB300(g[f"{name}__samples"].astype(np.float32), shape, n_coils=C, n_batchs=B,
                            smaps=smaps, density=dens, squeeze_dims=False)


@pytest.mark.parametrize("name", CG_CASES)
def test_lipschitz_matches_reference(gpu_pkg, name):
    # tests/golden/cg_golden.npz: the reference's power_method on its FP64
    # NDFT backend from the GPU backends' seeded start vector
    g = _cg_golden()
    op = _cg_operator(gpu_pkg, g, name)
    np.random.seed(int(g[f"{name}__seed"]))
    L = op.get_lipschitz_cst(max_iter=10)
    L_ref = float(g[f"{name}__lipschitz"])
    assert abs(L - L_ref) / L_ref < 1e-4, (L, L_ref)


@pytest.mark.parametrize("name", CG_CASES)
def test_cg_matches_reference(gpu_pkg, name):
    # tests/golden/cg_golden.npz: the reference's cg (extras/optim.py:801-902,
    # 10 iterations) on its FP64 NDFT backend, same seed
    g = _cg_golden()
    op = _cg_operator(gpu_pkg, g, name)
    kw = {"damp": float(g[f"{name}__damp"]), "max_iter": 10}
    if f"{name}__x0" in g:
        kw["x0"] = g[f"{name}__x0"].astype(np.complex64)
    np.random.seed(int(g[f"{name}__seed"]))
    x = op.pinv_solver(g[f"{name}__ksp"].astype(np.complex64), optim="cg", **kw)
    assert rel_l2(x, g[f"{name}__x"]) < 1e-4
