"""CUDA parity of op / adj_op / data_consistency against the FP64 NDFT.

Tolerance: relative l2 error <= 1e-4 against the FP64 NDFT at eps = 1e-6
(the accuracy bar of the backend), unless a test states otherwise.
"""

import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import ndft
from oracle.operator import NDFTOperator

pytestmark = pytest.mark.gpu

TOL = 1e-4
CASES = ["random2D", "random3D", "grid2D", "grid3D", "radial2D"]


def _case(golden, name):
    s = golden[f"{name}__samples"]
    shape = tuple(int(v) for v in golden[f"{name}__shape"])
    return s, shape


@pytest.mark.parametrize("name", CASES)
def test_op_adj_match_reference_ndft(gpu_pkg, golden, name):
    s, shape = _case(golden, name)
    op = gpu_pkg.MRIGB300(s, shape)
    y = op.op(golden[f"{name}__img"])
    x = op.adj_op(golden[f"{name}__ksp"])
    assert isinstance(y, np.ndarray) and y.dtype == np.complex64
    assert rel_l2(y, golden[f"{name}__op"]) < TOL
    assert rel_l2(x, golden[f"{name}__adj"]) < TOL


def test_sense_calibless_dc_batched(gpu_pkg, golden):
    s = golden["sense__samples"]
    shape = tuple(int(v) for v in golden["sense__shape"])
    smaps = golden["sense__smaps"]
    B, C = 2, smaps.shape[0]
    op = gpu_pkg.MRIGB300(s, shape, n_coils=C, n_batchs=B, smaps=smaps, squeeze_dims=True)
    assert rel_l2(op.op(golden["sense__img"]), golden["sense__op"]) < TOL
    assert rel_l2(op.adj_op(golden["sense__ksp"]), golden["sense__adj"]) < TOL
    assert rel_l2(op.data_consistency(golden["sense__img"], golden["sense__ksp"]),
                  golden["sense__dc"]) < TOL
    opc = gpu_pkg.MRIGB300(s, shape, n_coils=C, n_batchs=B, squeeze_dims=True)
    assert rel_l2(opc.op(golden["calib__img"]), golden["calib__op"]) < TOL
    assert rel_l2(opc.adj_op(golden["sense__ksp"]), golden["calib__adj"]) < TOL
    assert rel_l2(opc.data_consistency(golden["calib__img"], golden["sense__ksp"]),
                  golden["calib__dc"]) < TOL


def test_chunked_passes_equal_single_pass(gpu_pkg):
    # 5 coils in passes of 2 (small fine-grid budget) == all 5 in one pass
    rng = np.random.default_rng(3)
    shape = (40, 36)
    s = rng.uniform(-0.5, 0.5, (3000, 2)).astype(np.float32)
    smaps = (rng.standard_normal((5, *shape)) + 1j * rng.standard_normal((5, *shape))).astype(np.complex64)
    x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    big = gpu_pkg.MRIGB300(s, shape, n_coils=5, smaps=smaps)
    G = 80 * 72 * 8
    small = gpu_pkg.MRIGB300(s, shape, n_coils=5, smaps=smaps, fine_budget_bytes=2 * G)
    assert small._ntrans == 2 and big._ntrans == 5
    y1, y2 = big.op(x), small.op(x)
    assert rel_l2(y2, y1) < 1e-6
    assert rel_l2(small.adj_op(y1), big.adj_op(y1)) < 1e-6


def test_adjointness(gpu_pkg):
    # test_interfaces.py:138-158: <A x, y> == <x, A^H y>
    rng = np.random.default_rng(5)
    for shape, M in [((64, 48), 5000), ((24, 20, 28), 20000)]:
        s = rng.uniform(-0.5, 0.5, (M, len(shape))).astype(np.float32)
        op = gpu_pkg.MRIGB300(s, shape)
        rel = []
        for _ in range(5):
            x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
            y = (rng.standard_normal(M) + 1j * rng.standard_normal(M)).astype(np.complex64)
            lhs = np.vdot(op.op(x).astype(np.complex128), y)
            rhs = np.vdot(x.astype(np.complex128), op.adj_op(y))
            rel.append(abs(lhs - rhs) / abs(rhs))
        assert np.mean(rel) < 5e-5


def test_3d_multicoil_kooshball_subset(gpu_pkg, pkg):
    from mrinufft_gb300 import workloads

    traj = workloads.kooshball_3d(256, 64).reshape(-1, 3).astype(np.float32)
    shape = (32, 32, 32)
    img = workloads.phantom(shape, seed=1)
    smaps = workloads.coil_maps(shape, 4, seed=1)
    op = gpu_pkg.MRIGB300(traj, shape, n_coils=4, smaps=smaps)
    y = op.op(img)
    rows = np.random.default_rng(0).choice(traj.shape[0], 512, replace=False)
    nf = ndft.norm_factor(shape)
    for c in range(4):
        ref = ndft.ndft_type2_rows(traj, smaps[c] * img, shape, rows) / nf
        assert rel_l2(y[c, rows], ref) < TOL
    ksp = (np.random.default_rng(1).standard_normal((4, traj.shape[0])) * (1 + 0j)).astype(np.complex64)
    x = op.adj_op(ksp).reshape(-1)
    vox = np.random.default_rng(2).choice(np.prod(shape), 256, replace=False)
    ref = sum(np.conj(smaps[c].reshape(-1)[vox]) * ndft.ndft_type1_voxels(traj, ksp[c], shape, vox)
              for c in range(4)) / nf
    assert rel_l2(x[vox], ref) < TOL


@pytest.mark.parametrize("eps,tol", [(1e-6, 1e-4), (1e-3, 5e-3)])
@pytest.mark.parametrize("C", [1, 2, 3, 5])
def test_3d_dense_columns_coil_counts(gpu_pkg, eps, tol, C):
    # 3D adjoint with samples packed into a few columns of the fine grid (many
    # spread chunks per column, long z runs), for every coils-per-pass count
    # and both the fixed-width and the generic-width kernels
    rng = np.random.default_rng(13)
    shape = (24, 20, 28)
    M = 30000
    s = np.clip(rng.normal(0.0, 0.08, (M, 3)), -0.5, 0.4999)
    s[: M // 3, 2] = rng.uniform(-0.5, 0.5, M // 3)
    s[:2] = [[-0.5, -0.5, -0.5], [0.4999, 0.4999, 0.4999]]
    s = s.astype(np.float32)
    ksp = (rng.standard_normal((C, M)) + 1j * rng.standard_normal((C, M))).astype(np.complex64)
    op = gpu_pkg.MRIGB300(s, shape, n_coils=C, eps=eps)
    x = op.adj_op(ksp).reshape(C, -1)
    vox = rng.choice(int(np.prod(shape)), 200, replace=False)
    nf = ndft.norm_factor(shape)
    for c in range(C):
        ref = ndft.ndft_type1_voxels(s, ksp[c], shape, vox) / nf
        assert rel_l2(x[c, vox], ref) < tol


def test_pruned_fft_equals_full_fft(gpu_pkg, monkeypatch):
    # 3D transforms skip the all-zero planes of the padded grid; the result
    # must equal the full 3D FFT's (op, adj_op, data_consistency; several
    # transforms per pass so that the plane spans of neighbouring coils join)
    rng = np.random.default_rng(17)
    shape = (20, 17, 22)
    M, B, C = 4000, 2, 3
    s = rng.uniform(-0.5, 0.5, (M, 3)).astype(np.float32)
    smaps = (rng.standard_normal((C, *shape)) + 1j * rng.standard_normal((C, *shape))).astype(np.complex64)
    x = (rng.standard_normal((B, *shape)) + 1j * rng.standard_normal((B, *shape))).astype(np.complex64)
    y = (rng.standard_normal((B, C, M)) + 1j * rng.standard_normal((B, C, M))).astype(np.complex64)
    pruned = gpu_pkg.MRIGB300(s, shape, n_coils=C, n_batchs=B, smaps=smaps)
    monkeypatch.setenv("GBN_FFT_PRUNE", "0")
    full = gpu_pkg.MRIGB300(s, shape, n_coils=C, n_batchs=B, smaps=smaps)
    assert rel_l2(pruned.op(x), full.op(x)) < 1e-5
    assert rel_l2(pruned.adj_op(y), full.adj_op(y)) < 1e-5
    assert rel_l2(pruned.data_consistency(x, y), full.data_consistency(x, y)) < 1e-5


def test_density_and_boundaries(gpu_pkg):
    rng = np.random.default_rng(7)
    shape = (32, 32)
    s = rng.uniform(-0.5, 0.5, (1500, 2))
    s[:4] = [[-0.5, -0.5], [0.5 - 1e-7, 0.0], [0.0, -0.5], [-0.5, 0.49999]]
    d = rng.uniform(0.1, 2.0, s.shape[0]).astype(np.float32)
    op = gpu_pkg.MRIGB300(s.astype(np.float32), shape, density=d)
    ref = NDFTOperator(s.astype(np.float32), shape, density=d)
    y = (rng.standard_normal(s.shape[0]) + 1j * rng.standard_normal(s.shape[0])).astype(np.complex64)
    x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    assert rel_l2(op.adj_op(y), ref.adj(y)) < TOL
    assert rel_l2(op.op(x), ref.op(x)) < TOL
    assert rel_l2(op.data_consistency(x, y), ref.dc(x, y)) < TOL


@pytest.mark.parametrize("shape", [(33, 45), (15, 17, 19)])
def test_odd_sizes_integer_modes(gpu_pkg, shape):
    # odd sizes use finufft's integer modes -(N//2) .. N - N//2 - 1
    rng = np.random.default_rng(11)
    M = 3000
    s = rng.uniform(-0.5, 0.5, (M, len(shape))).astype(np.float32)
    op = gpu_pkg.MRIGB300(s, shape)
    ref = NDFTOperator(s, shape, grid="finufft")
    x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    y = (rng.standard_normal(M) + 1j * rng.standard_normal(M)).astype(np.complex64)
    assert rel_l2(op.op(x), ref.op(x)) < TOL
    assert rel_l2(op.adj_op(y), ref.adj(y)) < TOL


@pytest.mark.parametrize("eps,tol", [(1e-3, 5e-3), (1e-4, 5e-4), (1e-5, 5e-5)])
def test_other_eps_generic_width(gpu_pkg, golden, eps, tol):
    s, shape = _case(golden, "random2D")
    op = gpu_pkg.MRIGB300(s, shape, eps=eps)
    assert op.plan.info()["width"] != 7
    assert rel_l2(op.op(golden["random2D__img"]), golden["random2D__op"]) < tol
    assert rel_l2(op.adj_op(golden["random2D__ksp"]), golden["random2D__adj"]) < tol


def test_array_types_and_no_mutation(gpu_pkg, golden):
    s, shape = _case(golden, "random2D")
    op = gpu_pkg.MRIGB300(s, shape)
    img = golden["random2D__img"].astype(np.complex64)
    img_copy = img.copy()
    y_np = op.op(img)
    np.testing.assert_array_equal(img, img_copy)
    y_cpu = op.op(torch.from_numpy(img))
    assert isinstance(y_cpu, torch.Tensor) and y_cpu.device.type == "cpu"
    t = torch.from_numpy(img).cuda()
    t0 = t.clone()
    y_gpu = op.op(t)
    assert isinstance(y_gpu, torch.Tensor) and y_gpu.is_cuda
    assert torch.equal(t, t0)
    np.testing.assert_allclose(y_cpu.numpy(), y_np, rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(y_gpu.cpu().numpy(), y_np, rtol=1e-6, atol=1e-7)
    x_gpu = op.adj_op(y_gpu)
    assert x_gpu.is_cuda and x_gpu.shape == shape


def test_numpy_results_pinned_and_chained(gpu_pkg, golden, monkeypatch):
    """numpy results come back in page-locked memory, stay valid across later
    calls, and feed the next call (asynchronous copy) with the values of the
    device path; the pageable route gives the same values."""
    from mrinufft_gb300 import _array

    s, shape = _case(golden, "random2D")
    op = gpu_pkg.MRIGB300(s, shape)
    img = golden["random2D__img"]
    y = op.op(img)
    assert isinstance(y, np.ndarray) and torch.from_numpy(y).is_pinned()
    x = op.adj_op(y)
    assert isinstance(x, np.ndarray) and torch.from_numpy(x).is_pinned()
    t = torch.from_numpy(img).cuda()
    x_dev = op.adj_op(op.op(t)).cpu().numpy()
    # the adjoint's float atomics may add in another order from run to run
    np.testing.assert_allclose(x, x_dev, rtol=1e-5, atol=1e-6)
    y_copy = y.copy()
    for _ in range(3):
        op.adj_op(op.op(img * 2))
    np.testing.assert_array_equal(y, y_copy)
    monkeypatch.setattr(_array, "PINNED_RESULTS", False)
    y2 = op.op(img)
    assert not torch.from_numpy(y2).is_pinned()
    np.testing.assert_array_equal(y2, y_copy)
    np.testing.assert_allclose(op.adj_op(y2), x, rtol=1e-5, atol=1e-6)


def test_no_samples(gpu_pkg):
    op = gpu_pkg.MRIGB300(np.zeros((0, 2), np.float32), (16, 16))
    y = op.op(np.ones((16, 16), np.complex64))
    assert y.size == 0
    x = op.adj_op(np.zeros((0,), np.complex64))
    assert x.shape == (16, 16) and not np.any(x)


def test_shape_errors(gpu_pkg, golden):
    s, shape = _case(golden, "random2D")
    op = gpu_pkg.MRIGB300(s, shape)
    with pytest.raises(ValueError):
        op.op(np.zeros((shape[0] + 1, shape[1]), np.complex64))
    with pytest.raises(ValueError):
        op.adj_op(np.zeros(s.shape[0] + 1, np.complex64))
    with pytest.raises(ValueError):
        gpu_pkg.MRIGB300(s, shape, smaps=np.ones((2, 3, 3), np.complex64))


def test_update_samples_equals_fresh(gpu_pkg, golden):
    s, shape = _case(golden, "random2D")
    s2, _ = _case(golden, "radial2D")
    s2 = s2[:1000] * 0.9
    op = gpu_pkg.MRIGB300(s, shape)
    op.update_samples(s2)
    fresh = gpu_pkg.MRIGB300(s2, shape)
    img = golden["random2D__img"]
    np.testing.assert_allclose(op.op(img), fresh.op(img), rtol=1e-6, atol=1e-6)
