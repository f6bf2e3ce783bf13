"""Updates of the trajectory, density and coil maps of a live operator.

Mirrors mri-nufft's ``tests/operators/test_update.py:131-248``: after
``samples +=``, ``density +=`` / ``density = ...`` / ``density = None`` or
``smaps = ...`` on an existing operator, ``op`` and ``adj_op`` must equal
those of a fresh operator built from the updated attributes
(``update_operator``).  Tolerances are the reference's GPU ones: 1e-3
(absolute and relative) for the sample and density updates, 1e-4 for the
coil-map update of the adjoint, 6 decimals for the forward.
"""

import numpy as np
import numpy.testing as npt
import pytest

pytestmark = pytest.mark.gpu

CONFIGS = [(1, 1, False), (3, 1, False), (1, 4, True), (1, 4, False), (3, 2, True), (3, 2, False)]


def _traj(dim):
    rng = np.random.default_rng(dim)
    if dim == 2:
        return rng.uniform(-0.5, 0.5, (1000, 2)).astype(np.float32), (24, 20)
    return rng.uniform(-0.5, 0.5, (1500, 3)).astype(np.float32), (12, 10, 8)


def _make(pkg, dim, n_batch, n_coils, sense, density):
    np.random.seed(7)
    kspace_locs, shape = _traj(dim)
    smaps = None
    if sense:
        smaps = 1j * np.random.rand(n_coils, *shape)
        smaps += np.random.rand(n_coils, *shape)
        smaps = smaps.astype(np.complex64)
        smaps /= np.linalg.norm(smaps, axis=0)
    return pkg.MRIGB300(kspace_locs, shape, n_coils=n_coils, n_batchs=n_batch, squeeze_dims=False,
                        density=density, smaps=smaps)


def _fresh(pkg, op):
    """update_operator of the reference test: a new operator from the attributes."""
    smaps = op.smaps
    if smaps is not None:
        smaps = smaps.cpu().numpy()
    dens = op.density
    if dens is not None:
        dens = dens.cpu().numpy()
    return pkg.MRIGB300(op.samples, op.shape, n_coils=op.n_coils, n_batchs=op.n_batchs,
                        density=dens if dens is not None else False, smaps=smaps,
                        squeeze_dims=False)


def _image(op):
    shape = (op.n_batchs, *op.shape) if op.uses_sense else (op.n_batchs, op.n_coils, *op.shape)
    img = (1j * np.random.rand(*shape)).astype(np.complex64)
    img += np.random.rand(*shape).astype(np.complex64)
    return img


def _kspace(op):
    shape = (op.n_batchs, op.n_coils, op.n_samples)
    k = (1j * np.random.rand(*shape)).astype(np.complex64)
    k += np.random.rand(*shape).astype(np.complex64)
    return k


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("density", [False, True])
@pytest.mark.parametrize("n_batch,n_coils,sense", CONFIGS)
def test_update_samples_density_smaps(gpu_pkg, dim, density, n_batch, n_coils, sense):
    op = _make(gpu_pkg, dim, n_batch, n_coils, sense, density)
    img, ksp = _image(op), _kspace(op)

    # test_op_samples / test_adj_op_samples
    jitter = np.random.rand(*op.samples.shape).astype(np.float32)
    op.samples += jitter / 100
    new = _fresh(gpu_pkg, op)
    npt.assert_array_almost_equal(op.op(img), new.op(img))
    npt.assert_allclose(op.adj_op(ksp), new.adj_op(ksp), atol=1e-3, rtol=1e-3)

    # test_adj_op_density
    jitter = np.random.rand(op.n_samples).astype(np.float32)
    if op.uses_density:
        op.density += _like(op.density, jitter / 100)
    else:
        op.density = 1e-2 + jitter / 100
    new = _fresh(gpu_pkg, op)
    npt.assert_allclose(op.adj_op(ksp), new.adj_op(ksp), atol=1e-3, rtol=1e-3)
    op.density = None
    new = _fresh(gpu_pkg, op)
    assert not new.uses_density and not op.uses_density
    npt.assert_allclose(op.adj_op(ksp), new.adj_op(ksp), atol=1e-3, rtol=1e-3)

    # test_op_smaps_update / test_adj_op_smaps_update
    if sense:
        smaps = 1j * np.random.rand(op.n_coils, *op.shape)
        smaps += np.random.rand(op.n_coils, *op.shape)
        smaps = smaps.astype(np.complex64)
        smaps /= np.linalg.norm(smaps, axis=0)
        op.smaps = smaps
        new = _fresh(gpu_pkg, op)
        npt.assert_array_almost_equal(op.op(img), new.op(img))
        npt.assert_allclose(op.adj_op(ksp), new.adj_op(ksp), atol=1e-4, rtol=1e-4)


def _like(t, arr):
    """A host array in the device tensor's type (the reference adds an array
    of the density's own array module)."""
    import torch

    return torch.as_tensor(arr, device=t.device, dtype=t.dtype)
