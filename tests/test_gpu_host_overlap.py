"""numpy host arrays of many coils through op / adj_op.

Above 32 MB of k-space, op of a numpy image transforms coil groups whose
device-to-host copies into the page-locked result overlap the next group's
kernels.  The results must equal those of the device-array path (same
kernels on the same coils: relative l2 <= 1e-6), for SENSE and
calibrationless operators, several batches, with and without density; the
page-locked result fed back to adj_op (asynchronous copy) and pageable
k-space give the device path's adjoint.
"""

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("sense", [True, False])
@pytest.mark.parametrize("density", [False, True])
def test_host_groups_equal_device_path(gpu_pkg, sense, density):
    rng = np.random.default_rng(3)
    shape, C, B, M = (40, 36, 32), 9, 2, 480000
    k = np.clip(rng.normal(0, 0.15, (M, 3)), -0.5, 0.4999).astype(np.float32)
    smaps = ((rng.standard_normal((C, *shape)) + 1j * rng.standard_normal((C, *shape))).astype(np.complex64)
             if sense else None)
    dens = rng.uniform(0.5, 1.5, M).astype(np.float32) if density else False
    op = gpu_pkg.MRIGB300(k, shape, n_coils=C, n_batchs=B, smaps=smaps, density=dens, squeeze_dims=False)
    assert op._host_groups() > 1
    img_shape = (B, 1, *shape) if sense else (B, C, *shape)
    x = (rng.standard_normal(img_shape) + 1j * rng.standard_normal(img_shape)).astype(np.complex64)
    y = (rng.standard_normal((B, C, M)) + 1j * rng.standard_normal((B, C, M))).astype(np.complex64)
    y_host = op.op(x)
    assert isinstance(y_host, np.ndarray) and y_host.shape == (B, C, M)
    assert torch.from_numpy(y_host).is_pinned()
    y_dev = op.op(torch.from_numpy(x).cuda()).cpu().numpy()
    assert rel_l2(y_host, y_dev) < 1e-6
    # pageable k-space
    z_host = op.adj_op(y)
    assert isinstance(z_host, np.ndarray) and z_host.shape == img_shape
    z_dev = op.adj_op(torch.from_numpy(y).cuda()).cpu().numpy()
    assert rel_l2(z_host, z_dev) < 1e-6
    # page-locked k-space (an op result)
    z_pin = op.adj_op(y_host)
    assert z_pin.shape == img_shape
    assert rel_l2(z_pin, op.adj_op(torch.from_numpy(y_dev).cuda()).cpu().numpy()) < 1e-6
    # twice in a row (the copy stream and buffers are reused)
    assert rel_l2(op.adj_op(op.op(x)), z_pin) < 1e-6
