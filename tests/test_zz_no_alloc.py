"""gbn_pipe_static: the pipe iteration for callers that cannot allocate.

Some callers cannot call cudaMalloc when they need the density estimate: a
process whose device memory belongs to another framework's pool (JAX and
TensorFlow reserve most of it up front), or a real-time reconstruction
service that allows no allocation after start-up.  ``gbn_pipe_static`` runs
the ``gbn_pipe`` iteration with its grid in a fixed device array of the
library instead of a plan's memory.  These tests call it through the C ABI
and check, on two calls in a row, that its weights match those of the plan
path (``gbn_plan_create`` + ``gbn_setpts`` + ``gbn_pipe``) within the 1e-4
relative l2 tolerance the parity tests use, and that grids larger than the
array are refused.

The file is named so that pytest collects it last.
"""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _cases():
    from mrinufft_gb300 import workloads

    yield workloads.radial_2d(128, 16).reshape(-1, 2), (32, 32)
    yield workloads.kooshball_3d(256, 32).reshape(-1, 3), (24, 24, 24)
    rng = np.random.default_rng(9)
    yield rng.uniform(-0.5, 0.5, (5000, 2)), (48, 40)


def _plan_pipe(pkg, k, shape, iters, scale2):
    plan = pkg.NufftPlan(shape, eps=1e-6, upsampfac=2.0, ntrans=1, spread_only=True)
    plan.setpts(k)
    w = torch.ones(k.shape[0], dtype=torch.complex64, device="cuda")
    plan.pipe(w, iters, scale2)
    return w


def _static_pipe(lib, k, shape, iters, scale2):
    cols = [k[:, d].contiguous() for d in range(k.shape[1])]
    ptrs = [ctypes.c_void_p(c.data_ptr()) for c in cols] + [None] * (3 - len(cols))
    w = torch.ones(k.shape[0], dtype=torch.complex64, device="cuda")
    dims = (ctypes.c_int64 * len(shape))(*shape)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = lib.gbn_pipe_static(len(shape), dims, 2.0, 1e-6, k.shape[0], ptrs[0], ptrs[1], ptrs[2],
                             ctypes.c_void_p(w.data_ptr()), iters, scale2, stream)
    assert st == 0, lib.gbn_last_error()
    return w


def test_static_pipe_matches_plan_pipe(gpu_pkg):
    lib = gpu_pkg.load_library()
    for traj, shape in _cases():
        k = torch.from_numpy(np.asarray(traj, np.float32) * np.float32(2 * np.pi)).cuda()
        nrm = float(np.sqrt(np.prod(shape) * 2 ** len(shape)))
        scale2 = 1.0 / (nrm * nrm)
        ref = _plan_pipe(gpu_pkg, k, shape, 10, scale2)
        for _ in range(2):  # two calls in a row share the static grid
            w = _static_pipe(lib, k, shape, 10, scale2)
            torch.cuda.synchronize()
            err = float(torch.linalg.vector_norm(w - ref) / torch.linalg.vector_norm(ref))
            assert err < TOL, (shape, err)


@pytest.mark.parametrize("dims", [(256, 256, 256), (2097152, 2097152, 2097152), (1, 2097153, 1),
                                  (2048, 1025, 1)])
def test_static_pipe_rejects_oversize_grid(gpu_pkg, dims):
    """Grids beyond the array, including sizes whose cell count would not fit
    64 bits, are refused before anything runs and leave w untouched."""
    lib = gpu_pkg.load_library()
    k = torch.zeros((4, 3), dtype=torch.float32, device="cuda")
    cols = [k[:, d].contiguous() for d in range(3)]
    w = torch.ones(4, dtype=torch.complex64, device="cuda")
    cdims = (ctypes.c_int64 * 3)(*dims)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = lib.gbn_pipe_static(3, cdims, 2.0, 1e-6, 4, *[ctypes.c_void_p(c.data_ptr()) for c in cols],
                             ctypes.c_void_p(w.data_ptr()), 1, 1.0, stream)
    torch.cuda.synchronize()
    assert st == 1
    assert b"exceeds the static grid" in lib.gbn_last_error()
    assert torch.all(w == 1)


def test_static_pipe_osf_rule_matches_plan(gpu_pkg):
    """An oversampling factor <= 1 takes the osf = 2 kernel on both paths."""
    lib = gpu_pkg.load_library()
    from mrinufft_gb300 import workloads

    shape = (40, 40)
    k = torch.from_numpy(workloads.radial_2d(96, 32).reshape(-1, 2).astype(np.float32) *
                         np.float32(2 * np.pi)).cuda()
    scale2 = 1.0 / (np.prod(shape) * 4.0)
    plan = gpu_pkg.NufftPlan(shape, eps=1e-6, upsampfac=1.0, ntrans=1, spread_only=True)
    plan.setpts(k)
    ref = torch.ones(k.shape[0], dtype=torch.complex64, device="cuda")
    plan.pipe(ref, 5, scale2)
    cols = [k[:, d].contiguous() for d in range(2)]
    w = torch.ones(k.shape[0], dtype=torch.complex64, device="cuda")
    dims = (ctypes.c_int64 * 2)(*shape)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = lib.gbn_pipe_static(2, dims, 1.0, 1e-6, k.shape[0], ctypes.c_void_p(cols[0].data_ptr()),
                             ctypes.c_void_p(cols[1].data_ptr()), None, ctypes.c_void_p(w.data_ptr()),
                             5, scale2, stream)
    assert st == 0, lib.gbn_last_error()
    torch.cuda.synchronize()
    err = float(torch.linalg.vector_norm(w - ref) / torch.linalg.vector_norm(ref))
    assert err < TOL, err
