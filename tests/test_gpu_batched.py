"""Batched form (multi-stream graph and persistent work-table modes) ==
per-instance operators.

Tolerance: relative l2 <= 1e-5 between the batched and the single-instance
results (same kernels and arithmetic, different launch decomposition), and
exact equality between eager and CUDA-graph replays.
"""

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _instances(rng, dim=2):
    from mrinufft_gb300 import workloads

    out = []
    specs = [(40, 1, "radial"), (64, 3, "spiral"), (48, 2, "random"), (32, 4, "radial"),
             (56, 1, "spiral"), (36, 2, "random")] if dim == 2 else [(16, 2, "koosh"), (24, 1, "random"), (20, 3, "koosh")]
    for N, C, kind in specs:
        shape = (N,) * dim
        if kind == "radial":
            traj = workloads.radial_2d(int(rng.integers(16, 48)), int(rng.integers(64, 200))).reshape(-1, 2)
        elif kind == "spiral":
            traj = workloads.spiral_2d(int(rng.integers(4, 12)), int(rng.integers(200, 600)), power=2).reshape(-1, 2)
        elif kind == "koosh":
            traj = workloads.kooshball_3d(int(rng.integers(32, 96)), int(rng.integers(16, 48))).reshape(-1, 3)
        else:
            traj = rng.uniform(-0.5, 0.5, (int(rng.integers(500, 3000)), dim))
        smaps = (rng.standard_normal((C, *shape)) + 1j * rng.standard_normal((C, *shape))).astype(np.complex64)
        inst = {"samples": traj.astype(np.float32), "shape": shape, "smaps": smaps}
        if kind == "random":
            inst["density"] = rng.uniform(0.5, 1.5, traj.shape[0]).astype(np.float32)
        out.append(inst)
    return out


@pytest.mark.parametrize("mode", ["streams", "persistent"])
@pytest.mark.parametrize("dim", [2, 3])
def test_batched_equals_single(gpu_pkg, tmp_path, dim, mode):
    from mrinufft_gb300.autotune import Autotuner
    from mrinufft_gb300.batched import BatchedNufft

    rng = np.random.default_rng(dim)
    insts = _instances(rng, dim)
    tuner = Autotuner(cache_path=tmp_path / "tune.json", interp_methods=("auto",))
    bat = BatchedNufft(insts, tuner=tuner, mode=mode)
    assert (tmp_path / "tune.json").exists()
    imgs = [(rng.standard_normal(i["shape"]) + 1j * rng.standard_normal(i["shape"])).astype(np.complex64)
            for i in insts]
    bat.set_images(imgs)
    ksps = [k.clone() for k in bat.op()]
    xs = [x.clone() for x in bat.adj()]
    for inst, x0, y, x in zip(insts, imgs, ksps, xs):
        op = gpu_pkg.MRIGB300(inst["samples"], inst["shape"], n_coils=inst["smaps"].shape[0],
                              smaps=inst["smaps"], density=inst.get("density"), squeeze_dims=False)
        y_ref = op.op(torch.from_numpy(x0).cuda())
        assert rel_l2(y.cpu().numpy(), y_ref.cpu().numpy()) < 1e-5
        x_ref = op.adj_op(y)
        assert rel_l2(x.cpu().numpy(), x_ref.cpu().numpy()) < 1e-5


@pytest.mark.parametrize("mode", ["streams", "persistent"])
def test_batched_graph_replay(gpu_pkg, tmp_path, mode):
    from mrinufft_gb300.autotune import Autotuner
    from mrinufft_gb300.batched import BatchedNufft

    rng = np.random.default_rng(11)
    insts = _instances(rng, 2)
    bat = BatchedNufft(insts, tuner=Autotuner(cache_path=tmp_path / "t.json", interp_methods=("auto",)),
                       mode=mode)
    imgs = [(rng.standard_normal(i["shape"]) + 1j * rng.standard_normal(i["shape"])).astype(np.complex64)
            for i in insts]
    bat.set_images(imgs)
    bat.step()
    torch.cuda.synchronize()
    eager = [x.clone() for x in bat.imgs]
    bat.set_images(imgs)
    bat.capture()
    bat.set_images(imgs)
    bat.replay()
    torch.cuda.synchronize()
    for a, b in zip(eager, bat.imgs):
        assert rel_l2(b.cpu().numpy(), a.cpu().numpy()) < 1e-6


def test_batch_rejects_mismatched_dims(gpu_pkg, tmp_path):
    from mrinufft_gb300.batched import BatchedNufft

    rng = np.random.default_rng(0)
    insts = [_instances(rng, 2)[0], _instances(rng, 3)[0]]
    with pytest.raises(ValueError):
        BatchedNufft(insts, autotune=False)
