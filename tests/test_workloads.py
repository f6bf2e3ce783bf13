"""The synthetic trajectory generators against mri-nufft's own.

``tests/golden/traj_golden.npz`` holds trajectories written by the
reference's ``initialize_2D_radial``, ``initialize_3D_phyllotaxis_radial`` and
``initialize_2D_spiral(..., spiral="galilean")`` (``make_traj_golden.py``),
at the sizes the benchmark configurations use and at small sizes.  The
benchmark casts trajectories to float32, so they must agree there to within
two float32 ulps of the largest coordinate (0.5).
"""

from pathlib import Path

import numpy as np
import pytest

G = np.load(Path(__file__).resolve().parent / "golden" / "traj_golden.npz")
ATOL = 2 * np.spacing(np.float32(0.5))


def _cases(prefix):
    return sorted({k.split("__")[0] for k in G.files if k.startswith(prefix)})


def _check(name, traj):
    shape = tuple(G[f"{name}__shape"])
    assert traj.shape == shape, (traj.shape, shape)
    flat = traj.reshape(-1, shape[-1])
    f32 = flat.astype(np.float32)
    if f"{name}__full" in G.files:
        np.testing.assert_allclose(f32, G[f"{name}__full"].astype(np.float32), rtol=0, atol=ATOL)
        return
    idx = G[f"{name}__idx"]
    np.testing.assert_allclose(f32[idx], G[f"{name}__sub"].astype(np.float32), rtol=0, atol=ATOL)
    np.testing.assert_allclose(traj[0].astype(np.float32), G[f"{name}__first"].astype(np.float32),
                               rtol=0, atol=ATOL)
    if f"{name}__ends" in G.files:
        np.testing.assert_allclose(traj[:, -1, :].astype(np.float32), G[f"{name}__ends"], rtol=0,
                                   atol=ATOL)


@pytest.mark.parametrize("name", _cases("radial2d"))
def test_radial_2d(pkg, name):
    from mrinufft_gb300 import workloads

    Nc, Ns = map(int, name.split("_")[1:])
    _check(name, workloads.radial_2d(Nc, Ns))


@pytest.mark.parametrize("name", _cases("koosh3d"))
def test_phyllotaxis_kooshball(pkg, name):
    from mrinufft_gb300 import workloads

    Nc, Ns = map(int, name.split("_")[1:])
    _check(name, workloads.kooshball_3d(Nc, Ns))


@pytest.mark.parametrize("name", _cases("spiral2d"))
def test_galilean_spiral(pkg, name):
    from mrinufft_gb300 import workloads

    Nc, Ns = map(int, name.split("_")[1:])
    _check(name, workloads.spiral_2d(Nc, Ns, power=2))


def test_benchmark_configs_use_reference_trajectories(pkg):
    """The 2D single-coil and 3D multi-coil configurations are the
    reference's 100 x 500 radial and 4096 x 512 phyllotaxis kooshball."""
    from mrinufft_gb300 import workloads

    t1, _, _ = workloads.config1()
    g = "radial2d_100_500"
    np.testing.assert_allclose(t1[G[f"{g}__idx"]], G[f"{g}__sub"].astype(np.float32), rtol=0, atol=ATOL)
    t2 = workloads.kooshball_3d(4096, 512).reshape(-1, 3).astype(np.float32)
    g = "koosh3d_4096_512"
    np.testing.assert_allclose(t2[G[f"{g}__idx"]], G[f"{g}__sub"].astype(np.float32), rtol=0, atol=ATOL)
