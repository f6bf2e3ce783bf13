"""Low-frequency coil sensitivity estimation on the GPU against the reference's
own ``low_frequency`` (golden fixtures from ``tests/golden/make_smaps_golden.py``,
FP64 NDFT backend and the reference's LSQR).

Tolerance: relative l2 <= 1e-4.
"""

from pathlib import Path

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden" / "smaps_golden.npz"


@pytest.mark.parametrize("name", ["lowf_ellipse", "lowf_hann"])
def test_low_frequency_matches_reference(gpu_pkg, name):
    from mrinufft_gb300.smaps import low_frequency

    g = np.load(GOLD)
    shape = tuple(int(v) for v in g[f"{name}__shape"])
    maps = low_frequency(g[f"{name}__traj"].astype(np.float32), shape,
                         g[f"{name}__ksp"].astype(np.complex64), threshold=float(g[f"{name}__threshold"]),
                         window_fun=str(g[f"{name}__window"]), max_iter=10)
    assert maps.shape == g[f"{name}__maps"].shape
    assert rel_l2(maps, g[f"{name}__maps"]) < 1e-4


def test_operator_compute_smaps_low_frequency(gpu_pkg):
    g = np.load(GOLD)
    name = "lowf_ellipse"
    shape = tuple(int(v) for v in g[f"{name}__shape"])
    ksp = g[f"{name}__ksp"].astype(np.complex64)
    op = gpu_pkg.MRIGB300(g[f"{name}__traj"].astype(np.float32), shape, n_coils=ksp.shape[0],
                          smaps={"name": "low_frequency", "kspace_data": ksp,
                                 "threshold": float(g[f"{name}__threshold"])})
    assert op.uses_sense and op.n_coils == ksp.shape[0]
    assert rel_l2(op.smaps.cpu().numpy(), g[f"{name}__maps"]) < 1e-4
