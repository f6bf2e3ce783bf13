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


ESP = Path(__file__).resolve().parent / "golden" / "espirit_golden.npz"


def _masked_cmp(maps, eig, g, name, crop=0.95, margin=1e-3):
    """Eigenvalues everywhere; maps only where the mask decision is not within
    ``margin`` of the crop threshold (a float32 eigenvalue there may fall on
    either side)."""
    e_ref = g[f"{name}__eig"]
    assert rel_l2(eig, e_ref) < 1e-4
    sure = np.abs(e_ref - crop) > margin
    inside = sure & (e_ref > crop)
    assert inside.sum() > 0.1 * inside.size
    ref = g[f"{name}__maps"]
    assert rel_l2(maps[:, inside], ref[:, inside]) < 1e-4
    return sure


@pytest.mark.parametrize("name", ["cart2d", "cart3d"])
def test_cartesian_espirit_matches_reference(gpu_pkg, name):
    # tests/golden/espirit_golden.npz: the reference's ESPIRiT steps
    # (extras/smaps.py:393-463) on its own helpers
    from mrinufft_gb300.smaps import cartesian_espirit, espirit_eigen

    g = np.load(ESP)
    shape = tuple(int(v) for v in g[f"{name}__shape"])
    cw, kw = int(g[f"{name}__calib_width"]), int(g[f"{name}__kernel_width"])
    maps, eig = espirit_eigen(g[f"{name}__kspace"], cw, kw, 0.02)
    sure = _masked_cmp(maps.cpu().numpy(), eig.cpu().numpy(), g, name)
    out = cartesian_espirit(g[f"{name}__kspace"], shape, cw, kw, 0.02, 0.95)
    assert isinstance(out, np.ndarray) and out.shape == (g[f"{name}__kspace"].shape[0], *shape)
    assert rel_l2(out[:, sure], g[f"{name}__masked"][:, sure]) < 1e-4


def test_espirit_non_cartesian_matches_reference(gpu_pkg):
    # the non-Cartesian front end: rectangle of the k-space centre, LSQR on
    # the device, centred FFT, then the Cartesian steps
    from mrinufft_gb300.smaps import espirit

    g = np.load(ESP)
    name = "radial"
    shape = tuple(int(v) for v in g[f"{name}__shape"])
    cw, kw = int(g[f"{name}__calib_width"]), int(g[f"{name}__kernel_width"])
    out = espirit(g[f"{name}__samples"].astype(np.float32), shape,
                  g[f"{name}__kspace"].astype(np.complex64), calib_width=cw, kernel_width=kw)
    e_ref = g[f"{name}__eig"]
    sure = np.abs(e_ref - 0.95) > 1e-3
    # the fixture's front end runs the reference's LSQR in complex64, as this
    # backend does (in FP64 it moves by 5e-3 on this system)
    assert rel_l2(out[:, sure], g[f"{name}__masked"][:, sure]) < 1e-4


def test_operator_compute_smaps_espirit(gpu_pkg):
    g = np.load(ESP)
    name = "radial"
    shape = tuple(int(v) for v in g[f"{name}__shape"])
    ksp = g[f"{name}__kspace"].astype(np.complex64)
    op = gpu_pkg.MRIGB300(g[f"{name}__samples"].astype(np.float32), shape, n_coils=ksp.shape[0],
                          smaps={"name": "espirit", "kspace_data": ksp,
                                 "calib_width": int(g[f"{name}__calib_width"]),
                                 "kernel_width": int(g[f"{name}__kernel_width"])})
    assert op.uses_sense and op.smaps.shape == (ksp.shape[0], *shape)
