"""Off-resonance corrected operator on the GPU against the reference's own
``MRIFourierCorrected`` (golden fixtures from
``tests/golden/make_offres_golden.py``, FP64 NDFT backend).

Tolerance: relative l2 <= 1e-4 (eps = 1e-6 transforms; for the factorised
cases the interpolators are recomputed here and agree to ~1e-5).
"""

from pathlib import Path

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-4
GOLD = Path(__file__).resolve().parent / "golden" / "offres_golden.npz"


def _make(gpu_pkg, g, name, interpolator=None):
    shape = tuple(int(v) for v in g[f"{name}__shape"])
    smaps = g[f"{name}__smaps"].astype(np.complex64) if f"{name}__smaps" in g else None
    C = int(g[f"{name}__n_coils"])
    op = gpu_pkg.MRIGB300(g[f"{name}__samples"].astype(np.float32), shape, n_coils=C, smaps=smaps,
                          squeeze_dims=False)
    if interpolator is None:
        interpolator = (g[f"{name}__B"], g[f"{name}__C"])
    return gpu_pkg.MRIFourierCorrectedGB300(op, b0_map=g[f"{name}__b0"], readout_time=g[f"{name}__t"],
                                            interpolator=interpolator)


@pytest.mark.parametrize("name", ["orc_tuple", "orc_svd", "orc_mti3d"])
def test_op_adj_with_reference_interpolators(gpu_pkg, name):
    g = np.load(GOLD)
    cor = _make(gpu_pkg, g, name)
    y = cor.op(g[f"{name}__img"].astype(np.complex64))
    assert rel_l2(y, g[f"{name}__op"]) < TOL
    x = cor.adj_op(g[f"{name}__ksp"].astype(np.complex64))
    assert rel_l2(x, g[f"{name}__adj"]) < TOL


@pytest.mark.parametrize("name,method", [("orc_svd", "svd"), ("orc_mti3d", "mti")])
def test_factorisations_end_to_end(gpu_pkg, name, method):
    g = np.load(GOLD)
    cor = _make(gpu_pkg, g, name, interpolator=method)
    assert cor.n_interpolators == g[f"{name}__B"].shape[1]
    assert rel_l2(cor.op(g[f"{name}__img"].astype(np.complex64)), g[f"{name}__op"]) < TOL
    assert rel_l2(cor.adj_op(g[f"{name}__ksp"].astype(np.complex64)), g[f"{name}__adj"]) < TOL


def test_adjointness_dc_and_lipschitz(gpu_pkg):
    g = np.load(GOLD)
    name = "orc_tuple"
    cor = _make(gpu_pkg, g, name)
    rng = np.random.default_rng(41)
    x = (rng.standard_normal((1, 1, 16, 12)) + 1j * rng.standard_normal((1, 1, 16, 12))).astype(np.complex64)
    y = (rng.standard_normal((1, 2, 240)) + 1j * rng.standard_normal((1, 2, 240))).astype(np.complex64)
    lhs = np.vdot(cor.op(x).astype(np.complex128), y)
    rhs = np.vdot(x.astype(np.complex128), cor.adj_op(y))
    assert abs(lhs - rhs) / abs(rhs) < 5e-5
    dc = cor.data_consistency(x, y)
    assert rel_l2(dc, cor.adj_op(cor.op(x) - y)) < 1e-5
    xt = torch.from_numpy(x).cuda()
    assert isinstance(cor.op(xt), torch.Tensor)
    L = cor.get_lipschitz_cst(20)
    assert np.isfinite(L) and L > 0
