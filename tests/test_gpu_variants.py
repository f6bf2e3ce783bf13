"""Every kernel variant that an environment setting can select, against the
FP64 NDFT oracle.

``gbn_plan_create`` reads tuning overrides from the environment: the spread
kernel (``GBN_SPREAD``: per-sample global atomics, warp-cooperative atomics,
column streaming, bin-tile rows, quadrant streaming, quadrant tiles on the
tensor cores), the interpolation kernel
(``GBN_INTERP``: direct, double-buffered tiles, warp-cooperative, tile +
warp-cooperative, tiles), coils per pass (``GBN_INTERP_CG``,
``GBN_SPREAD_CG``), the interp CTA size (``GBN_INTERP_THREADS``), the bin
sizes (``GBN_BINS2`` / ``GBN_BINS3``) and the pruned 3D FFT
(``GBN_FFT_PRUNE``).  Each setting runs SENSE op, adj and data consistency
in 2D and 3D (and a calibrationless case) with relative l2 <= 1e-4.  The
fused 256^3 transforms (``GBN_FUSED_FFT``) need 256-point fine axes and are
covered by test_gpu_fft256.py.
"""

import os

import numpy as np
import pytest

from conftest import rel_l2
from oracle.operator import NDFTOperator

pytestmark = pytest.mark.gpu

TOL = 1e-4

VARIANTS = [
    {},
    {"GBN_SPREAD": "gm"}, {"GBN_SPREAD": "wc"}, {"GBN_SPREAD": "stream"},
    {"GBN_SPREAD": "rows"}, {"GBN_SPREAD": "quad"}, {"GBN_SPREAD": "mma"},
    {"GBN_QUAD_PACKED": "0"},
    {"GBN_INTERP": "gm"}, {"GBN_INTERP": "db"}, {"GBN_INTERP": "wc"},
    {"GBN_INTERP": "twc"}, {"GBN_INTERP": "tile"},
    {"GBN_INTERP_CG": "2"}, {"GBN_INTERP_CG": "4"},
    {"GBN_SPREAD_CG": "1"}, {"GBN_SPREAD_CG": "2"},
    {"GBN_INTERP_THREADS": "64"},
    {"GBN_BINS2": "16,16", "GBN_BINS3": "9,9,9"},
    {"GBN_BINS2": "25,32", "GBN_BINS3": "4,4,4"},
    {"GBN_BINS2": "8,8", "GBN_BINS3": "16,16,16"},
    {"GBN_FFT_PRUNE": "0"},
    {"GBN_SPREAD": "stream", "GBN_BINS3": "12,12,8"},
]


def _ids(v):
    return ",".join(f"{k}={x}" for k, x in v.items()) or "default"


def _case(dim, sense, seed):
    rng = np.random.default_rng(seed)
    if dim == 2:
        shape, M = (48, 40), 3000
        k = np.concatenate([rng.uniform(-0.5, 0.5, (M // 2, 2)),
                            np.clip(rng.normal(0, 0.08, (M // 2, 2)), -0.5, 0.4999)])
    else:
        shape, M = (20, 18, 16), 4000
        k = np.concatenate([rng.uniform(-0.5, 0.5, (M // 2, 3)),
                            np.clip(rng.normal(0, 0.08, (M // 2, 3)), -0.5, 0.4999)])
    C = 4
    cpx = lambda *s: (rng.standard_normal(s) + 1j * rng.standard_normal(s)).astype(np.complex64)
    smaps = cpx(C, *shape) if sense else None
    x = cpx(1, *shape) if sense else cpx(1, C, *shape)
    y = cpx(1, C, M)
    dens = rng.uniform(0.5, 1.5, M).astype(np.float32)
    return k.astype(np.float32), shape, smaps, x, y, dens


@pytest.mark.parametrize("env", VARIANTS, ids=_ids)
@pytest.mark.parametrize("dim,sense", [(2, True), (3, True), (2, False), (3, False)])
def test_variant_matches_oracle(gpu_pkg, monkeypatch, env, dim, sense):
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    k, shape, smaps, x, y, dens = _case(dim, sense, seed=dim * 10 + sense)
    C = 4
    op = gpu_pkg.MRIGB300(k, shape, n_coils=C, smaps=smaps, density=dens, squeeze_dims=False)
    ref = NDFTOperator(k.astype(np.float64), shape, n_coils=C, smaps=smaps, density=dens)
    assert rel_l2(op.op(x), ref.op(x)) < TOL
    assert rel_l2(op.adj_op(y), ref.adj(y)) < TOL
    assert rel_l2(op.data_consistency(x, y), ref.dc(x, y)) < TOL


@pytest.mark.parametrize("env", [{}, {"GBN_SPREAD_CG": "8"}, {"GBN_QUAD_MINB": "4"},
                                 {"GBN_QUAD_PACKED": "0"}, {"GBN_SPREAD": "mma"}], ids=_ids)
@pytest.mark.parametrize("C", [8, 9, 17])
def test_quadrant_spreader_coil_groups(gpu_pkg, monkeypatch, env, C):
    """The 3D quadrant spreader with 8 coils per pass or 3 CTAs per SM, on
    coil counts that leave a partial last pass."""
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    rng = np.random.default_rng(C)
    shape, M = (24, 20, 16), 5000
    k = np.concatenate([rng.uniform(-0.5, 0.5, (M // 2, 3)),
                        np.clip(rng.normal(0, 0.06, (M // 2, 3)), -0.5, 0.4999)]).astype(np.float32)
    y = (rng.standard_normal((1, C, M)) + 1j * rng.standard_normal((1, C, M))).astype(np.complex64)
    op = gpu_pkg.MRIGB300(k, shape, n_coils=C, squeeze_dims=False)
    ref = NDFTOperator(k.astype(np.float64), shape, n_coils=C)
    assert rel_l2(op.adj_op(y), ref.adj(y)) < TOL
