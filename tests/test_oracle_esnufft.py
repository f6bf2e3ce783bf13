"""The CPU ES NUFFT restatement (oracle/esnufft.c through oracle/esnufft.py).

It is the oracle of the pipe density and of the served reconstructions'
CG, and the timed CPU baseline, so it is pinned here on the CPU:

* type 2 / type 1 against the exact FP64 NDFT of the oracle (relative l2
  <= 1e-5 at eps = 1e-6) in 2D and 3D, odd and even sizes, clustered and
  uniform samples, samples on the fold boundary (+-pi);
* spread and interp are adjoint (<A x, y> = <x, A^H y> to 1e-12 in FP64);
* one thread and many threads give the same spread (the parallel schedules
  add the same values in another order: 1e-12);
* the float build (the CPU baseline) stays within 1e-5 of the double build.
"""

import numpy as np
import pytest

from conftest import rel_l2
from oracle import esnufft, ndft


def _samples(d, M, seed):
    rng = np.random.default_rng(seed)
    k = np.concatenate([rng.uniform(-0.5, 0.5, (M // 2, d)),
                        np.clip(rng.normal(0, 0.05, (M - M // 2, d)), -0.5, 0.4999)])
    k[:4] = 0.5  # on the fold boundary (+pi, wraps to -pi)
    return k


@pytest.mark.parametrize("shape", [(40, 36), (33, 28), (20, 18, 16), (17, 20, 15)])
def test_type2_type1_against_ndft(shape):
    d = len(shape)
    M = 3000 if d == 2 else 4000
    k = _samples(d, M, seed=sum(shape))
    rng = np.random.default_rng(1)
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    c = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    e = esnufft.EsNufft(k * 2 * np.pi, shape)
    ku = ndft.proper_trajectory_unit(k)
    assert rel_l2(e.type2(x), ndft.ndft_type2(ku, x, shape, grid="finufft")) < 1e-5
    assert rel_l2(e.type1(c), ndft.ndft_type1(ku, c, shape, grid="finufft")) < 1e-5


@pytest.mark.parametrize("d", [2, 3])
def test_spread_interp_adjoint_and_threads(d):
    shape = (48, 40) if d == 2 else (24, 20, 28)
    M = 5000
    k = _samples(d, M, seed=d)
    rng = np.random.default_rng(2)
    e1 = esnufft.EsNufft(k * 2 * np.pi, shape, nthreads=1)
    en = esnufft.EsNufft(k * 2 * np.pi, shape, nthreads=8)
    g = rng.standard_normal(e1.nf) + 1j * rng.standard_normal(e1.nf)
    c = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    lhs = np.vdot(c, en.interp(g))
    rhs = np.vdot(en.spread(c), g)
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    assert rel_l2(en.spread(c), e1.spread(c)) < 1e-12
    assert rel_l2(en.interp(g), e1.interp(g)) < 1e-12


@pytest.mark.parametrize("d", [2, 3])
def test_float_build_close_to_double(d):
    shape = (64, 64) if d == 2 else (24, 24, 24)
    M = 6000
    k = _samples(d, M, seed=10 + d)
    rng = np.random.default_rng(3)
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    c = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    ed = esnufft.EsNufft(k * 2 * np.pi, shape)
    ef = esnufft.EsNufft(k * 2 * np.pi, shape, dtype=np.float32)
    assert rel_l2(ef.type2(x), ed.type2(x)) < 1e-5
    assert rel_l2(ef.type1(c), ed.type1(c)) < 1e-5
