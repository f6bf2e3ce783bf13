"""The CPU oracle against golden vectors produced by the reference itself.

The fixtures in ``tests/golden/ndft_golden.npz`` were generated by
``tests/golden/make_golden.py`` running mri-nufft's own FP64 NDFT backend
(``MRInumpy``) on the reference's test trajectories.
"""

import numpy as np
import pytest

from conftest import rel_l2
from oracle import ndft
from oracle.operator import NDFTOperator

CASES = ["random2D", "random3D", "grid2D", "grid3D", "radial2D"]


@pytest.mark.parametrize("name", CASES)
def test_ndft_matches_reference(golden, name):
    s = golden[f"{name}__samples"]
    shape = tuple(int(v) for v in golden[f"{name}__shape"])
    su = ndft.proper_trajectory_unit(s)
    nf = ndft.norm_factor(shape)
    y = ndft.ndft_type2(su, golden[f"{name}__img"], shape) / nf
    x = ndft.ndft_type1(su, golden[f"{name}__ksp"], shape) / nf
    assert rel_l2(y, golden[f"{name}__op"]) < 1e-12
    assert rel_l2(x, golden[f"{name}__adj"]) < 1e-12


def test_ndft_subsets_match_full(golden):
    s = ndft.proper_trajectory_unit(golden["random3D__samples"])
    shape = tuple(int(v) for v in golden["random3D__shape"])
    img, ksp = golden["random3D__img"], golden["random3D__ksp"]
    rows = np.array([0, 5, 17, 1999])
    full = ndft.ndft_type2(s, img, shape)
    np.testing.assert_allclose(ndft.ndft_type2_rows(s, img, shape, rows), full[rows], rtol=1e-12)
    vox = np.array([0, 7, 4000, 13311])
    full1 = ndft.ndft_type1(s, ksp, shape).reshape(-1)
    np.testing.assert_allclose(ndft.ndft_type1_voxels(s, ksp, shape, vox), full1[vox], rtol=1e-10)


def test_ndft_grid_is_fft(golden):
    # test_ndft.py:58-79 of the reference: NDFT on a Cartesian grid is an FFT
    N = 16
    s = golden["grid2D__samples"]
    img = golden["grid2D__img"]
    y = ndft.ndft_type2(ndft.proper_trajectory_unit(s), img, (N, N)).reshape(N, N)
    ref = np.fft.fftn(np.fft.fftshift(img)).T  # meshgrid "xy" ordering swaps axes
    np.testing.assert_allclose(y, ref, atol=1e-9, rtol=1e-9)


def test_operator_sense_calib_dc(golden):
    s = golden["sense__samples"]
    shape = tuple(int(v) for v in golden["sense__shape"])
    smaps = golden["sense__smaps"]
    B, C = 2, smaps.shape[0]
    op = NDFTOperator(s, shape, n_batchs=B, smaps=smaps)
    assert rel_l2(op.op(golden["sense__img"]), golden["sense__op"]) < 1e-12
    assert rel_l2(op.adj(golden["sense__ksp"]), golden["sense__adj"]) < 1e-12
    assert rel_l2(op.dc(golden["sense__img"], golden["sense__ksp"]), golden["sense__dc"]) < 1e-12
    opc = NDFTOperator(s, shape, n_coils=C, n_batchs=B)
    assert rel_l2(opc.op(golden["calib__img"]), golden["calib__op"]) < 1e-12
    assert rel_l2(opc.adj(golden["sense__ksp"]), golden["calib__adj"]) < 1e-12
    assert rel_l2(opc.dc(golden["calib__img"], golden["sense__ksp"]), golden["calib__dc"]) < 1e-12


def test_proper_trajectory_oracle(golden):
    np.testing.assert_allclose(ndft.proper_trajectory_pi(golden["proper__unit_in"]),
                               golden["proper__unit_to_pi"])
    np.testing.assert_allclose(ndft.proper_trajectory_unit(golden["proper__unit_to_pi"]),
                               golden["proper__pi_to_unit"])
    np.testing.assert_allclose(ndft.proper_trajectory_unit(golden["proper__wrap_in"]),
                               golden["proper__wrap_unit"])


def test_odd_size_grids_differ_by_half_shift():
    # the NDFT grid of the reference is linspace(-N/2, N/2-1, N): for odd N it
    # is shifted by half a cell from the integer modes of finufft
    k = np.array([[0.1, -0.2]])
    x = np.zeros((5, 4), complex)
    x[0, 0] = 1.0
    a = ndft.ndft_type2(k, x, (5, 4), grid="ndft")
    b = ndft.ndft_type2(k, x, (5, 4), grid="finufft")
    # n0 = -2.5 vs -2
    np.testing.assert_allclose(a / b, np.exp(-2j * np.pi * 0.1 * (-0.5)), rtol=1e-12)


TOEP = ["toep2D_w", "toep2D", "toep3D_w"]


@pytest.mark.parametrize("name", TOEP)
def test_toeplitz_oracle_matches_reference(name):
    # tests/golden/toeplitz_golden.npz: the reference's own compute_toeplitz_kernel
    # and apply_toeplitz_kernel on its FP64 NDFT backend
    from pathlib import Path

    from oracle import toeplitz

    g = np.load(Path(__file__).resolve().parent / "golden" / "toeplitz_golden.npz")
    s = g[f"{name}__samples"]
    shape = tuple(int(v) for v in g[f"{name}__shape"])
    w = g[f"{name}__weights"]
    k = toeplitz.toeplitz_kernel(s, shape, w)
    assert rel_l2(k, g[f"{name}__kernel"]) < 1e-12
    x = g[f"{name}__img"]
    assert rel_l2(toeplitz.apply_toeplitz(x, k), g[f"{name}__gram"]) < 1e-12
    ref = NDFTOperator(s, shape, density=w)
    assert rel_l2(ref.adj(ref.op(x)), g[f"{name}__gram"]) < 1e-12


@pytest.mark.parametrize("name", ["stack_sense", "stack_calib"])
def test_stacked_oracle_matches_reference(name):
    # tests/golden/stacked_golden.npz: the reference's MRIStackedNUFFT on its
    # FP64 NDFT backend
    from pathlib import Path

    from oracle import stacked

    g = np.load(Path(__file__).resolve().parent / "golden" / "stacked_golden.npz")
    shape = tuple(int(v) for v in g[f"{name}__shape"])
    kw = dict(smaps=g[f"{name}__smaps"] if f"{name}__smaps" in g else None,
              n_coils=int(g[f"{name}__n_coils"]), n_batchs=int(g[f"{name}__n_batchs"]))
    s, zi = g[f"{name}__samples"], g[f"{name}__z_index"]
    y = stacked.stacked_op(s, shape, zi, g[f"{name}__img"], **kw)
    assert rel_l2(y, g[f"{name}__op"]) < 1e-12
    x = stacked.stacked_adj(s, shape, zi, g[f"{name}__ksp"], **kw)
    assert rel_l2(x, g[f"{name}__adj"]) < 1e-12


ORC = ["orc_tuple", "orc_svd", "orc_mti3d"]


def _orc_golden():
    from pathlib import Path

    return np.load(Path(__file__).resolve().parent / "golden" / "offres_golden.npz")


@pytest.mark.parametrize("name", ORC)
def test_offres_formula_matches_reference(name):
    # y = sum_l B_l * A(C_l x) on the FP64 NDFT with the reference's own
    # interpolators reproduces the reference's MRIFourierCorrected
    g = _orc_golden()
    shape = tuple(int(v) for v in g[f"{name}__shape"])
    smaps = g[f"{name}__smaps"] if f"{name}__smaps" in g else None
    C = int(g[f"{name}__n_coils"])
    B, Cm = g[f"{name}__B"], g[f"{name}__C"]
    NK = B.shape[0]
    ref = NDFTOperator(g[f"{name}__samples"], shape, n_coils=C, smaps=smaps)
    x = g[f"{name}__img"]
    y = sum(ref.op(Cm[l] * x).reshape(1, C, -1, NK) * B[:, l] for l in range(B.shape[1]))
    assert rel_l2(y.reshape(1, C, -1), g[f"{name}__op"]) < 1e-12
    yk = g[f"{name}__ksp"].reshape(1, C, -1, NK)
    a = sum(np.conj(Cm[l]) * ref.adj((yk * np.conj(B[:, l])).reshape(1, C, -1), use_density=False)
            for l in range(B.shape[1]))
    assert rel_l2(a, g[f"{name}__adj"]) < 1e-12


@pytest.mark.parametrize("name,method", [("orc_svd", "svd"), ("orc_mti3d", "mti")])
def test_offres_factorisations_match_reference(pkg, name, method):
    from mrinufft_gb300 import offres

    g = _orc_golden()
    fm = offres.get_complex_fieldmap_rad(g[f"{name}__b0"])
    fn = offres.FACTORISATIONS[method]
    B, Cm, _ = fn(field_map=fm, readout_time=g[f"{name}__t"], mask=None)
    Bg, Cg = g[f"{name}__B"], g[f"{name}__C"]
    assert B.shape == Bg.shape and Cm.shape == Cg.shape
    # the interpolated phase matrix B C is independent of the basis of B
    prod = np.einsum("kl,l...->k...", B, Cm)
    prodg = np.einsum("kl,l...->k...", Bg, Cg)
    assert rel_l2(prod, prodg) < 1e-4


@pytest.mark.parametrize("name", ["cg_sense", "cg_density", "cg_damp", "cg_calib", "cg_3d"])
def test_oracle_cg_and_power_method_match_reference(name):
    """The oracle's power method and CG against the reference's own
    (``tests/golden/cg_golden.npz``, made by ``make_cg_golden.py``)."""
    from pathlib import Path

    from oracle import operator as oop

    g = np.load(Path(__file__).resolve().parent / "golden" / "cg_golden.npz")
    shape = tuple(int(v) for v in g[f"{name}__shape"])
    s = g[f"{name}__samples"]
    smaps = g[f"{name}__smaps"] if f"{name}__smaps" in g else None
    dens = g[f"{name}__density"] if f"{name}__density" in g else None
    C, B = int(g[f"{name}__n_coils"]), int(g[f"{name}__n_batchs"])
    np.random.seed(int(g[f"{name}__seed"]))
    x0 = 1j * np.random.random(shape).astype(np.complex128)
    x0 += np.random.random(shape).astype(np.complex128)
    L, _ = oop.power_method(10, oop.NDFTOperator(s, shape, density=dens).gram, x0.reshape(1, 1, *shape))
    assert abs(L - float(g[f"{name}__lipschitz"])) <= 1e-10 * L
    op = oop.NDFTOperator(s, shape, n_coils=C, n_batchs=B, smaps=smaps, density=dens)
    xp = g[f"{name}__x0"] if f"{name}__x0" in g else None
    x = oop.cg(op, g[f"{name}__ksp"], L, max_iter=10, damp=float(g[f"{name}__damp"]), x0=xp)
    ref = g[f"{name}__x"]
    assert np.linalg.norm(x.reshape(ref.shape) - ref) <= 1e-10 * np.linalg.norm(ref)
