"""Trajectory and k-space file formats against files and arrays written by
mri-nufft's own ``mrinufft.io`` (``tests/golden/make_io_golden.py``).

Bar: byte-identical gradient (``.bin`` / ``.txt``) and BART (``.cfl`` /
``.hdr``) files, bit-identical arrays read back (SHA-256 of dtype, shape and
bytes), equal header parameters; the k-space phase shift within 1e-12.
"""

import hashlib
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden" / "io_golden.npz"

CASES = {
    "2D": ((0.23, 0.23), (256, 256), 0.5, 2, 42_576_000.0, 1.1),
    "3D": ((0.23, 0.23, 0.1248), (64, 64, 32), 0, 5, 11_262_000.0, 1.2),
}


def _digest(a):
    a = np.ascontiguousarray(a)
    return f"{a.dtype.str}{a.shape}" + hashlib.sha256(a.tobytes()).hexdigest()


def _file(p):
    return hashlib.sha256(Path(p).read_bytes()).hexdigest()


@pytest.fixture(scope="module")
def g():
    return np.load(GOLD)


@pytest.fixture(scope="module")
def io(pkg):
    from mrinufft_gb300 import io

    return io


@pytest.mark.parametrize("name", ["2D", "3D"])
@pytest.mark.parametrize("version", [4.2, 5.0, 5.1])
def test_write_and_read_trajectory(io, g, tmp_path, name, version):
    fov, size, te, osf, gamma, tag = CASES[name]
    traj = g[f"traj_{name}"]
    key = f"{name}_v{version}"
    base = str(tmp_path / key)
    io.write_trajectory(trajectory=traj, FOV=fov, img_size=size, check_constraints=True,
                        grad_filename=base, TE_pos=te, version=version, min_osf=osf,
                        recon_tag=tag, gamma=gamma, timestamp=1.7e9, keep_txt_file=True)
    assert _file(base + ".bin") == str(g[f"bin_{key}"])
    assert _file(base + ".txt") == str(g[f"txt_{key}"])
    k, params = io.read_trajectory(base + ".bin", gamma=gamma, read_shots=True)
    assert _digest(k) == str(g[f"read_{key}"])
    for p in ("version", "dimension", "num_shots", "num_samples_per_shot", "min_osf", "gamma",
              "recon_tag", "TE_pos", "FOV", "img_size"):
        np.testing.assert_array_equal(np.asarray(params[p]), g[f"param_{key}_{p}"])
    assert params["timestamp"].timestamp() == float(g[f"param_{key}_timestamp"])
    # the reference test's own round-trip bar (test_io.py:90-103)
    assert params["num_samples_per_shot"] == traj.shape[1] - 1
    np.testing.assert_almost_equal(k, traj, decimal=3.5)
    if version == 5.1:
        for opt, kw in {"minosf": dict(dwell_time="min_osf"), "adc": dict(num_adc_samples=300),
                        "preskip": dict(pre_skip=3, dwell_time=0.005),
                        "raw": dict(normalize_factor=None)}.items():
            k, _ = io.read_trajectory(base + ".bin", gamma=gamma, **kw)
            assert _digest(k) == str(g[f"read_{key}_{opt}"]), opt


def test_write_gradients_layouts(io, g, tmp_path):
    grads, init, final = g["wg_grads"], g["wg_init"], g["wg_final"]
    kws = {"v40": dict(version=4.0),
           "v51skip": dict(version=5.1, final_positions=final, start_skip_samples=4,
                           end_skip_samples=3, timestamp=1.6e9),
           "v42": dict(version=4.2, timestamp=1.5e9, TE_pos=0.25, min_osf=3)}
    for key, kw in kws.items():
        base = str(tmp_path / key)
        io.write_gradients(grads, init, base, img_size=(96, 96, 64), FOV=(0.2, 0.2, 0.15), **kw)
        assert _file(base + ".bin") == str(g[f"bin_{key}"]), key
        if key != "v40":
            k, _ = io.read_trajectory(base + ".bin")
            assert _digest(k) == str(g[f"read_{key}"]), key
    # version 4.0 files (no header beyond the sizes) read without normalisation;
    # they hold the same gradients as the 4.2 file
    k40, p40 = io.read_trajectory(str(tmp_path / "v40.bin"), normalize_factor=None)
    k42, _ = io.read_trajectory(str(tmp_path / "v42.bin"), normalize_factor=None)
    assert p40["version"] == 1.0 and k40.shape == k42.shape == (3, 40, 3)
    np.testing.assert_allclose(k40, k42, rtol=1e-6, atol=1e-6 * np.abs(k42).max())
    with pytest.raises(ValueError):
        io.write_gradients(grads, init, str(tmp_path / "v5"), img_size=(96, 96, 64),
                           FOV=(0.2, 0.2, 0.15), version=5.0)


def test_write_trajectory_unsupported_gradients(io, g, tmp_path):
    fov, size, te, osf, gamma, tag = CASES["2D"]
    with pytest.raises(ValueError):
        io.write_trajectory(g["traj_2D"], fov, size, str(tmp_path / "x"), pregrad="prephase",
                            version=5.0)
    with pytest.raises(NotImplementedError):
        io.write_trajectory(g["traj_2D"], fov, size, str(tmp_path / "x"), postgrad="slowdown_to_edge",
                            version=5.1)


@pytest.mark.parametrize("name", ["2D", "3D"])
def test_bart_cfl(io, g, tmp_path, name):
    traj = g[f"traj_{name}"]
    shape = CASES[name][1]
    base = str(tmp_path / f"cfl_{name}")
    io.traj2cfl(traj, shape, base)
    assert _file(base + ".cfl") == str(g[f"cfl_{name}"])
    assert _file(base + ".hdr") == str(g[f"hdr_{name}"])
    assert _digest(io.cfl2traj(base, shape)) == str(g[f"cfl2traj_{name}"])
    assert _digest(io.cfl2traj(base)) == str(g[f"cfl2traj_{name}_noshape"])
    # raw round trip of an arbitrary complex array
    a = (np.arange(24).reshape(2, 3, 4) * (1 + 2j)).astype(np.complex64)
    io.writecfl(a, str(tmp_path / "raw"))
    np.testing.assert_array_equal(io.readcfl(str(tmp_path / "raw")), a)


def test_kspace_helpers(io, g):
    import torch

    loc, data, shifts = g["shift_loc"], g["shift_data"], g["shift_shifts"]
    out = io.add_phase_to_kspace_with_shifts(data, loc, shifts)
    np.testing.assert_allclose(out, g["shift_out"], rtol=1e-12, atol=1e-12)
    t = io.add_phase_to_kspace_with_shifts(torch.from_numpy(data), torch.from_numpy(loc), shifts)
    assert isinstance(t, torch.Tensor)
    np.testing.assert_allclose(t.numpy(), g["shift_out"], rtol=1e-12, atol=1e-12)
    with pytest.raises(ValueError):
        io.add_phase_to_kspace_with_shifts(data, loc, shifts[:2])
    np.testing.assert_array_equal(io.remove_extra_kspace_samples(g["extra_in"], 64), g["extra_out"])
    assert io.remove_extra_kspace_samples(g["extra_in"], 80).shape[-1] == 70
