"""Host-side logic and the C ABI, without a GPU.

* every entry point declared in ``include/gbnufft.h`` is exported by
  ``libgbnufft.so`` and bound in ``_lib.SIGNATURES``;
* the library loads and reports errors (not crashes) when no device exists;
* host parameter rules (kernel width / beta, fine grid sizes);
* ``proper_trajectory`` against the reference's golden outputs;
* the backend registry.
"""

import ctypes
import os
import re
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import __graft_entry__

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "gbnufft.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(gbn_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def lib(pkg):
    b = __graft_entry__._load_build_module()
    b.build()
    return pkg.load_library()


def test_header_matches_bindings(pkg):
    from mrinufft_gb300 import _lib

    decl = declared_symbols()
    assert len(decl) >= 15
    assert set(decl) == set(_lib.SIGNATURES), set(decl) ^ set(_lib.SIGNATURES)


def test_library_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert lib.gbn_version() == 100


def test_library_reports_errors_without_device(lib, pkg):
    import torch

    if torch.cuda.is_available():
        pytest.skip("error path of a machine without CUDA devices")
    h = ctypes.c_void_p()
    dims = (ctypes.c_int64 * 2)(16, 16)
    st = lib.gbn_plan_create(2, dims, 2.0, 1e-6, 1, 0, 0, ctypes.byref(h))
    assert st != 0
    assert h.value is None
    assert len(lib.gbn_last_error()) > 0
    # argument errors are reported before touching the device
    st = lib.gbn_plan_create(4, dims, 2.0, 1e-6, 1, 0, 0, ctypes.byref(h))
    assert st == 1
    assert b"dim" in lib.gbn_last_error()
    assert lib.gbn_plan_destroy(None) == 0


def test_kernel_params(pkg):
    from mrinufft_gb300.params import fine_shape, kernel_params, next_smooth_even

    assert kernel_params(1e-6) == (7, pytest.approx(2.30 * 7))
    assert kernel_params(1e-3)[0] == 4
    assert kernel_params(1e-3)[1] == pytest.approx(2.38 * 4)
    assert kernel_params(1e-2)[0] == 3
    w, beta = kernel_params(1e-6, 1.5)
    assert w == 8  # ceil(ln(1e6) / (pi sqrt(1/3))) = ceil(7.62)
    assert beta == pytest.approx(0.97 * np.pi * 8 * (1 - 1 / 3))
    assert next_smooth_even(257) == 270
    assert next_smooth_even(512) == 512
    assert fine_shape((256, 256)) == (512, 512)
    assert fine_shape((128, 128, 128)) == (256, 256, 256)
    assert fine_shape((192, 320)) == (384, 640)
    assert fine_shape((4, 4)) == (16, 16)  # >= 2w = 14, 2-3-5 smooth
    assert fine_shape((33, 33), spread_only=True) == (33, 33)


def test_proper_trajectory_matches_reference(pkg, golden):
    from mrinufft_gb300 import proper_trajectory

    np.testing.assert_allclose(proper_trajectory(golden["proper__unit_in"], "pi"),
                               golden["proper__unit_to_pi"])
    np.testing.assert_allclose(proper_trajectory(golden["proper__unit_to_pi"], "unit"),
                               golden["proper__pi_to_unit"])
    np.testing.assert_allclose(proper_trajectory(golden["proper__wrap_in"], "unit"),
                               golden["proper__wrap_unit"])
    import torch

    t = proper_trajectory(torch.from_numpy(golden["proper__unit_in"]), "pi")
    np.testing.assert_allclose(t.numpy(), golden["proper__unit_to_pi"])


def test_registry_and_unknown_backend(pkg):
    from mrinufft_gb300 import MRIGB300, get_operator

    if pkg.HAVE_MRINUFFT:
        from mrinufft.operators.base import FourierOperatorBase
    else:
        from mrinufft_gb300._base import FourierOperatorBase
    avail, cls = FourierOperatorBase.interfaces["gb300"]
    assert cls is MRIGB300
    with pytest.raises(ValueError):
        get_operator("no-such-backend")
    import torch

    if not torch.cuda.is_available():
        assert avail is False
        with pytest.raises(ValueError):
            get_operator("gb300")


def test_registers_in_mrinufft_when_installed(tmp_path):
    if not os.environ.get("MRINUFFT_SRC"):
        pytest.skip("MRINUFFT_SRC (a directory holding the mrinufft package) is not set")
    ref_src = Path(os.environ["MRINUFFT_SRC"])
    if not (ref_src / "mrinufft").is_dir():
        pytest.skip("MRINUFFT_SRC does not hold the mrinufft package")
    code = (
        "import sys; sys.path.insert(0, %r); import __graft_entry__ as g; g.import_package();"
        "import mrinufft; from mrinufft.operators.base import FourierOperatorBase as F;"
        "import mrinufft_gb300 as m; assert m.HAVE_MRINUFFT;"
        "assert F.interfaces['gb300'][1] is m.MRIGB300; print('ok')" % str(ROOT)
    )
    env = dict(os.environ, PYTHONPATH=str(ref_src), PYTHONDONTWRITEBYTECODE="1")
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "ok" in r.stdout


def test_traj3d2stacked_matches_reference(pkg):
    # the reference's traj3d2stacked on a stacked2traj3d trajectory
    from pathlib import Path

    from mrinufft_gb300.stacked import traj3d2stacked

    g = np.load(Path(__file__).resolve().parent / "golden" / "stacked_golden.npz")
    t2, zi = traj3d2stacked(g["traj3d__samples3d"], 10)
    np.testing.assert_array_equal(zi, g["traj3d__z_index"])
    np.testing.assert_allclose(t2, g["traj3d__samples2d"])
