"""The backend through mri-nufft's own operator machinery on the GPU.

Runs only where the mri-nufft sources are importable: ``MRINUFFT_SRC`` names
a directory holding the ``mrinufft`` package (there is no default).  Each
check runs in a child process whose ``MRIGB300`` derives from mri-nufft's
``FourierOperatorBase``:

* ``get_operator("gb300")(..., density=True, smaps=...)`` builds, and its
  ``op`` / ``adj_op`` match the FP64 NDFT golden cases;
* mri-nufft's own ``pinv_solver(optim="cg")`` (``base.py:667-690`` ->
  ``extras/optim.py:801-902``) and ``make_autograd``
  (``operators/autodiff.py:157-456``) run through ``MRIGB300`` and agree with
  the stand-alone paths within 1e-5;
* ``get_density("pipe")`` (``density/nufft_based.py:6-28``) dispatches to the
  backend's ``pipe``.
"""

import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent

CHILD = r'''
import sys
sys.path.insert(0, {root!r})
import numpy as np, torch
import __graft_entry__ as g
pkg = g.import_package()
import mrinufft
from mrinufft import get_operator
from mrinufft.operators.base import FourierOperatorBase
from mrinufft.density import get_density
assert pkg.HAVE_MRINUFFT and issubclass(pkg.MRIGB300, FourierOperatorBase)
gold = np.load({golden!r})

def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm(a.reshape(b.shape) - b) / np.linalg.norm(b))

# op / adj against the FP64 NDFT golden (the SENSE + batch case of the fixtures)
s = gold["sense__samples"].astype(np.float32)
shape = tuple(int(v) for v in gold["sense__shape"])
smaps = gold["sense__smaps"].astype(np.complex64)
img = gold["sense__img"].astype(np.complex64)
B = img.shape[0]
op = get_operator("gb300")(s, shape, n_coils=smaps.shape[0], n_batchs=B, smaps=smaps,
                           squeeze_dims=False)
assert type(op).__name__ == "MRIGB300"
assert rel(op.op(img), gold["sense__op"]) < 1e-4
assert rel(op.adj_op(gold["sense__ksp"].astype(np.complex64)), gold["sense__adj"]) < 1e-4
op = get_operator("gb300")(s, shape, n_coils=smaps.shape[0], smaps=smaps, squeeze_dims=False)
x = img[0]

# density=True through mri-nufft's constructor -> backend pipe
opd = get_operator("gb300")(s, shape, n_coils=smaps.shape[0], smaps=smaps, density=True)
w = pkg.MRIGB300.pipe(s, shape)
assert rel(opd.density.cpu().numpy(), w) < 1e-5
wd = get_density("pipe")(s, shape, backend="gb300")
assert rel(wd, w) < 1e-5

# mri-nufft's own CG against the stand-alone device CG
yk = op.op(x)
np.random.seed(3)
x_ref = op.pinv_solver(yk, optim="cg", max_iter=5)
from mrinufft.extras.optim import cg as ref_cg
np.random.seed(3)
x_mr = ref_cg(op, yk, max_iter=5, progressbar=False)
assert rel(x_mr, x_ref) < 1e-5, rel(x_mr, x_ref)

# make_autograd through mri-nufft's MRINufftAutoGrad
ad = op.make_autograd(wrt_data=True)
xt = torch.from_numpy(x).cuda().reshape(1, 1, *shape).requires_grad_(True)
loss = torch.sum(torch.abs(ad.op(xt)) ** 2)
loss.backward()
g_ref = 2 * op.adj_op(op.op(x))
assert rel(xt.grad.cpu().numpy(), g_ref) < 1e-5
print("dropin ok")
'''


def test_dropin_through_mrinufft(gpu_pkg):
    src = os.environ.get("MRINUFFT_SRC")
    if not src or not (Path(src) / "mrinufft").is_dir():
        pytest.skip("MRINUFFT_SRC (a directory holding the mrinufft package) is not set")
    code = CHILD.format(root=str(ROOT), golden=str(ROOT / "tests" / "golden" / "ndft_golden.npz"))
    env = dict(os.environ, PYTHONPATH=src, PYTHONDONTWRITEBYTECODE="1")
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-4000:])
    assert "dropin ok" in r.stdout
