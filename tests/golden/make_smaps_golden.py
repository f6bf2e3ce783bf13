"""Generate golden low-frequency sensitivity maps from the mri-nufft reference.

Run in a container where the reference sources are present::

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_smaps_golden.py <mri-nufft src>

It imports ``mrinufft`` from the given source tree and runs the reference's
``low_frequency`` (``extras/smaps.py``) with its default LSQR, on a backend
that is the reference's FP64 NDFT ``MRInumpy`` accepting ``squeeze_dims``
(the argument the method passes).  The method imports scikit-image at its
start even when, as here, no mask and no smoothing are requested; when
scikit-image is absent, placeholder modules that raise if called stand in
for those imports.  Stored per case: trajectory, shape, k-space, window
settings and the maps.
"""

from __future__ import annotations

import os
import sys
import types
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
from _refsrc import reference_src  # noqa: E402

HERE = Path(__file__).resolve().parent


def _placeholder_skimage():
    def unused(*a, **k):
        raise RuntimeError("scikit-image placeholder called")

    sk = types.ModuleType("skimage")
    filt = types.ModuleType("skimage.filters")
    morph = types.ModuleType("skimage.morphology")
    filt.gaussian = filt.threshold_otsu = unused
    morph.convex_hull_image = unused
    sk.filters, sk.morphology = filt, morph
    sys.modules.update({"skimage": sk, "skimage.filters": filt, "skimage.morphology": morph})


def main(ref_src):
    os.environ.setdefault("PYTHONDONTWRITEBYTECODE", "1")
    sys.dont_write_bytecode = True
    sys.path.insert(0, ref_src)
    try:
        import skimage  # noqa: F401
    except ImportError:
        _placeholder_skimage()
    from mrinufft.extras.smaps import low_frequency
    from mrinufft.operators.interfaces.nudft_numpy import MRInumpy

    class _NDFT(MRInumpy):
        backend = "ndft-squeeze"
        available = True

        def __init__(self, samples, shape, n_coils=1, squeeze_dims=True, **kwargs):
            super().__init__(samples, shape, n_coils=n_coils)
            self.squeeze_dims = squeeze_dims

    out = {}
    specs = {
        "lowf_ellipse": ((24, 20), 4, 0.2, "ellipse"),
        "lowf_hann": ((20, 20), 3, 0.25, "hann"),
    }
    for name, (shape, C, thr, win) in specs.items():
        rng = np.random.default_rng(len(name) + 5)
        traj = rng.uniform(-0.5, 0.5, (900, 2))
        ksp = rng.standard_normal((C, 900)) + 1j * rng.standard_normal((C, 900))
        maps = low_frequency(traj, shape, ksp, backend="ndft-squeeze", threshold=thr,
                             window_fun=win, max_iter=10)
        out[f"{name}__traj"] = traj
        out[f"{name}__shape"] = np.array(shape)
        out[f"{name}__ksp"] = ksp
        out[f"{name}__threshold"] = np.array(thr)
        out[f"{name}__window"] = np.array(win)
        out[f"{name}__maps"] = np.asarray(maps)
    np.savez_compressed(HERE / "smaps_golden.npz", **out)
    print("wrote", HERE / "smaps_golden.npz", sorted(out))


if __name__ == "__main__":
    main(reference_src())
