"""Generate ``traj_golden.npz`` from mri-nufft's own trajectory generators
(run where the reference sources are importable; not used at test time).

The benchmark configurations draw their trajectories from these generators:

* 2D radial ``initialize_2D_radial(Nc, Ns)`` (``trajectories/inits/radial.py:12-43``):
  100 x 500 (the 2D single-coil case), 256 x 512 (the served 2D radial
  template) and the radial sizes of the uneven batched instances;
* 3D kooshball ``initialize_3D_phyllotaxis_radial(Nc, Ns)`` (radial.py:46-94):
  4096 x 512 (the 3D multi-coil case), 2048 x 512 (the served 3D template)
  and small cases;
* Galilean spirals ``initialize_2D_spiral(Nc, Ns, spiral="galilean")``
  (``inits/spiral.py:26-130``): 64 x 2048 (the differentiable case),
  32 x 4096 (the served spiral template) and small cases.

Small trajectories are stored whole (float64); large ones as their first
shot and a seeded subset of 2048 samples (indices and float64 values), plus,
in 3D, every spoke's last sample in float32.

    python tests/golden/make_traj_golden.py <mri-nufft src>
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
from _refsrc import reference_src  # noqa: E402

OUT = Path(__file__).resolve().parent / "traj_golden.npz"


def main(ref_src):
    sys.path.insert(0, ref_src)
    from mrinufft.trajectories import (initialize_2D_radial, initialize_2D_spiral,
                                       initialize_3D_phyllotaxis_radial)

    out = {}
    rng = np.random.default_rng(0)

    def store(name, traj):
        traj = np.asarray(traj, dtype=np.float64)
        out[f"{name}__shape"] = np.array(traj.shape)
        flat = traj.reshape(-1, traj.shape[-1])
        if flat.shape[0] <= 20000:
            out[f"{name}__full"] = flat
            return
        idx = np.sort(rng.choice(flat.shape[0], 2048, replace=False)).astype(np.int32)
        out[f"{name}__idx"] = idx
        out[f"{name}__sub"] = flat[idx]
        out[f"{name}__first"] = traj[0]
        if traj.shape[-1] == 3:  # spoke directions
            out[f"{name}__ends"] = traj[:, -1, :].astype(np.float32)

    for Nc, Ns in [(100, 500), (256, 512), (64, 256), (200, 1000), (7, 33)]:
        store(f"radial2d_{Nc}_{Ns}", initialize_2D_radial(Nc, Ns))
    for Nc, Ns in [(4096, 512), (2048, 512), (256, 32), (64, 16), (5, 9)]:
        store(f"koosh3d_{Nc}_{Ns}", initialize_3D_phyllotaxis_radial(Nc, Ns))
    for Nc, Ns in [(64, 2048), (32, 4096), (16, 1024), (48, 4096), (3, 17)]:
        store(f"spiral2d_{Nc}_{Ns}", initialize_2D_spiral(Nc, Ns, spiral="galilean"))
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(out)} arrays)")


if __name__ == "__main__":
    main(reference_src())
