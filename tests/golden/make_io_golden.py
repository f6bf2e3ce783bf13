"""Generate ``io_golden.npz`` from mri-nufft's own ``mrinufft.io`` (run in a
container where the reference sources are importable; not used at test
time).

Cases follow the reference's ``tests/test_io.py`` (``test_write_n_read``
without prephasing / spoiling gradients, ``test_add_shift``) at smaller
sizes, plus direct ``write_gradients`` calls for the version 4.0 layout and
the version 5.1 skip counters, and ``read_trajectory`` options (dwell time
from ``min_osf``, explicit ADC sample counts, ``pre_skip``, no
normalisation).  The reference's reader raises on version 4.0 files (it
sets its skip counters only for versions above 4.0), so that case keeps
only the writer's digest.  Files and arrays are stored as SHA-256 digests
of their bytes (with dtype and shape), inputs and small outputs as arrays.

    python tests/golden/make_io_golden.py /path/to/mri-nufft/src
"""

import hashlib
import sys
import tempfile
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
from _refsrc import reference_src  # noqa: E402


def digest(a):
    a = np.ascontiguousarray(a)
    return f"{a.dtype.str}{a.shape}" + hashlib.sha256(a.tobytes()).hexdigest()


def file_digest(p):
    return hashlib.sha256(Path(p).read_bytes()).hexdigest()


def main(src):
    sys.path.insert(0, src)
    from mrinufft.io import (add_phase_to_kspace_with_shifts, cfl2traj, read_trajectory,
                             remove_extra_kspace_samples, traj2cfl, write_gradients,
                             write_trajectory)
    from mrinufft.trajectories import initialize_2D_radial, initialize_3D_cones
    from mrinufft.trajectories.utils import Gammas

    out = {}
    tmp = Path(tempfile.mkdtemp())
    cases = {
        "2D": (initialize_2D_radial(Nc=16, Ns=256, tilt="uniform", in_out=False).astype(np.float32),
               (0.23, 0.23), (256, 256), 0.5, 2, float(Gammas.H), 1.1),
        "3D": (initialize_3D_cones(Nc=16, Ns=256, tilt="uniform", in_out=True).astype(np.float32),
               (0.23, 0.23, 0.1248), (64, 64, 32), 0, 5, float(Gammas.Na), 1.2),
    }
    for name, (traj, fov, size, te, osf, gamma, tag) in cases.items():
        out[f"traj_{name}"] = traj
        for version in (4.2, 5.0, 5.1):
            key = f"{name}_v{version}"
            base = str(tmp / key)
            write_trajectory(trajectory=traj, FOV=fov, img_size=size, check_constraints=True,
                             grad_filename=base, TE_pos=te, version=version, min_osf=osf,
                             recon_tag=tag, gamma=gamma, timestamp=1.7e9, keep_txt_file=True)
            out[f"bin_{key}"] = file_digest(base + ".bin")
            out[f"txt_{key}"] = file_digest(base + ".txt")
            k, params = read_trajectory(base + ".bin", gamma=gamma, read_shots=True)
            out[f"read_{key}"] = digest(k)
            for p in ("version", "dimension", "num_shots", "num_samples_per_shot", "min_osf",
                      "gamma", "recon_tag", "TE_pos"):
                out[f"param_{key}_{p}"] = np.asarray(params[p])
            out[f"param_{key}_FOV"] = np.asarray(params["FOV"])
            out[f"param_{key}_img_size"] = np.asarray(params["img_size"])
            out[f"param_{key}_timestamp"] = np.asarray(params["timestamp"].timestamp())
            if version == 5.1:
                for opt, kw in {"minosf": dict(dwell_time="min_osf"),
                                "adc": dict(num_adc_samples=300),
                                "preskip": dict(pre_skip=3, dwell_time=0.005),
                                "raw": dict(normalize_factor=None)}.items():
                    k, params = read_trajectory(base + ".bin", gamma=gamma, **kw)
                    out[f"read_{key}_{opt}"] = digest(k)

    # direct gradient files: version 4.0 layout; version 5.1 with skipped samples
    rng = np.random.default_rng(0)
    grads = (0.01 * rng.standard_normal((3, 40, 3))).astype(np.float32)
    init = (50 * rng.standard_normal((3, 3))).astype(np.float32)
    final = (50 * rng.standard_normal((3, 3))).astype(np.float32)
    out["wg_grads"], out["wg_init"], out["wg_final"] = grads, init, final
    for key, kw in {"v40": dict(version=4.0),
                    "v51skip": dict(version=5.1, final_positions=final, start_skip_samples=4,
                                    end_skip_samples=3, timestamp=1.6e9),
                    "v42": dict(version=4.2, timestamp=1.5e9, TE_pos=0.25, min_osf=3)}.items():
        base = str(tmp / key)
        write_gradients(grads, init, base, img_size=(96, 96, 64), FOV=(0.2, 0.2, 0.15), **kw)
        out[f"bin_{key}"] = file_digest(base + ".bin")
        if key == "v40":
            continue  # the reference's reader fails on version 4.0 files (unbound skip counts)
        k, _ = read_trajectory(base + ".bin")
        out[f"read_{key}"] = digest(k)

    # BART trajectory files
    for name in ("2D", "3D"):
        traj = out[f"traj_{name}"]
        shape = cases[name][2]
        base = str(tmp / f"cfl_{name}")
        traj2cfl(traj, shape, base)
        out[f"cfl_{name}"] = file_digest(base + ".cfl")
        out[f"hdr_{name}"] = file_digest(base + ".hdr")
        out[f"cfl2traj_{name}"] = digest(cfl2traj(base, shape))
        out[f"cfl2traj_{name}_noshape"] = digest(cfl2traj(base))

    # k-space helpers
    loc = rng.uniform(-0.5, 0.5, (500, 3))
    data = rng.standard_normal(500) + 1j * rng.standard_normal(500)
    shifts = rng.uniform(size=3)
    out["shift_loc"], out["shift_data"], out["shift_shifts"] = loc, data, shifts
    out["shift_out"] = add_phase_to_kspace_with_shifts(data, loc, shifts)
    ks = rng.standard_normal((2, 3, 70)).astype(np.complex64)
    out["extra_in"], out["extra_out"] = ks, remove_extra_kspace_samples(ks, 64)

    dst = Path(__file__).resolve().parent / "io_golden.npz"
    np.savez_compressed(dst, **{k: np.asarray(v) for k, v in out.items()})
    print("wrote", dst, len(out), "entries")


if __name__ == "__main__":
    main(reference_src())
