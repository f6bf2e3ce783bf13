"""Seeded synthetic workloads: trajectories, phantoms and coil maps.

The trajectory generators restate mri-nufft's own initialisations
(``src/mrinufft/trajectories/inits/radial.py:12-43`` for 2D radial,
``inits/spiral.py:26-130`` for algebraic spirals, ``KMAX = 0.5`` of
``trajectories/utils.py:18``, and ``initialize_3D_phyllotaxis_radial``,
radial.py:46-94, for the 3D kooshball); ``tests/test_workloads.py`` checks
them against fixtures written by those generators.  Phantoms are sums of
random ellipses / ellipsoids with complex amplitudes plus complex Gaussian
noise; coil maps are complex Gaussians centred on a sphere, normalised so
that sum_c |s_c|^2 = 1 at every voxel.
"""

from __future__ import annotations

import numpy as np

KMAX = 0.5


def _rot2(theta):
    c, s = np.cos(theta), np.sin(theta)
    return np.array([[c, -s], [s, c]])


def radial_2d(Nc: int, Ns: int, in_out: bool = False) -> np.ndarray:
    """(Nc, Ns, 2) radial spokes with uniform tilt 2 pi / Nc (in_out: pi / Nc)."""
    seg = np.linspace(-1 if in_out else 0, 1, Ns)
    traj = np.zeros((Nc, Ns, 2))
    traj[0, :, 0] = KMAX * seg
    rot = _rot2(2 * np.pi / Nc / (1 + in_out)).T
    for i in range(1, Nc):
        traj[i] = traj[i - 1] @ rot
    return traj


def spiral_2d(Nc: int, Ns: int, power: float = 1.0, nb_revolutions: float = 1.0) -> np.ndarray:
    """(Nc, Ns, 2) algebraic spiral r = theta^power (1: Archimedes, 2: Galilean)."""
    ang = 2 * np.pi * nb_revolutions * np.linspace(0, 1, Ns)
    rad = np.abs(ang) ** power
    shot = np.sign(ang) * rad * np.exp(1j * np.abs(ang))
    traj = np.zeros((Nc, Ns, 2))
    traj[0] = np.stack([shot.real, shot.imag], axis=-1)
    rot = _rot2(2 * np.pi / Nc).T
    for i in range(1, Nc):
        traj[i] = traj[i - 1] @ rot
    return KMAX * traj / np.max(np.linalg.norm(traj, axis=-1))


def kooshball_3d(Nc: int, Ns: int) -> np.ndarray:
    """(Nc, Ns, 3) centre-out phyllotaxis spokes (radial.py:46-94).

    The reference builds them as zero-width 3D cones (inits/cones.py:57-143):
    a straight centre-out line whose sample radii are those of a normalised
    Archimedes spiral, KMAX * linspace(0, 1, Ns), laid along -z and rotated
    onto the Fibonacci directions v_i = (cos(phi_i) r_i, sin(phi_i) r_i, z_i)
    with z_i = linspace(-1, 1, Nc), phi_i = i pi (3 - sqrt(5)), r_i =
    sqrt(1 - z_i^2) (tools/transforms.py:113-189).  Spoke i is therefore
    -v_i times the radii."""
    z = np.linspace(-1, 1, Nc)
    phi = np.pi * (3 - np.sqrt(5)) * np.arange(Nc)
    r = np.sqrt(1 - z * z)
    v = np.stack([np.cos(phi) * r, np.sin(phi) * r, z], axis=-1)  # (Nc, 3)
    seg = KMAX * np.linspace(0, 1, Ns)
    return -v[:, None, :] * seg[None, :, None]


def stack_of_radial_3d(Nc: int, Ns: int, Nr: int) -> np.ndarray:
    """2D radial disc rotated Nr times about axis 0 (a 3D radial coverage)."""
    disc = radial_2d(Nc, Ns)
    out = np.zeros((Nr, Nc, Ns, 3))
    for r in range(Nr):
        a = np.pi * r / Nr
        out[r, :, :, 0] = disc[..., 0]
        out[r, :, :, 1] = disc[..., 1] * np.cos(a)
        out[r, :, :, 2] = disc[..., 1] * np.sin(a)
    return out.reshape(Nr * Nc, Ns, 3)


def phantom(shape, n_shapes: int = 20, noise: float = 0.01, seed: int = 0) -> np.ndarray:
    """complex64 sum of random ellipses / ellipsoids plus N(0, noise^2) complex noise."""
    rng = np.random.default_rng(seed)
    d = len(shape)
    grids = np.meshgrid(*[np.linspace(-1, 1, n) for n in shape], indexing="ij")
    pts = np.stack(grids, axis=-1)
    img = np.zeros(shape, dtype=np.complex128)
    for _ in range(n_shapes):
        c = rng.uniform(-0.6, 0.6, d)
        ax = rng.uniform(0.05, 0.5, d)
        if d == 2:
            t = rng.uniform(0, np.pi)
            R = _rot2(t)
        else:
            q = rng.standard_normal((3, 3))
            R, _ = np.linalg.qr(q)
        loc = (pts - c) @ R
        inside = np.sum((loc / ax) ** 2, axis=-1) <= 1
        amp = rng.uniform(0.1, 1.0) * np.exp(1j * rng.uniform(0, 2 * np.pi))
        img[inside] += amp
    img += noise * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    return img.astype(np.complex64)


def coil_maps(shape, n_coils: int, seed: int = 0, radius: float = 0.4) -> np.ndarray:
    """complex64 (C, *shape) Gaussian maps centred on a sphere, sum |s|^2 = 1."""
    rng = np.random.default_rng(seed + 1000)
    d = len(shape)
    grids = np.meshgrid(*[np.linspace(-0.5, 0.5, n) for n in shape], indexing="ij")
    pts = np.stack(grids, axis=-1)
    maps = np.empty((n_coils, *shape), dtype=np.complex128)
    for c in range(n_coils):
        if d == 2:
            a = 2 * np.pi * c / n_coils
            ctr = radius * np.array([np.cos(a), np.sin(a)])
        else:
            z = 1 - 2 * (c + 0.5) / n_coils
            r = np.sqrt(1 - z * z)
            a = np.pi * (3 - np.sqrt(5)) * c
            ctr = radius * np.array([r * np.cos(a), r * np.sin(a), z])
        dist2 = np.sum((pts - ctr) ** 2, axis=-1)
        mag = np.exp(-dist2 / (2 * 0.3 ** 2))
        ph = np.exp(1j * (rng.uniform(0, 2 * np.pi) + 2 * np.pi * (pts @ rng.uniform(-0.5, 0.5, d))))
        maps[c] = mag * ph
    maps /= np.sqrt(np.sum(np.abs(maps) ** 2, axis=0, keepdims=True))
    return maps.astype(np.complex64)


def config1():
    """2D 256^2 single coil, radial 100 x 500 (50 000 samples)."""
    traj = radial_2d(100, 500).reshape(-1, 2).astype(np.float32)
    return traj, (256, 256), phantom((256, 256), seed=0)


def config2(n_spokes: int = 4096, n_samples: int = 512, n_coils: int = 16, N: int = 128):
    """3D 128^3, 16 coils, kooshball 4096 x 512 (2 097 152 samples)."""
    shape = (N, N, N)
    traj = kooshball_3d(n_spokes, n_samples).reshape(-1, 3).astype(np.float32)
    return traj, shape, phantom(shape, seed=0), coil_maps(shape, n_coils, seed=0)


def config3(n_instances: int = 32, seed: int = 0):
    """Uneven 2D instances: grids from {128, 192, 256, 320, 384}^2, even
    instances variable-density (Galilean) spirals with Nc in [16, 64] and Ns in
    [1024, 4096], odd instances radial with Nc in [64, 256] and Ns in
    [256, 1024], coil counts from {1, 4, 8, 16, 32}; seeded phantoms and maps."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_instances):
        N = int(rng.choice([128, 192, 256, 320, 384]))
        C = int(rng.choice([1, 4, 8, 16, 32]))
        if i % 2 == 0:
            traj = spiral_2d(int(rng.integers(16, 65)), int(rng.integers(1024, 4097)), power=2)
        else:
            traj = radial_2d(int(rng.integers(64, 257)), int(rng.integers(256, 1025)))
        shape = (N, N)
        out.append({
            "samples": traj.reshape(-1, 2).astype(np.float32),
            "shape": shape,
            "smaps": coil_maps(shape, C, seed=seed + i),
            "image": phantom(shape, seed=seed + i),
        })
    return out


# Request templates of the served mix: key, share of the stream, trajectory,
# image shape, coils (70 % 2D 256^2 radial 256 x 512 with 8-32 coils, 20 %
# 2D 384^2 Galilean spiral 32 x 4096 with 16 coils, 10 % 3D 128^3 kooshball
# 2048 x 512 with 8 coils).
SERVE_MIX = [
    ("a8", 0.175, "radial", (256, 256), 8),
    ("a16", 0.175, "radial", (256, 256), 16),
    ("a24", 0.175, "radial", (256, 256), 24),
    ("a32", 0.175, "radial", (256, 256), 32),
    ("b16", 0.2, "spiral", (384, 384), 16),
    ("c8", 0.1, "koosh", (128, 128, 128), 8),
]


def serve_template(index: int):
    """Trajectory (float32, unit), coil maps and phantom of template ``index``
    of ``SERVE_MIX`` (seeded by the index)."""
    key, _, kind, shape, C = SERVE_MIX[index]
    if kind == "radial":
        traj = radial_2d(256, 512).reshape(-1, 2)
    elif kind == "spiral":
        traj = spiral_2d(32, 4096, power=2).reshape(-1, 2)
    else:
        traj = kooshball_3d(2048, 512).reshape(-1, 3)
    return traj.astype(np.float32), coil_maps(shape, C, seed=index), phantom(shape, seed=index)
