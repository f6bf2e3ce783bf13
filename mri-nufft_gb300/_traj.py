"""Trajectory normalisation, restating ``src/mrinufft/_utils.py:58-100``.

``proper_trajectory`` flattens ``(..., d)`` sample arrays to ``(M, d)`` and
rescales them: with ``normalize="pi"`` samples whose max |k| is below
0.5 + 1e-4 are taken to be in [-0.5, 0.5) and multiplied by 2 pi; with
``normalize="unit"`` samples above that bound are divided by 2 pi, and
samples at or beyond 0.5 are wrapped into [-0.5, 0.5).  Works on numpy
arrays and torch tensors (either device).
"""

from __future__ import annotations

import logging
import math

import numpy as np
import torch

logger = logging.getLogger("mrinufft_gb300")


def proper_trajectory(trajectory, normalize="pi"):
    is_torch = isinstance(trajectory, torch.Tensor)
    if not is_torch and not isinstance(trajectory, np.ndarray):
        if hasattr(trajectory, "__cuda_array_interface__") or hasattr(trajectory, "__dlpack__"):
            trajectory = torch.as_tensor(trajectory)
            is_torch = True
        else:
            trajectory = np.asarray(trajectory)
    new_traj = trajectory.reshape(-1, trajectory.shape[-1])
    if new_traj.shape[0] == 0:
        return new_traj
    if is_torch:
        max_abs = float(new_traj.abs().max())
    else:
        max_abs = float(np.max(np.abs(new_traj)))
    if normalize == "pi" and max_abs - 1e-4 < 0.5:
        logger.warning("Samples will be rescaled to [-pi, pi), assuming they were in [-0.5, 0.5)")
        new_traj = new_traj * 2 * math.pi
    elif normalize == "unit" and max_abs - 1e-4 > 0.5:
        logger.warning("Samples will be rescaled to [-0.5, 0.5), assuming they were in [-pi, pi)")
        new_traj = new_traj * (1 / (2 * math.pi))
    if normalize == "unit" and max_abs >= 0.5:
        new_traj = (new_traj + 0.5) % 1 - 0.5
    return new_traj
