"""On-disk trajectory and k-space formats that feed the operators.

Restates mri-nufft's ``src/mrinufft/io`` readers and writers for the host:

* the NeuroSpin gradient file (``nsp.py:38-575``): ``write_gradients``,
  ``write_trajectory`` (trajectory -> gradients by finite differences,
  ``trajectories/utils.py:441-474``, hardware check 618-660) and
  ``read_trajectory`` (gradients -> k-space locations at the ADC dwell time);
* BART's ``.cfl`` / ``.hdr`` pair (``cfl.py:19-146``): ``traj2cfl``,
  ``cfl2traj`` and the raw ``readcfl`` / ``writecfl``;
* k-space helpers (``utils.py:7-67``): ``add_phase_to_kspace_with_shifts``
  and ``remove_extra_kspace_samples``, on numpy arrays or torch tensors
  (computed on the tensor's device).

The gradient file is a flat float32 array: a header, the initial (and, from
version 5, final) k-space position of every shot, the maximum gradient in
mT/m and every gradient sample divided by it.  Header values and samples
take the values of their decimal text form (``str`` for header scalars,
4 decimals for positions, 6 for gradients) before the float32 cast, so files
written here are byte-identical to the reference's.  Reading integrates the
gradients on the gradient raster and samples the result at the ADC dwell
time, with the reference's float32 / float64 arithmetic.

Siemens twix (``siemens.py``, ``read_arbgrad_rawdat``) and Pulseq readers
need pymapVBVD / pypulseq and are not restated.
"""

from __future__ import annotations

import logging
from datetime import datetime
from pathlib import Path

import numpy as np

logger = logging.getLogger(__name__)

KMAX = 0.5
DEFAULT_RASTER_TIME = 10e-3  # ms
DEFAULT_GMAX = 0.04  # T/m
DEFAULT_SMAX = 0.1  # T/m/ms
GAMMA_HYDROGEN = 42_576_000.0  # Hz/T


# --------------------------------------------------------------------------
# NeuroSpin gradient files
# --------------------------------------------------------------------------
def _rows(values, fmt):
    return "\n".join(" ".join(format(v, fmt) for v in row) for row in values) + "\n"


def _gradient_text(gradients, initial_positions, img_size, FOV, TE_pos, min_osf, gamma, version,
                   recon_tag, timestamp, final_positions, start_skip_samples, end_skip_samples):
    """Text image of a gradient file; one value per token (nsp.py:96-178).
    Header scalars use ``str`` (for numpy float32 it differs from ``format``)."""
    num_shots, num_samples = gradients.shape[0], gradients.shape[1]
    dimension = initial_positions.shape[-1]
    if gradients.ndim == 3:
        gradients = gradients.reshape(-1, gradients.shape[-1])
    gradients = gradients * 1e3  # mT/m
    max_grad = np.max(np.abs(gradients))
    out = []
    if version >= 4.1:
        out.append(str(version) + "\n")
    out.append(str(dimension) + "\n")
    if version >= 4.1:
        if isinstance(img_size, int):
            img_size = (img_size,) * dimension
        if isinstance(FOV, float):
            FOV = (FOV,) * dimension
        out += [str(v) + "\n" for v in FOV]
        out += [str(v) + "\n" for v in img_size]
        out.append(str(min_osf) + "\n")
        out.append(str(gamma * 1000) + "\n")
    out.append(str(num_shots) + "\n" + str(num_samples) + "\n")
    if version >= 4.1:
        if TE_pos == 0 and np.sum(initial_positions) != 0:
            logger.warning("The initial positions are not all zero for center-out trajectory")
        out.append("".join(str(v) + "\n" for v in (TE_pos, max_grad, recon_tag)))
        spare = 10
        if version >= 4.2:
            if timestamp is None:
                timestamp = float(datetime.now().timestamp())
            out.append(str(timestamp) + "\n")
            spare -= 1
        if version >= 5.1:
            out.append(str(start_skip_samples) + "\n" + str(end_skip_samples) + "\n")
            spare -= 2
        out.append("0\n" * spare)
    out.append(_rows(initial_positions, "5.4f"))
    if version >= 5:
        if final_positions is None:
            raise ValueError("final_positions are required for gradient files of version >= 5")
        out.append(_rows(final_positions, "5.4f"))
    if version < 4.1:
        out.append(str(max_grad) + "\n")
    out.append(_rows(gradients / max_grad, "5.6f"))
    return "".join(out)


def write_gradients(gradients, initial_positions, grad_filename, img_size, FOV, TE_pos=0.5,
                    min_osf=5, gamma=GAMMA_HYDROGEN, version=4.2, recon_tag=1.1, timestamp=None,
                    keep_txt_file=False, final_positions=None, start_skip_samples=0,
                    end_skip_samples=0):
    """Write ``grad_filename + ".bin"`` from gradients (shots, samples, d) in
    T/m and initial positions (shots, d) (nsp.py:38-189).  With
    ``keep_txt_file`` the text image is kept beside it as ``.txt``."""
    text = _gradient_text(np.asarray(gradients), np.asarray(initial_positions), img_size, FOV,
                          TE_pos, min_osf, gamma, version, recon_tag, timestamp,
                          None if final_positions is None else np.asarray(final_positions),
                          start_skip_samples, end_skip_samples)
    if keep_txt_file:
        Path(grad_filename + ".txt").write_text(text)
    values = np.array([float(tok) for line in text.splitlines() for tok in line.split(" ")],
                      dtype=np.float32)
    values.tofile(grad_filename + ".bin")


def _check_constraints(gradients, raster_time, gmax, smax, pregrad):
    """Amplitude / slew-rate warnings of write_trajectory (nsp.py:336-360)."""
    slew = np.diff(gradients, axis=1) / raster_time
    max_g = np.max(np.linalg.norm(gradients, axis=-1))
    max_s = np.max(np.linalg.norm(slew, axis=-1))
    if not (max_g < gmax and max_s < smax):
        logger.warning("Hard constraints violated! "
                       f"Maximum gradient amplitude: {max_g:.3f} > {gmax:.3f}"
                       f"Maximum slew rate: {max_s:.3f} > {smax:.3f}")
    if pregrad != "prephase":
        border = gradients[:, 0] / raster_time
        if np.any(np.abs(border) > smax):
            logger.warning("Slew rate at start of trajectory exceeds maximum slew rate!"
                           f"Maximum slew rate: {np.max(np.abs(border)):.3f}"
                           f" > {smax:.3f}. Please use prephase gradient to avoid this "
                           " issue.")


def write_trajectory(trajectory, FOV, img_size, grad_filename, norm_factor=KMAX,
                     gamma=GAMMA_HYDROGEN / 1e3, raster_time=DEFAULT_RASTER_TIME,
                     check_constraints=True, TE_pos=0.5, gmax=DEFAULT_GMAX, smax=DEFAULT_SMAX,
                     pregrad=None, postgrad=None, grad_method="auto", version=5, **kwargs):
    """Gradients of a normalised trajectory (shots, samples, d), written as a
    gradient file (nsp.py:218-381).

    The k-space positions are ``trajectory / norm_factor / (2 * FOV / img_size)``
    (1/m) and the gradients their per-shot differences divided by
    ``gamma * raster_time`` (trajectories/utils.py:441-474).  Prephasing and
    spoiling gradients (``pregrad`` / ``postgrad``) come from mri-nufft's
    gradient-connection solver, which is not restated: they raise.
    """
    if pregrad or postgrad:
        if version < 5.1:
            raise ValueError("pregrad and postgrad are only supported for version >= 5.1, "
                             "please set version to 5.1 or higher.")
        raise NotImplementedError("pregrad / postgrad need mri-nufft's gradient connection")
    trajectory = np.asarray(trajectory)
    d = trajectory.shape[-1]
    res = np.array([f / s for f, s in zip(FOV, img_size)])
    k = trajectory / norm_factor / (2 * res[:d])
    gradients = np.diff(k, axis=1) / gamma / raster_time
    initial_positions, final_positions = k[:, 0, :], k[:, -1, :]
    if check_constraints:
        _check_constraints(gradients, raster_time, gmax, smax, pregrad)
    write_gradients(gradients=gradients, initial_positions=initial_positions,
                    final_positions=final_positions, grad_filename=grad_filename,
                    img_size=img_size, FOV=FOV, TE_pos=TE_pos, gamma=gamma, version=version,
                    start_skip_samples=0, end_skip_samples=0, **kwargs)


class _Cursor:
    """Sequential reader over the float32 values of a gradient file."""

    def __init__(self, data):
        self.data, self.pos = data, 0

    def take(self, n=1, dtype=np.float32):
        v = self.data[self.pos:self.pos + n].astype(dtype, copy=False)
        self.pos += n
        return v[0] if n == 1 else v


def read_trajectory(grad_filename, dwell_time=DEFAULT_RASTER_TIME, num_adc_samples=None,
                    gamma=GAMMA_HYDROGEN, raster_time=DEFAULT_RASTER_TIME, read_shots=False,
                    normalize_factor=KMAX, pre_skip=0):
    """K-space locations (shots, adc samples, d) and header parameters of a
    gradient file (nsp.py:384-575).

    ``dwell_time`` in ms, or ``"min_osf"`` for ``raster_time / min_osf``
    from the header.  Sample i >= 1 sits at ``t_i = i * dwell`` on the
    gradient raster (q, r) = divmod(t_i, raster): the initial position plus
    the gradient integral up to raster step q and r ns of step q, times gamma.
    """
    cur = _Cursor(np.fromfile(grad_filename, dtype=np.float32))
    if float(cur.data[0]) > 4:
        version = int(np.around(cur.take() * 10))
    else:
        version = 10
    dimension = cur.take(dtype="int")
    if version >= 41:
        fov = cur.take(dimension)
        img_size = cur.take(dimension, dtype="int")
        min_osf = cur.take(dtype="int")
        gamma = cur.take() / 1000
        if dwell_time == "min_osf":
            dwell_time = raster_time / min_osf
    num_shots, num_samples_per_shot = cur.take(2, dtype="int")
    start_skip, end_skip = 0, 0
    if version > 40:
        TE_pos = cur.take()
        grad_max = cur.take()
        recon_tag = np.around(cur.take(), 2)
        spare = 10
        if version > 41:
            timestamp = datetime.fromtimestamp(float(cur.take()))
            spare -= 1
        if version > 50:
            start_skip, end_skip = cur.take(2, dtype="int")
            spare -= 2
        cur.take(spare)
    initial_positions = cur.take(dimension * num_shots).reshape(num_shots, dimension)
    if version > 45:
        cur.take(dimension * num_shots)  # final positions
    dwell_ns = dwell_time * 1e6
    raster_ns = raster_time * 1e6
    if version < 41:
        grad_max = cur.take()
    gradients = cur.take(dimension * num_samples_per_shot * num_shots)
    gradients = np.reshape(grad_max * gradients * 1e-3, (num_shots, num_samples_per_shot, dimension))
    if start_skip > 0:
        initial_positions += np.sum(gradients[:, :start_skip], axis=1) * raster_time * gamma
        gradients = gradients[:, start_skip:, :]
        num_samples_per_shot -= start_skip
    if end_skip > 0:
        gradients = gradients[:, :-end_skip, :]
        num_samples_per_shot -= end_skip
    if num_adc_samples is None:
        if read_shots:
            num_adc_samples = num_samples_per_shot + 1
        else:
            num_adc_samples = int(num_samples_per_shot * (raster_time / dwell_time))
    kspace_loc = np.zeros((num_shots, num_adc_samples, dimension), dtype=np.float32)
    kspace_loc[:, 0, :] = initial_positions
    Q, R = divmod(dwell_ns * np.arange(1, num_adc_samples), raster_ns)
    Q = Q.astype("int")
    if not np.all((Q < num_adc_samples) | ((Q == num_adc_samples) & (R == 0))):
        logger.warning("Binary file doesn't seem right! Proceeding anyway")
    n = gradients.shape[1]
    acc = np.cumsum(gradients, axis=1) * raster_ns
    ip = initial_positions[:, None, :]
    Rb = R[None, :, None]
    past = Q >= n
    if np.any(Q > n):
        logger.warning("Number of samples is more than what was obtained in binary file!\n"
                       "Data will be extended")
    if n > 0:
        Qc = np.minimum(Q, n - 1)
        # three cases, each with the reference's order of operations
        v_past = ip + (acc[:, n - 1:n, :] + gradients[:, n - 1:n, :] * Rb) * gamma * 1e-6
        v_first = ip + gradients[:, Qc, :] * Rb * gamma * 1e-6
        v_mid = ip + (acc[:, np.maximum(Qc - 1, 0), :] + gradients[:, Qc, :] * Rb) * gamma * 1e-6
        sel = np.where(past[None, :, None], v_past, np.where((Q == 0)[None, :, None], v_first, v_mid))
        kspace_loc[:, 1:, :] = sel
    params = {"version": version / 10, "dimension": dimension, "num_shots": num_shots,
              "num_samples_per_shot": num_samples_per_shot}
    if version >= 41:
        params.update(FOV=fov, img_size=img_size, min_osf=min_osf, gamma=gamma,
                      recon_tag=recon_tag, TE_pos=TE_pos)
        if version >= 42:
            params["timestamp"] = timestamp
    if normalize_factor is not None:
        Kmax = img_size / 2 / fov
        kspace_loc = kspace_loc / Kmax * normalize_factor
        if np.abs(kspace_loc).max() > normalize_factor:
            logger.warning("K-space locations exceed the normalization factor after "
                           "normalization! Clipping the values.")
            kspace_loc = np.clip(kspace_loc, -normalize_factor, normalize_factor)
    if pre_skip > 0:
        if pre_skip >= num_samples_per_shot:
            raise ValueError("skip_first_Nsamples should be less than num_adc_samples")
        skip = pre_skip * int(num_adc_samples / num_samples_per_shot)
        kspace_loc = kspace_loc[:, skip:]
        params["num_adc_samples"] = num_adc_samples - skip
    return kspace_loc, params


# --------------------------------------------------------------------------
# BART .cfl / .hdr
# --------------------------------------------------------------------------
def _pair(cfl_file, hdr_file):
    base = Path(cfl_file).with_suffix("")
    return base.with_suffix(".cfl"), (base.with_suffix(".hdr") if hdr_file is None else hdr_file)


def readcfl(cfl_file, hdr_file=None):
    """Complex64 array of a .cfl / .hdr pair, Fortran order, trailing
    singleton dimensions dropped (cfl.py:19-53)."""
    cfl_file, hdr_file = _pair(cfl_file, hdr_file)
    with open(hdr_file) as h:
        h.readline()
        dims = [int(v) for v in h.readline().split()]
    n = int(np.prod(dims))
    dims = dims[: int(np.searchsorted(np.cumprod(dims), n)) + 1]
    return np.fromfile(cfl_file, dtype=np.complex64, count=n).reshape(dims, order="F")


def writecfl(array, cfl_file, hdr_file=None):
    """Write a .cfl / .hdr pair (complex64, Fortran order; cfl.py:56-86)."""
    cfl_file, hdr_file = _pair(cfl_file, hdr_file)
    array = np.asarray(array)
    with open(hdr_file, "w") as h:
        h.write("# Dimensions\n" + "".join(f"{v} " for v in array.shape) + "\n")
    np.ascontiguousarray(array.astype(np.complex64, copy=False).T).tofile(cfl_file)


def traj2cfl(traj, shape, basename):
    """Trajectory (shots, samples, 2 or 3) in [-0.5, 0.5) -> BART trajectory
    file scaled by ``shape - 1`` with a zero third axis in 2D (cfl.py:89-113)."""
    traj = np.asarray(traj)
    scaled = traj * (np.array(shape) - 1)
    if traj.shape[-1] == 2:
        padded = np.zeros(scaled.shape[:-1] + (3,), dtype=scaled.dtype)
        padded[..., :2] = scaled
        scaled = padded
    writecfl(scaled[None, None].T, basename)


def cfl2traj(basename, shape=None):
    """BART trajectory file -> (shots, samples, d) trajectory (cfl.py:116-146);
    without ``shape`` the extent of the points is used."""
    raw = readcfl(basename)
    traj = np.ascontiguousarray(raw.T.real.astype(np.float32))
    if np.all(traj[..., -1] == 0):
        logger.warning("2D Trajectory Detected")
        traj = traj[..., :-1]
    if shape is None:
        span = traj.reshape(-1, traj.shape[-1])
        shape = span.max(0) - span.min(0)
        logger.warning("Estimated shape %s", shape)
    else:
        shape = np.asarray(shape) - 1
    traj /= np.asarray(shape)
    return np.squeeze(traj)


# --------------------------------------------------------------------------
# k-space helpers
# --------------------------------------------------------------------------
def add_phase_to_kspace_with_shifts(kspace_data, kspace_loc, normalized_shifts):
    """``kspace_data * exp(-2 i pi <k, shift>)`` (utils.py:7-40)."""
    if len(normalized_shifts) != kspace_loc.shape[1]:
        raise ValueError("Dimension mismatch between shift and kspace locations! "
                         "Ensure that shifts are right")
    try:
        import torch
    except ImportError:  # pragma: no cover
        torch = None
    if torch is not None and isinstance(kspace_data, torch.Tensor):
        loc = torch.as_tensor(kspace_loc, device=kspace_data.device)
        shifts = torch.as_tensor(np.asarray(normalized_shifts), device=loc.device, dtype=loc.dtype)
        phi = (loc * shifts).sum(-1)
        return kspace_data * torch.exp(-2j * np.pi * phi)
    phi = np.sum(kspace_loc * normalized_shifts, axis=-1)
    return kspace_data * np.exp(-2 * np.pi * 1j * phi)


def remove_extra_kspace_samples(kspace_data, num_samples_per_shot):
    """Drop ADC samples beyond ``num_samples_per_shot`` on the last axis
    (utils.py:43-67)."""
    extra = kspace_data.shape[-1] - num_samples_per_shot
    return kspace_data[..., :-extra] if extra > 0 else kspace_data
