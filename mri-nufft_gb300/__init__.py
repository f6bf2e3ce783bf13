"""GB300-native NUFFT backend for mri-nufft.

``MRIGB300`` (backend ``"gb300"``) is a drop-in NUFFT operator whose op,
adj_op, data consistency, pipe density, Lipschitz estimate and CG solver run
on hand-written sm_103a CUDA kernels in ``libgbnufft.so`` (C ABI in
``include/gbnufft.h``).  When ``mrinufft`` is installed, the class registers
in its backend table, so ``mrinufft.get_operator("gb300")`` returns it.
"""

from ._lib import GB300Error, library_path, load as load_library
from .operator import HAVE_MRINUFFT, MRIGB300, power_method
from .stacked import MRIStackedGB300
from .offres import MRIFourierCorrectedGB300
from .plan import NufftPlan, dotu_f64, norm2_f64
from ._traj import proper_trajectory

if HAVE_MRINUFFT:  # pragma: no cover - depends on the environment
    from mrinufft.operators.base import get_operator  # type: ignore
else:
    from ._base import get_operator

__all__ = [
    "MRIGB300",
    "MRIStackedGB300",
    "MRIFourierCorrectedGB300",
    "NufftPlan",
    "GB300Error",
    "get_operator",
    "power_method",
    "proper_trajectory",
    "norm2_f64",
    "dotu_f64",
    "library_path",
    "load_library",
    "HAVE_MRINUFFT",
]
