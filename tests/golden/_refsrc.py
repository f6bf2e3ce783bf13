"""Location of the mri-nufft sources that the fixture scripts run.

Every ``make_*_golden.py`` script imports mri-nufft from a source tree given
as its first argument or, failing that, by the ``MRINUFFT_SRC`` environment
variable (the directory that holds the ``mrinufft`` package).  There is no
default: the scripts regenerate fixtures from a checkout the caller names.
"""

from __future__ import annotations

import os
import sys
from pathlib import Path


def reference_src(argv=None) -> str:
    argv = sys.argv if argv is None else argv
    src = argv[1] if len(argv) > 1 else os.environ.get("MRINUFFT_SRC")
    if not src:
        raise SystemExit("usage: python %s <mri-nufft src directory>  (or set MRINUFFT_SRC)"
                         % Path(argv[0]).name)
    if not (Path(src) / "mrinufft").is_dir():
        raise SystemExit(f"{src!r} does not contain the mrinufft package")
    return src
