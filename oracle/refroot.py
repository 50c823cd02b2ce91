"""Where the reference checkout (MasterSPP/S_SPI_SPRING) lies, for the
recipes that compile or import parts of it as checkers: the environment
variable SPRING_REFERENCE_ROOT, else the checkout's usual place in the build
container.  The GPU host has no checkout; everything that needs one checks
for it and skips."""
from __future__ import annotations

import os
from pathlib import Path

ENV = "SPRING_REFERENCE_ROOT"
_USUAL = "/root/reference"


def reference_root() -> Path:
    return Path(os.environ.get(ENV) or _USUAL)
