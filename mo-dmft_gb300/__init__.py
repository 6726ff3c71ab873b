"""GB300 exact-diagonalization impurity solver for MO-DMFT (sm_103a).

The product is the C-ABI library ``lib/libmoed.so`` (sources in ``csrc/``,
declared in ``include/mo_ed.h`` at the repository root); ``ed.py`` mirrors the
reference's ED / bath-fit routines on top of it; ``dmft.py`` runs the
reference's DMFT loop through it; ``configs.py`` holds the seeded synthetic
benchmark models and the FDF input reader / writer.
"""
from . import configs  # noqa: F401
from .dmft import dmft_loop  # noqa: F401
from .ed import (EDError, EDSolver, FP32, FP64, Options, ev_to_x, icom, lib, matsubara,  # noqa: F401
                 x_to_ev)
