"""xcape_gb300 -- GB300 (sm_103a) CUDA kernels behind xcape's calc_cape / calc_srh.

``from xcape_gb300 import calc_cape, calc_srh`` is a drop-in for
``from xcape.core import calc_cape, calc_srh`` with ``method='cuda'`` as the
default.  The compute path is ``libxcape_gb300.so`` (C ABI declared in
``include/xcape_gb300.h``); there is no CPU fallback.
"""
from .core import (calc_cape, calc_cape_diagnostics, calc_cape_sources, calc_cape_srh,  # noqa: F401
                   calc_srh)
from ._lib import XcapeError, version  # noqa: F401

__all__ = ["calc_cape", "calc_cape_diagnostics", "calc_cape_sources", "calc_cape_srh", "calc_srh",
           "XcapeError", "version"]
__version__ = "0.1.0"
