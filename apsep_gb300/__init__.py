"""apsep_gb300 -- GB300-native All Previous Smaller Element engine.

The compute path is libapsep.so (hand-written CUDA for sm_103a behind a C
ABI, include/apsep.h); this package is its Python host mirror.  Importing
the package does not load the library; the first call does, and fails
loudly if it was not built (`python -m apsep_gb300.build`).
"""
from .api import (  # noqa: F401
    ApsepError,
    Plan,
    alloc_spt_scratch,
    alloc_wstl_scratch,
    apse,
    apse64,
    apse_segmented,
    free_spt_scratch,
    free_wstl_scratch,
    launch_spt,
    launch_wstl,
    run_spt,
    run_wstl,
)

__version__ = "0.1.0"
