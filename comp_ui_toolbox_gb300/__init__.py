"""GB300-native Born scattering operator of the Computational Ultrasound Imaging Toolbox.

The compute lives in ``libcui_born.so`` (hand-written CUDA for sm_103a behind
the C-ABI in ``include/cui_born.h``); this package holds the build recipe and
the Python host mirror of the reference's operator interface.
"""

from .born import (BornForward, CuiError, OperatorBorn, born_forward, launch_count,  # noqa: F401
                   load_library)

__all__ = ["OperatorBorn", "CuiError", "BornForward", "born_forward", "load_library", "launch_count"]
