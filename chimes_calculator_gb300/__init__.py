"""GB300-native ChIMES force evaluation.

The hot path of the ChIMES calculator -- cluster-list build, Morse/Chebyshev
stage and coefficient contraction with energy/force/virial reduction -- as
hand-written sm_103a CUDA behind the reference's own C interfaces
(``libchimescalc.so``).  ``Calculator`` is the Python entry point,
``chimescalc_serial_py`` mirrors the reference's ctypes wrapper.
"""

from .api import FP64, MIXED, Calculator, ChimesError  # noqa: F401

__all__ = ["Calculator", "ChimesError", "FP64", "MIXED"]
