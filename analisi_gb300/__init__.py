"""analisi_gb300: GB300-native (sm_103a) van Hove g(r,t) -- analisi's Gofrt.

The engine is CUDA behind the C ABI of include/gofr_gb300.h
(analisi_gb300/_build/libgofr_gb300.so).  Front ends:
  analisi_gb300.engine     ctypes binding of the C ABI
  analisi_gb300.pyanalisi  pybind11 module with the reference's Gofrt /
                           Trajectory / BoxFormat API (built in _build/)
  analisi_gb300/_build/analisi   command line with the reference's -g/-F options
"""
import os
import sys

__all__ = ["engine", "load_pyanalisi"]

_BUILD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build")


def load_pyanalisi():
    """Import the pybind11 module built in analisi_gb300/_build/."""
    if _BUILD not in sys.path:
        sys.path.insert(0, _BUILD)
    import pyanalisi  # noqa: E402
    return pyanalisi
