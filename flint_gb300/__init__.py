"""flint_gb300: FLINT's per-cell chemistry hot path on GB300 (sm_103a).

The compute path is the in-tree CUDA library ``_lib/libflint_gb300.so``
reached through the C-ABI of include/flint_gpu.h (``flint_gb300.native``);
``flint_gb300.api`` mirrors FLINT's Fortran procedures over it.
"""
import os

__version__ = "0.1.0"

_HERE = os.path.dirname(os.path.abspath(__file__))


def data_path(name):
    """Path of a packaged data file (mechanisms, species pool)."""
    return os.path.join(_HERE, "data", name)
