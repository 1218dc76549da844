"""GB300-native Kaiser-Bessel Fourier gridder.

Drop-in for the setVolume / forwardProject / backProject / getVol /
reconstructVol path of tagarelab/MultiGPUGridder: hand-written sm_103a CUDA
kernels behind the C ABI of include/gg_gridder.h (libgg_gridder.so, built in
tree), with this package as the Python face of that ABI.
"""
from ._lib import GridderError, lib  # noqa: F401
from .gridder import MultiGPUGridder, adjust_interp_factor  # noqa: F401

__all__ = ["MultiGPUGridder", "GridderError", "adjust_interp_factor", "lib"]
