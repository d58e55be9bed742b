"""Enumerations with the same integer values as USTB's MATLAB enums.

dimension.m:27-32, code.m:23-28, +uff/window.m, +uff/wavefront.m,
spherical_transmit_delay_model.m:32-37.  ``Code.python`` is the value the
reference's Python package adds (python/src/ustb/enums.py:36-42); ``Code.gb300``
selects this library.
"""
from enum import IntEnum


class Dimension(IntEnum):
    none = 0
    receive = 1
    transmit = 2
    both = 3


class Code(IntEnum):
    matlab = 0
    mex = 1
    python = 2
    matlab_gpu = 3
    mex_gpu = 4
    gb300 = 5


class Window(IntEnum):
    none = 0
    boxcar = 1
    rectangular = 1
    flat = 1
    hanning = 2
    hamming = 3
    tukey25 = 4
    tukey50 = 5
    tukey75 = 6
    sta = 7
    scanline = 8
    triangle = 9


class Wavefront(IntEnum):
    plane = 0
    spherical = 1
    photoacoustic = 2


class SphericalTransmitDelayModel(IntEnum):
    spherical = 1
    unified = 2
    hybrid = 3
    blended = 4


class Precision(IntEnum):
    """Storage type of channel data on the device (arithmetic is always FP32)."""
    fp32 = 0
    fp16 = 1
    bf16 = 2
