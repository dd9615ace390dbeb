"""GB300-native (sm_103a) VESPER alignment hot path: fastVEC, query rotation,
per-rotation FFT cross-correlation (modes V/O/C/P/L and the probability
channels) and top-N selection, behind the reference's Python API and
``main.py orig|prob`` command line.  The compute runs in the C-ABI library
``libvesper_gb300.so`` (include/vesper_gb300.h); there is no CPU fallback."""
from ._native import VesperError, build, load  # noqa: F401

__version__ = "0.1.0"
