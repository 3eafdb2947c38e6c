"""namsa_gb300 -- GB300-native STEM/CBED multislice engine.

``MSAGPU`` keeps the simulator-class surface of namsa's ``MSAGPU``
(namsa/msa.py:529-992); the compute runs in libmsx.so (hand-written CUDA for
sm_103a) reached through the C ABI in include/msx.h.
"""
from .msa import MSAGPU, XYZ_dtype  # noqa: F401
from .optics import voltage2Lambda, sigma_int, scherzer_defocus  # noqa: F401

__version__ = '1.0.0'
