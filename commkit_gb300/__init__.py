"""commkit-gb300: commkit's coded-modulation receiver back end on GB300 (sm_103a).

The soft LLR demapper (:func:`compute_llr`) and the layered QC-LDPC
decoder (:func:`decode` with :class:`LDPCCode` and :class:`MinSum` or
:class:`SumProduct`) of commkit, rebuilt as hand-written CUDA behind the
reference's public signatures and kernel-registry interface
(:mod:`commkit_gb300.plugin`), with the steps around them on the device:
:func:`encode`, :func:`gmi` / :func:`ngmi` and the Monte-Carlo
:func:`error_rate_curve`.
"""

from .coding import DecodeResult, LDPCCode, MinSum, SumProduct, decode, decode_mixed, encode
from .mapping import Constellation, PrecisionWarning, compute_llr, compute_llr_frames
from .metrics import gmi, ngmi
from .performance import ErrorRateCurve, error_rate_curve

__all__ = [
    "Constellation",
    "DecodeResult",
    "ErrorRateCurve",
    "LDPCCode",
    "MinSum",
    "PrecisionWarning",
    "SumProduct",
    "compute_llr",
    "compute_llr_frames",
    "decode",
    "decode_mixed",
    "encode",
    "error_rate_curve",
    "gmi",
    "ngmi",
]

__version__ = "0.1.0"
