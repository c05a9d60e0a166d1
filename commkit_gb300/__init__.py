"""commkit-gb300: commkit's coded-modulation receiver back end on GB300 (sm_103a).

The soft LLR demapper (:func:`compute_llr`) and the layered QC-LDPC min-sum
decoder (:func:`decode` with :class:`LDPCCode` and :class:`MinSum`) of
commkit, rebuilt as hand-written CUDA behind the reference's public
signatures and kernel-registry interface (:mod:`commkit_gb300.plugin`).
"""

from .coding import DecodeResult, LDPCCode, MinSum, SumProduct, decode, decode_mixed
from .mapping import Constellation, PrecisionWarning, compute_llr, compute_llr_frames

__all__ = [
    "Constellation",
    "DecodeResult",
    "LDPCCode",
    "MinSum",
    "PrecisionWarning",
    "SumProduct",
    "compute_llr",
    "compute_llr_frames",
    "decode",
    "decode_mixed",
]

__version__ = "0.1.0"
