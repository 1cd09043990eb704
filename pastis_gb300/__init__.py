"""pastis_gb300 -- GB300-native batched pairwise alignment for PASTIS.

The alignment stage of PASTIS (affine Smith-Waterman, --sfa, and seeded X-drop
extension + global alignment, --sxa) as hand-written sm_103a CUDA kernels
behind a C ABI (include/pastis_gb300.h), with the reference's aligner plug-in
interface mirrored in C++ (include/pastis_gb300_pwalign.hpp).
"""
from . import build  # noqa: F401
from .capi import (Context, PgError, config, load, pw_aln_batch, PAIR_DTYPE,  # noqa: F401
                   RESULT_DTYPE, KMERLOC_DTYPE, KMERLIGHT_DTYPE, MODE_SW, MODE_XDROP,
                   GAPS_AS_CALLED, GAPS_NOMINAL)

__all__ = ["build", "Context", "PgError", "config", "load", "pw_aln_batch", "PAIR_DTYPE",
           "RESULT_DTYPE", "KMERLOC_DTYPE", "KMERLIGHT_DTYPE", "MODE_SW", "MODE_XDROP",
           "GAPS_AS_CALLED", "GAPS_NOMINAL"]
