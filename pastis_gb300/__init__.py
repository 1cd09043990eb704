"""pastis_gb300 -- GB300-native batched pairwise alignment for PASTIS.

The alignment stage of PASTIS (affine Smith-Waterman, --sfa, and seeded X-drop
extension + global alignment, --sxa) as hand-written sm_103a CUDA kernels
behind a C ABI (include/pastis_gb300.h), with the reference's aligner plug-in
interface mirrored in C++ (include/pastis_gb300_pwalign.hpp).

The bindings (``capi``) are imported on first use of one of their names, so
that the generator (``synth``) and the record layouts (``records``) can be
used without the CUDA library.
"""
from . import build  # noqa: F401
from .records import (KMERLIGHT_DTYPE, KMERLOC_DTYPE, PAIR_DTYPE,  # noqa: F401
                      RESULT_DTYPE)

_CAPI_NAMES = ("Context", "PgError", "config", "load", "pw_aln_batch", "MODE_SW", "MODE_XDROP",
               "GAPS_AS_CALLED", "GAPS_NOMINAL")

__all__ = ["build", "PAIR_DTYPE", "RESULT_DTYPE", "KMERLOC_DTYPE", "KMERLIGHT_DTYPE",
           *_CAPI_NAMES]


def __getattr__(name):
    if name in _CAPI_NAMES:
        from . import capi
        return getattr(capi, name)
    raise AttributeError("module %r has no attribute %r" % (__name__, name))
