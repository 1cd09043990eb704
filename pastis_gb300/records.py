"""Record layouts and residue letters shared by the bindings and the generator.

This module loads no native library: the synthetic-data generator and the CPU
timing of the reference path use it without mapping the CUDA library.

  PAIR_DTYPE      pg_pair (20 B): row, col, two seeds (row off, col off), count,
                  k-mer score; filled from CommonKmerLoc (inc/Types.hpp:163-215)
  RESULT_DTYPE    pg_result (40 B): score, statistics, coordinates, identity,
                  score_aln (the value PASTIS keeps), flags, DP cells
  KMERLOC_DTYPE   CommonKmerLoc as laid out in inc/Types.hpp:163-215
  KMERLIGHT_DTYPE CommonKmerLight as laid out in inc/Types.hpp:220-266
"""
import ctypes
import os

import numpy as np

NRES = 25
LETTERS = "ARNDCQEGHILKMFPSTWYVBZX*J"

PAIR_DTYPE = np.dtype([("row", "<u4"), ("col", "<u4"), ("rs0", "<u2"), ("cs0", "<u2"),
                       ("rs1", "<u2"), ("cs1", "<u2"), ("count", "<u2"), ("score", "<i2")])
RESULT_DTYPE = np.dtype([("score", "<i4"), ("aln_len", "<u4"), ("matches", "<u4"),
                         ("gap_opens", "<u4"), ("beg_h", "<u2"), ("end_h", "<u2"),
                         ("beg_v", "<u2"), ("end_v", "<u2"), ("identity", "<f4"),
                         ("score_aln", "<f4"), ("seed_used", "u1"), ("flags", "u1"),
                         ("pad", "<u2"), ("cells", "<u4")])
KMERLOC_DTYPE = np.dtype([("count", "<u2"), ("score", "<i2"), ("score_aln", "<f4"),
                          ("first_r", "<u2"), ("first_c", "<u2"),
                          ("second_r", "<u2"), ("second_c", "<u2")])
KMERLIGHT_DTYPE = np.dtype([("count", "<u2"), ("score", "<i2"), ("score_aln", "<f4")])
assert PAIR_DTYPE.itemsize == 20 and RESULT_DTYPE.itemsize == 40
assert KMERLOC_DTYPE.itemsize == 16 and KMERLIGHT_DTYPE.itemsize == 8

BUILD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build")


def decode(codes):
    """Residue codes (0..24) to ASCII letters."""
    lut = np.frombuffer(LETTERS.encode(), dtype=np.uint8)
    return lut[np.asarray(codes, dtype=np.uint8)]


def native_path(name):
    path = os.path.join(BUILD, name)
    if not os.path.exists(path):
        raise RuntimeError("native library %s is missing; run pastis_gb300.build.build()" % path)
    return path


def cdll(name):
    return ctypes.CDLL(native_path(name), mode=ctypes.RTLD_GLOBAL)
