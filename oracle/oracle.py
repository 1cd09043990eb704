"""ctypes front end of the CPU oracle (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this module.  The product library never calls it.
Parity with SeqAn is unpinned: see ``pastis_oracle.h``.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")

NRES = 25
LETTERS = "ARNDCQEGHILKMFPSTWYVBZX*J"

TIE_H_E_BEFORE_F = 1
TIE_GAP_OPEN_FIRST = 2
F_SKIP_SPURIOUS_SEED = 1
F_XDROP_AFFINE = 2

RF_EMPTY, RF_BAD_SEED, RF_PASSED = 1, 2, 4

PAIR_DTYPE = np.dtype([("row", "<u4"), ("col", "<u4"), ("rs0", "<u2"), ("cs0", "<u2"),
                       ("rs1", "<u2"), ("cs1", "<u2"), ("count", "<u2"), ("score", "<i2")])
RESULT_DTYPE = np.dtype([("score", "<i4"), ("aln_len", "<u4"), ("matches", "<u4"),
                         ("gap_opens", "<u4"), ("beg_h", "<u2"), ("end_h", "<u2"),
                         ("beg_v", "<u2"), ("end_v", "<u2"), ("identity", "<f4"),
                         ("score_aln", "<f4"), ("seed_used", "u1"), ("flags", "u1"),
                         ("pad", "<u2"), ("cells", "<u4")])
assert PAIR_DTYPE.itemsize == 20 and RESULT_DTYPE.itemsize == 40


class Params(ctypes.Structure):
    _fields_ = [("gap_first", ctypes.c_int32), ("gap_ext", ctypes.c_int32),
                ("xdrop_gap", ctypes.c_int32), ("xdrop", ctypes.c_int32),
                ("seed_len", ctypes.c_int32), ("seed_count", ctypes.c_int32),
                ("tie", ctypes.c_int32), ("flags", ctypes.c_int32),
                ("cov_thr", ctypes.c_double), ("ani_thr", ctypes.c_int32),
                ("sm", ctypes.c_int8 * (NRES * NRES))]


def build(force=False):
    """Compile the oracle with gcc (C99 + OpenMP, no ISA flags)."""
    src = os.path.join(HERE, "pastis_oracle.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "pastis_oracle.h"))):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O3", "-std=c99", "-fopenmp", "-shared", "-fPIC",
                           "-o", tmp, src])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        _lib.orc_batch.restype = ctypes.c_int
        _lib.orc_xdrop_extend.restype = ctypes.c_uint64
        _lib.orc_max_threads.restype = ctypes.c_int
    return _lib


def blosum62():
    out = (ctypes.c_int8 * (NRES * NRES))()
    lib().orc_blosum62(out)
    return np.frombuffer(out, dtype=np.int8).reshape(NRES, NRES).copy()


def encode(s):
    table = np.full(256, 22, dtype=np.uint8)
    for i, c in enumerate(LETTERS):
        table[ord(c)] = i
        table[ord(c.lower())] = i
    b = np.frombuffer(s.encode("ascii") if isinstance(s, str) else bytes(s), dtype=np.uint8)
    return table[b]


def make_params(gap_first=-11, gap_ext=-2, xdrop_gap=None, xdrop=49, seed_len=6,
                seed_count=2, tie=0, flags=0, cov_thr=0.7, ani_thr=30, sm=None):
    p = Params()
    p.gap_first, p.gap_ext = gap_first, gap_ext
    p.xdrop_gap = gap_ext if xdrop_gap is None else xdrop_gap
    p.xdrop, p.seed_len, p.seed_count = xdrop, seed_len, seed_count
    p.tie, p.flags, p.cov_thr, p.ani_thr = tie, flags, cov_thr, ani_thr
    m = blosum62() if sm is None else np.asarray(sm, dtype=np.int8)
    ctypes.memmove(p.sm, m.ctypes.data, NRES * NRES)
    return p


def pastis_params(as_called=True, **over):
    """PASTIS's alignment defaults (src/main.cpp:97-116, :158-166): gap open
    -11, gap extend -2, x = 49, k = 6, two seeds, coverage 0.7, ANI 30.

    as_called: the gaps reach SeqAn's Score(gapExtend, gapOpen) constructor in
    the order PASTIS passes them (src/align/SeqanXdropAligner.hpp:38-43), so
    the first gap position scores -2, further positions -11 and the X-drop
    extension's linear gap is -11.  Otherwise the nominal reading: first -11,
    further -2, X-drop gap -2."""
    first, ext = (-2, -11) if as_called else (-11, -2)
    kw = dict(gap_first=first, gap_ext=ext, xdrop_gap=ext, xdrop=49, seed_len=6, seed_count=2,
              tie=0, flags=0, cov_thr=0.7, ani_thr=30)
    kw.update(over)
    return make_params(**kw)


def _u8(a):
    return np.ascontiguousarray(a, dtype=np.uint8)


def _res1():
    return np.zeros(1, dtype=RESULT_DTYPE)


def local(v, h, p):
    v, h = _u8(v), _u8(h)
    out = _res1()
    lib().orc_local(v.ctypes.data_as(ctypes.c_void_p), len(v), h.ctypes.data_as(ctypes.c_void_p),
                    len(h), ctypes.byref(p), out.ctypes.data_as(ctypes.c_void_p))
    return out[0]


def global_(v, h, p):
    v, h = _u8(v), _u8(h)
    out = _res1()
    lib().orc_global(v.ctypes.data_as(ctypes.c_void_p), len(v), h.ctypes.data_as(ctypes.c_void_p),
                     len(h), ctypes.byref(p), out.ctypes.data_as(ctypes.c_void_p))
    return out[0]


def align_fast(v, h, p, local_):
    """The packed DP the batch entry points use (must equal local()/global_())."""
    v, h = _u8(v), _u8(h)
    out = _res1()
    lib().orc_align_fast(v.ctypes.data_as(ctypes.c_void_p), len(v), h.ctypes.data_as(ctypes.c_void_p),
                         len(h), ctypes.byref(p), ctypes.c_int(1 if local_ else 0),
                         out.ctypes.data_as(ctypes.c_void_p))
    return out[0]


def xdrop_extend(v, h, p, bh, eh, bv, ev):
    v, h = _u8(v), _u8(h)
    a = [ctypes.c_int(x) for x in (bh, eh, bv, ev)]
    cells = lib().orc_xdrop_extend(v.ctypes.data_as(ctypes.c_void_p), len(v),
                                   h.ctypes.data_as(ctypes.c_void_p), len(h), ctypes.byref(p),
                                   *[ctypes.byref(x) for x in a])
    return tuple(x.value for x in a), int(cells)


def batch(mode, rseq, roffs, cseq, coffs, pairs, p, bl_roff=0, bl_coff=0, nthreads=0):
    """mode 0 = SW (--sfa), 1 = X-drop (--sxa); returns a RESULT_DTYPE array."""
    rseq, cseq = _u8(rseq), _u8(cseq)
    roffs = np.ascontiguousarray(roffs, dtype=np.uint64)
    coffs = np.ascontiguousarray(coffs, dtype=np.uint64)
    pairs = np.ascontiguousarray(pairs, dtype=PAIR_DTYPE)
    out = np.zeros(len(pairs), dtype=RESULT_DTYPE)
    vp = ctypes.c_void_p
    rc = lib().orc_batch(ctypes.c_int(mode), rseq.ctypes.data_as(vp), roffs.ctypes.data_as(vp),
                         ctypes.c_uint64(len(roffs) - 1), cseq.ctypes.data_as(vp),
                         coffs.ctypes.data_as(vp), ctypes.c_uint64(len(coffs) - 1),
                         pairs.ctypes.data_as(vp), ctypes.c_uint64(len(pairs)),
                         ctypes.c_uint64(bl_roff), ctypes.c_uint64(bl_coff), ctypes.byref(p),
                         ctypes.c_int(nthreads), out.ctypes.data_as(vp))
    if rc != 0:
        raise IndexError("pair index out of range")
    return out


def max_threads():
    return int(lib().orc_max_threads())
