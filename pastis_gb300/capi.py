"""ctypes bindings of the C ABI (include/pastis_gb300.h) and the C++ host driver.

The CUDA library must be present: loading raises if it is missing, there is no
CPU fallback.
"""
import ctypes
import os

import numpy as np

from . import build as _build

BUILD = _build.BUILD

PG_OK = 0
PG_ERR_ARG, PG_ERR_CUDA, PG_ERR_OOM = -1, -2, -3
PG_ERR_STATE, PG_ERR_RANGE, PG_ERR_NODEV = -5, -6, -7
MODE_SW, MODE_XDROP = 0, 1
GAPS_AS_CALLED, GAPS_NOMINAL = 0, 1
TIE_H_E_BEFORE_F, TIE_GAP_OPEN_FIRST = 1, 2
F_SKIP_SPURIOUS_SEED = 1
F_XDROP_AFFINE = 2
RF_EMPTY, RF_BAD_SEED, RF_PASSED, RF_FILTERED = 1, 2, 4, 8
from .records import (KMERLIGHT_DTYPE, KMERLOC_DTYPE, LETTERS, NRES,  # noqa: F401
                      PAIR_DTYPE, RESULT_DTYPE, decode)

# every entry point declared in include/*.h (checked by the CPU tests)
EXPORTS = {
    "libpastis_gb300.so": ["pg_config_default", "pg_create", "pg_destroy", "pg_set_seqs",
                           "pg_share_row_seqs", "pg_align", "pg_align_device", "pg_sync",
                           "pg_last_launches", "pg_exec_cells", "pg_exec_cells_split",
                           "pg_kernel_ms", "pg_dpx_peak", "pg_strerror", "pg_last_error",
                           "pg_version", "pg_align_sw_noalloc", "pg_filter_create",
                           "pg_filter_destroy", "pg_filter_nparams", "pg_filter_params",
                           "pg_filter_features", "pg_filter_predict", "pg_filter_gradients",
                           "pg_filter_train_step", "pg_align_filtered", "pg_tuning_default",
                           "pg_get_tuning", "pg_set_tuning", "pg_kmer_config_default",
                           "pg_candidates", "pg_triples", "pg_set_seqs_fasta", "pg_get_seqs"],
    "libpastis_synth.so": ["pg_synth_generate", "pg_synth_free", "pg_synth_nseqs",
                           "pg_synth_nres", "pg_synth_npairs", "pg_synth_seq", "pg_synth_offs",
                           "pg_synth_family", "pg_synth_pairs", "pg_synth_homolog",
                           "pg_synth_spurious"],
    "libpastis_host.so": ["pgh_pw_aln_batch", "pgh_pw_aln_batch_resume", "pgh_last_error",
                          "pgh_write_mm"],
}


class Config(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int32), ("gap_open", ctypes.c_int32),
                ("gap_ext", ctypes.c_int32), ("gap_semantics", ctypes.c_int32),
                ("xdrop", ctypes.c_int32), ("seed_len", ctypes.c_int32),
                ("seed_count", ctypes.c_int32), ("tie", ctypes.c_int32),
                ("flags", ctypes.c_int32), ("ani_thr", ctypes.c_int32),
                ("cov_thr", ctypes.c_double), ("device", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("score_matrix", ctypes.c_void_p)]


class Tuning(ctypes.Structure):
    """pg_tuning: launch shape of a context (results never depend on it)."""
    _fields_ = [("dp_blocks_per_sm", ctypes.c_int32), ("xd_blocks_per_sm", ctypes.c_int32),
                ("bucket_order", ctypes.c_int32), ("rows_max", ctypes.c_int32),
                ("graph", ctypes.c_int32), ("xd_int16", ctypes.c_int32),
                ("dp_traceback", ctypes.c_int32), ("dir_arena_mb", ctypes.c_int32),
                ("xd_stepped", ctypes.c_int32)]

    FIELDS = ("dp_blocks_per_sm", "xd_blocks_per_sm", "bucket_order", "rows_max", "graph",
              "xd_int16", "dp_traceback", "dir_arena_mb", "xd_stepped")

    def as_dict(self):
        return {k: int(getattr(self, k)) for k in self.FIELDS}


_libs = {}


ALPH_PROTEIN, ALPH_MURPHY10 = 0, 1
PRUNE_NONE, PRUNE_EVEN_ODD, PRUNE_UPPER = 0, 1, 2


class KmerConfig(ctypes.Structure):
    """pg_kmer_config: k-mer candidate generation (the SpGEMM and its semiring)."""
    _fields_ = [("k", ctypes.c_int32), ("stride", ctypes.c_int32), ("alphabet", ctypes.c_int32),
                ("prune", ctypes.c_int32), ("ckthr", ctypes.c_int32), ("mosthr", ctypes.c_int32),
                ("max_products", ctypes.c_uint64)]


def kmer_config(**fields):
    kc = KmerConfig()
    load().pg_kmer_config_default(ctypes.byref(kc))
    for k, v in fields.items():
        setattr(kc, k, v)
    return kc


def triples_device(d_pairs, d_res, n, roff, coff, d_rows, d_cols, d_vals, stream=None):
    """Similarity triples (row, col, score_aln != 0) of an aligned batch, on
    the device; returns how many were written."""
    cnt = ctypes.c_uint64()
    _check(load().pg_triples(d_pairs, d_res, n, roff, coff, d_rows, d_cols, d_vals,
                             ctypes.byref(cnt), stream))
    return int(cnt.value)


def write_mm(path, nrows, ncols, rows, cols, vals):
    """Matrix Market file of similarity triples (host arrays)."""
    rows = np.ascontiguousarray(rows, dtype=np.uint64)
    cols = np.ascontiguousarray(cols, dtype=np.uint64)
    vals = np.ascontiguousarray(vals, dtype=np.float32)
    lib = load("libpastis_host.so")
    rc = lib.pgh_write_mm(str(path).encode(), nrows, ncols, rows.ctypes.data, cols.ctypes.data,
                          vals.ctypes.data, len(rows))
    if rc != PG_OK:
        raise PgError(rc, lib.pgh_last_error().decode(errors="replace"))


def default_tuning():
    t = Tuning()
    load().pg_tuning_default(ctypes.byref(t))
    return t


def load(name="libpastis_gb300.so"):
    """Load one of the native libraries (built in-tree by pastis_gb300.build)."""
    if name not in _libs:
        path = os.path.join(BUILD, name)
        if not os.path.exists(path):
            raise RuntimeError("native library %s is missing; run pastis_gb300.build.build()" % path)
        lib = ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)
        _declare(name, lib)
        _libs[name] = lib
    return _libs[name]


def _declare(name, lib):
    vp, u64, i32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32
    if name == "libpastis_gb300.so":
        lib.pg_config_default.argtypes = [ctypes.POINTER(Config), i32]
        lib.pg_config_default.restype = None
        lib.pg_create.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(vp)]
        lib.pg_destroy.argtypes = [vp]
        lib.pg_destroy.restype = None
        lib.pg_set_seqs.argtypes = [vp, i32, vp, vp, u64]
        lib.pg_share_row_seqs.argtypes = [vp]
        lib.pg_align.argtypes = [vp, vp, u64, u64, u64, vp]
        lib.pg_align_device.argtypes = [vp, vp, u64, u64, u64, vp, vp]
        lib.pg_sync.argtypes = [vp]
        lib.pg_last_launches.argtypes = [vp]
        lib.pg_exec_cells.argtypes = [vp]
        lib.pg_exec_cells.restype = ctypes.c_ulonglong
        lib.pg_exec_cells_split.argtypes = [vp, vp]
        lib.pg_kernel_ms.argtypes = [vp, vp]
        lib.pg_dpx_peak.argtypes = [i32, ctypes.POINTER(ctypes.c_double)]
        lib.pg_kmer_config_default.argtypes = [vp]
        lib.pg_kmer_config_default.restype = None
        lib.pg_candidates.argtypes = [vp, vp, u64, u64, u64, u64, vp, u64,
                                      ctypes.POINTER(u64), vp]
        lib.pg_set_seqs_fasta.argtypes = [vp, i32, ctypes.c_char_p, u64, i32, ctypes.POINTER(u64),
                                          ctypes.POINTER(u64), vp, u64]
        lib.pg_get_seqs.argtypes = [vp, i32, vp, vp, ctypes.POINTER(u64), ctypes.POINTER(u64)]
        lib.pg_triples.argtypes = [vp, vp, u64, u64, u64, vp, vp, vp, ctypes.POINTER(u64), vp]
        lib.pg_tuning_default.argtypes = [vp]
        lib.pg_tuning_default.restype = None
        lib.pg_get_tuning.argtypes = [vp, vp]
        lib.pg_set_tuning.argtypes = [vp, vp]
        lib.pg_align_sw_noalloc.argtypes = [ctypes.POINTER(Config), vp, vp, u64, vp, vp, u64,
                                            ctypes.c_uint32, vp, u64, u64, u64, vp, vp]
        lib.pg_filter_create.argtypes = [i32, u64, ctypes.POINTER(vp)]
        lib.pg_filter_destroy.argtypes = [vp]
        lib.pg_filter_destroy.restype = None
        lib.pg_filter_params.argtypes = [vp, vp, i32]
        lib.pg_filter_features.argtypes = [vp, vp, vp, u64, u64, u64, vp, vp]
        lib.pg_filter_predict.argtypes = [vp, vp, u64, vp, vp]
        lib.pg_filter_gradients.argtypes = [vp, vp, vp, vp, u64, vp, vp]
        lib.pg_filter_train_step.argtypes = [vp, vp, vp, vp, u64, ctypes.c_float,
                                             ctypes.POINTER(ctypes.c_float), vp]
        lib.pg_align_filtered.argtypes = [vp, vp, ctypes.c_float, vp, u64, u64, u64, vp, vp,
                                          ctypes.POINTER(ctypes.c_uint64)]
        lib.pg_strerror.argtypes = [i32]
        lib.pg_strerror.restype = ctypes.c_char_p
        lib.pg_last_error.restype = ctypes.c_char_p
        lib.pg_version.restype = ctypes.c_char_p
    elif name == "libpastis_synth.so":
        from .synth import declare
        declare(lib)
    elif name == "libpastis_host.so":
        lib.pgh_last_error.restype = ctypes.c_char_p
        lib.pgh_write_mm.argtypes = [ctypes.c_char_p, u64, u64, vp, vp, vp, u64]


class PgError(RuntimeError):
    def __init__(self, code, detail=""):
        self.code = code
        msg = load().pg_strerror(code).decode()
        super().__init__("%s (%d): %s" % (msg, code, detail))


def _check(rc):
    if rc != PG_OK:
        raise PgError(rc, load().pg_last_error().decode(errors="replace"))


def config(mode=MODE_XDROP, **kw):
    c = Config()
    load().pg_config_default(ctypes.byref(c), mode)
    for k, v in kw.items():
        if k == "score_matrix":
            continue
        setattr(c, k, v)
    return c


def resolved_gaps(cfg):
    """(first position, further positions, X-drop linear gap) the kernels use."""
    if cfg.gap_semantics == GAPS_AS_CALLED:
        return cfg.gap_ext, cfg.gap_open, cfg.gap_open
    return cfg.gap_open, cfg.gap_ext, cfg.gap_ext


def dpx_peak(device=0):
    """Measured DPX add-max instructions per second on a device."""
    v = ctypes.c_double()
    _check(load().pg_dpx_peak(device, ctypes.byref(v)))
    return v.value


class Context:
    """Owns one pg_ctx (one device, one mode)."""

    def __init__(self, cfg):
        self.lib = load()
        self.cfg = cfg
        self._sm = None
        h = ctypes.c_void_p()
        _check(self.lib.pg_create(ctypes.byref(cfg), ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.pg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_seqs(self, side, residues_ascii, offsets):
        res = np.ascontiguousarray(residues_ascii, dtype=np.uint8)
        offs = np.ascontiguousarray(offsets, dtype=np.uint64)
        _check(self.lib.pg_set_seqs(self.h, side, res.ctypes.data, offs.ctypes.data,
                                    len(offs) - 1))

    def share_row_seqs(self):
        _check(self.lib.pg_share_row_seqs(self.h))

    def align(self, pairs, bl_roff=0, bl_coff=0, out=None):
        pairs = np.ascontiguousarray(pairs, dtype=PAIR_DTYPE)
        if out is None:
            out = np.zeros(len(pairs), dtype=RESULT_DTYPE)
        _check(self.lib.pg_align(self.h, pairs.ctypes.data, len(pairs), bl_roff, bl_coff,
                                 out.ctypes.data))
        return out

    def align_device(self, d_pairs_ptr, n, d_out_ptr, stream_ptr=None, bl_roff=0, bl_coff=0):
        _check(self.lib.pg_align_device(self.h, d_pairs_ptr, n, bl_roff, bl_coff, d_out_ptr,
                                        stream_ptr))

    def sync(self):
        _check(self.lib.pg_sync(self.h))

    def last_launches(self):
        return int(self.lib.pg_last_launches(self.h))

    def exec_cells(self):
        return int(self.lib.pg_exec_cells(self.h))

    def exec_cells_split(self):
        """(X-drop band cells, alignment DP cells) computed since creation."""
        v = (ctypes.c_ulonglong * 2)()
        _check(self.lib.pg_exec_cells_split(self.h, v))
        return int(v[0]), int(v[1])

    def kernel_ms(self):
        """(extension ms, alignment ms) of the last batch (CUDA events)."""
        v = (ctypes.c_float * 2)()
        _check(self.lib.pg_kernel_ms(self.h, v))
        return float(v[0]), float(v[1])

    def set_seqs_fasta(self, side, fasta, k=6):
        """Parse FASTA text (bytes) on the GPU into one side; returns
        (kept record indices, removed count)."""
        fasta = bytes(fasta)
        nk, nrm = ctypes.c_uint64(), ctypes.c_uint64()
        cap = fasta.count(b">") + 1
        orig = np.zeros(cap, dtype=np.uint64)
        _check(self.lib.pg_set_seqs_fasta(self.h, side, fasta, len(fasta), k, ctypes.byref(nk),
                                          ctypes.byref(nrm), orig.ctypes.data, cap))
        return orig[:nk.value].copy(), int(nrm.value)

    def get_seqs(self, side):
        """(residue codes, offsets) resident for one side."""
        n, tot = ctypes.c_uint64(), ctypes.c_uint64()
        _check(self.lib.pg_get_seqs(self.h, side, None, None, ctypes.byref(n), ctypes.byref(tot)))
        codes = np.zeros(max(1, tot.value), dtype=np.uint8)
        offs = np.zeros(n.value + 1, dtype=np.uint64)
        _check(self.lib.pg_get_seqs(self.h, side, codes.ctypes.data, offs.ctypes.data, None,
                                    None))
        return codes[:tot.value], offs

    def candidates_device(self, kc, rows, cols, d_out, cap, stream=None):
        """Candidate pairs of the block rows x cols (ranges) into a device
        buffer; returns how many were written."""
        n = ctypes.c_uint64()
        _check(self.lib.pg_candidates(self.h, ctypes.byref(kc), rows[0], rows[1], cols[0], cols[1],
                                      d_out, cap, ctypes.byref(n), stream))
        return int(n.value)

    def candidates(self, kc, rows, cols):
        """The same into host memory (sizes the output with a first call)."""
        import torch
        dev = self.cfg.device
        n = ctypes.c_uint64()
        rc = self.lib.pg_candidates(self.h, ctypes.byref(kc), rows[0], rows[1], cols[0], cols[1],
                                    None, 0, ctypes.byref(n), None)
        if rc not in (PG_OK, PG_ERR_RANGE) or (rc == PG_ERR_RANGE and n.value == 0):
            _check(rc)
        cnt = int(n.value)
        if cnt == 0:
            return np.zeros(0, dtype=PAIR_DTYPE)
        buf = torch.empty(cnt * PAIR_DTYPE.itemsize, dtype=torch.uint8, device="cuda:%d" % dev)
        got = self.candidates_device(kc, rows, cols, buf.data_ptr(), cnt)
        return np.frombuffer(buf[:got * PAIR_DTYPE.itemsize].cpu().numpy().tobytes(),
                             dtype=PAIR_DTYPE).copy()

    def get_tuning(self):
        t = Tuning()
        _check(self.lib.pg_get_tuning(self.h, ctypes.byref(t)))
        return t

    def set_tuning(self, t=None, **fields):
        """Set a Tuning, or change the named fields of the current one."""
        if t is None:
            t = self.get_tuning()
        for k, v in fields.items():
            setattr(t, k, int(v))
        _check(self.lib.pg_set_tuning(self.h, ctypes.byref(t)))
        return t


ALIGN_CB = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64,
                            ctypes.c_uint64, ctypes.POINTER(ctypes.c_float), ctypes.c_void_p)
BATCH_CB = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                            ctypes.c_void_p)


class BatchCtl(ctypes.Structure):
    """pgh_batch_ctl: batch-level resume of pw_aln_batch."""
    _fields_ = [("start_batch", ctypes.c_uint64), ("next_batch", ctypes.c_uint64),
                ("last_end", ctypes.c_uint64), ("complete", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class BatchError(RuntimeError):
    """A batch of pw_aln_batch failed.  ``code`` is its PG_ERR_* code and
    ``partial`` the (rows, cols, vals, stats) the driver wrote back: the
    triples after the k-mer prune with score_aln set for every batch before
    stats["next_batch"], ready to resume from there."""

    def __init__(self, code, detail, partial):
        super().__init__("pw_aln_batch failed (%d): %s" % (code, detail))
        self.code = code
        self.partial = partial


def pw_aln_batch(mode, rows, cols, vals, row_res, row_offs, col_res=None, col_offs=None,
                 bl_roff=0, bl_coff=0, batch_sz=10 ** 10, ckthr=0, mosthr=-1.0, cfg=None,
                 callback=None, start_batch=0, on_batch=None):
    """Run the C++ pw_aln_batch driver (src/DistPWRunner.cpp:25-165) on one block.

    vals is a KMERLOC_DTYPE (X-drop) or KMERLIGHT_DTYPE (SW) array.  With
    ``callback(pairs, bl_roff, bl_coff) -> score_aln array`` the driver uses it
    as the aligner instead of the GPU (raising in it fails the batch with
    PG_ERR_STATE; returning an int < 0 fails it with that code).  Batch-level
    resume: ``start_batch`` skips the batches before it, and
    ``on_batch(batch, beg, end) -> bool`` is called after each batch, False
    stopping the run there.  Returns (rows, cols, vals, stats); stats holds
    next_batch, last_end and complete.  A failed batch raises BatchError."""
    lib = load("libpastis_host.so")
    rows = np.array(rows, dtype=np.uint64)
    cols = np.array(cols, dtype=np.uint64)
    vals = np.array(vals, dtype=KMERLOC_DTYPE if mode == MODE_XDROP else KMERLIGHT_DTYPE)
    rres = np.ascontiguousarray(row_res, dtype=np.uint8)
    roffs = np.ascontiguousarray(row_offs, dtype=np.uint64)
    if col_res is not None:
        cres = np.ascontiguousarray(col_res, dtype=np.uint8)
        coffs = np.ascontiguousarray(col_offs, dtype=np.uint64)
        cres_p, coffs_p, nc = cres.ctypes.data, coffs.ctypes.data, len(coffs) - 1
    else:
        cres_p, coffs_p, nc = None, None, 0
    stats = np.zeros(5, dtype=np.uint64)
    secs = np.zeros(4, dtype=np.float64)
    cb = None
    if callback is not None:
        def _cb(pp, n, ro, co, out, user):
            try:
                arr = np.ctypeslib.as_array((ctypes.c_char * (n * PAIR_DTYPE.itemsize))
                                            .from_address(pp)).view(PAIR_DTYPE).copy()
                r = callback(arr, ro, co)
                if isinstance(r, int):
                    return r if r < 0 else 1
                s = np.ascontiguousarray(r, dtype=np.float32)
                ctypes.memmove(out, s.ctypes.data, 4 * n)
                return 0
            except Exception:
                return 1
        cb = ALIGN_CB(_cb)
    bcb = None
    if on_batch is not None:
        def _bcb(b, beg, end, user):
            try:
                return 0 if on_batch(int(b), int(beg), int(end)) else 1
            except Exception:
                return 1
        bcb = BATCH_CB(_bcb)
    ctl = BatchCtl()
    ctl.start_batch = start_batch
    c = cfg if cfg is not None else config(mode)
    vp, u64 = ctypes.c_void_p, ctypes.c_uint64
    rc = lib.pgh_pw_aln_batch_resume(
        ctypes.c_int(mode), ctypes.byref(c), vp(rres.ctypes.data), vp(roffs.ctypes.data),
        u64(len(roffs) - 1), vp(cres_p), vp(coffs_p), u64(nc), u64(len(vals)),
        vp(rows.ctypes.data), vp(cols.ctypes.data), vp(vals.ctypes.data), u64(bl_roff),
        u64(bl_coff), u64(batch_sz), ctypes.c_int(ckthr), ctypes.c_float(mosthr), cb, None,
        vp(stats.ctypes.data), vp(secs.ctypes.data), ctypes.byref(ctl), bcb, None)
    k = int(stats[2])
    st = {"nnz_in": int(stats[0]), "nnz_kmer_thr": int(stats[1]), "nnz_aln": int(stats[2]),
          "batches": int(stats[3]), "empty_batches": int(stats[4]),
          "next_batch": int(ctl.next_batch), "last_end": int(ctl.last_end),
          "complete": bool(ctl.complete),
          "seconds": {"align|pre": secs[0], "align|gpu": secs[1], "align|post": secs[2],
                      "align": secs[3]}}
    if rc != PG_OK:
        raise BatchError(rc, lib.pgh_last_error().decode(errors="replace"),
                         (rows[:k], cols[:k], vals[:k], st))
    return rows[:k], cols[:k], vals[:k], st
