"""Seeded synthetic workloads (the stand-in for the reference's FASTA input and
its k-mer SpGEMM candidate pairs), generated by libpastis_synth.so.

Workload presets follow the benchmark definitions of this stage:

  sw100k     100k pairs from 20k proteins, lognormal lengths (median 250,
             sigma 0.5, clamp 30-1000), half homologs at 30-80 % identity with
             2 % indels (geometric, mean 3), local SW
  xdrop1m    1M pairs of the same generator, up to 2 seeds = shared exact
             6-mers, X-drop x = 49
  uneven10m  10M pairs, lengths 80 % lognormal (median 300) + 20 % uniform
             1000-5000, min 20
  uneven10m_sw  the same batch, aligned by local Smith-Waterman
  filter5m   5M pairs of the sw100k generator at a 30 % homolog rate (the
             learned filter's training and evaluation set)
  manytomany 1M proteins in families of 2-50 at 30-90 % identity; its
             candidate pairs come from the GPU k-mer SpGEMM, not the generator
"""
import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import records


def declare(lib):
    """Argument and return types of libpastis_synth.so's entry points."""
    vp, u64 = ctypes.c_void_p, ctypes.c_uint64
    lib.pg_synth_generate.argtypes = [vp]
    lib.pg_synth_generate.restype = vp
    for f in ("pg_synth_nseqs", "pg_synth_nres", "pg_synth_npairs"):
        getattr(lib, f).argtypes = [vp]
        getattr(lib, f).restype = u64
    for f in ("pg_synth_seq", "pg_synth_offs", "pg_synth_family", "pg_synth_pairs",
              "pg_synth_homolog", "pg_synth_spurious"):
        getattr(lib, f).argtypes = [vp]
        getattr(lib, f).restype = vp
    lib.pg_synth_free.argtypes = [vp]
    lib.pg_synth_free.restype = None


_lib = None


def _synth_lib():
    """The generator's own library (no CUDA library is loaded for it)."""
    global _lib
    if _lib is None:
        lib = records.cdll("libpastis_synth.so")
        declare(lib)
        _lib = lib
    return _lib


class SynthCfg(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint64), ("nseqs", ctypes.c_uint64),
                ("fam_min", ctypes.c_uint32), ("fam_max", ctypes.c_uint32),
                ("len_median", ctypes.c_double), ("len_sigma", ctypes.c_double),
                ("len_min", ctypes.c_uint32), ("len_max", ctypes.c_uint32),
                ("mix_frac", ctypes.c_double), ("mix_lo", ctypes.c_uint32),
                ("mix_hi", ctypes.c_uint32), ("id_lo", ctypes.c_double),
                ("id_hi", ctypes.c_double), ("indel_rate", ctypes.c_double),
                ("indel_mean", ctypes.c_double), ("npairs", ctypes.c_uint64),
                ("homolog_frac", ctypes.c_double), ("k", ctypes.c_uint32),
                ("alph", ctypes.c_int32)]


@dataclass
class Workload:
    name: str
    seq: np.ndarray          # residue codes (0..19), concatenated
    offs: np.ndarray         # uint64, nseqs + 1
    pairs: np.ndarray        # records.PAIR_DTYPE
    homolog: np.ndarray      # uint8 per pair
    spurious: np.ndarray     # uint8 per pair: no shared k-mer, random seed
    family: np.ndarray
    params: dict = field(default_factory=dict)

    @property
    def ascii(self):
        return records.decode(self.seq)

    def lengths(self):
        return np.diff(self.offs).astype(np.int64)

    def sw_cells(self):
        L = self.lengths()
        return int((L[self.pairs["row"]] * L[self.pairs["col"]]).sum())

    def subset(self, idx):
        return Workload(self.name, self.seq, self.offs, self.pairs[idx], self.homolog[idx],
                        self.spurious[idx], self.family, dict(self.params))


PRESETS = {
    "sw100k": dict(nseqs=20_000, npairs=100_000, len_median=250.0, len_sigma=0.5, len_min=30,
                   len_max=1000, mix_frac=0.0, mix_lo=0, mix_hi=0, id_lo=0.30, id_hi=0.80,
                   homolog_frac=0.5, k=6, alph=0, fam_min=6, fam_max=6),
    "xdrop1m": dict(nseqs=200_000, npairs=1_000_000, len_median=250.0, len_sigma=0.5, len_min=30,
                    len_max=1000, mix_frac=0.0, mix_lo=0, mix_hi=0, id_lo=0.30, id_hi=0.80,
                    homolog_frac=0.5, k=6, alph=0, fam_min=6, fam_max=6),
    "uneven10m": dict(nseqs=2_000_000, npairs=10_000_000, len_median=300.0, len_sigma=0.5,
                      len_min=20, len_max=5000, mix_frac=0.2, mix_lo=1000, mix_hi=5000,
                      id_lo=0.30, id_hi=0.80, homolog_frac=0.5, k=6, alph=0, fam_min=6,
                      fam_max=6),
    # the same batch, aligned by local Smith-Waterman (the X-drop and SW
    # modes of the uneven-length workload)
    "uneven10m_sw": dict(nseqs=2_000_000, npairs=10_000_000, len_median=300.0, len_sigma=0.5,
                         len_min=20, len_max=5000, mix_frac=0.2, mix_lo=1000, mix_hi=5000,
                         id_lo=0.30, id_hi=0.80, homolog_frac=0.5, k=6, alph=0, fam_min=6,
                         fam_max=6),
    "manytomany": dict(nseqs=1_000_000, npairs=1_000, len_median=250.0, len_sigma=0.5,
                       len_min=30, len_max=1000, mix_frac=0.0, mix_lo=0, mix_hi=0, id_lo=0.30,
                       id_hi=0.90, homolog_frac=0.5, k=6, alph=0, fam_min=2, fam_max=50),
    "filter5m": dict(nseqs=1_000_000, npairs=5_000_000, len_median=250.0, len_sigma=0.5,
                     len_min=30, len_max=1000, mix_frac=0.0, mix_lo=0, mix_hi=0, id_lo=0.30,
                     id_hi=0.80, homolog_frac=0.3, k=6, alph=0, fam_min=6, fam_max=6),
}


def generate(preset="xdrop1m", seed=20260101, scale=1.0, **over):
    """Generate a workload; scale multiplies the sequence and pair counts."""
    p = dict(PRESETS[preset])
    p.update(over)
    c = SynthCfg()
    c.seed = seed
    c.nseqs = max(2, int(round(p["nseqs"] * scale)))
    c.npairs = max(1, int(round(p["npairs"] * scale)))
    for k in ("fam_min", "fam_max", "len_median", "len_sigma", "len_min", "len_max", "mix_frac",
              "mix_lo", "mix_hi", "id_lo", "id_hi", "homolog_frac", "k", "alph"):
        setattr(c, k, p[k])
    c.indel_rate = p.get("indel_rate", 0.02)
    c.indel_mean = p.get("indel_mean", 3.0)
    lib = _synth_lib()
    h = lib.pg_synth_generate(ctypes.byref(c))
    if not h:
        raise MemoryError("synthetic generator failed")
    try:
        ns, nres, npairs = lib.pg_synth_nseqs(h), lib.pg_synth_nres(h), lib.pg_synth_npairs(h)

        def arr(ptr, dtype, n):
            if n == 0:
                return np.zeros(0, dtype=dtype)
            buf = (ctypes.c_char * (n * np.dtype(dtype).itemsize)).from_address(ptr)
            return np.frombuffer(buf, dtype=dtype).copy()

        w = Workload(preset, arr(lib.pg_synth_seq(h), np.uint8, nres),
                     arr(lib.pg_synth_offs(h), np.uint64, ns + 1),
                     arr(lib.pg_synth_pairs(h), records.PAIR_DTYPE, npairs),
                     arr(lib.pg_synth_homolog(h), np.uint8, npairs),
                     arr(lib.pg_synth_spurious(h), np.uint8, npairs),
                     arr(lib.pg_synth_family(h), np.uint32, ns),
                     dict(p, seed=seed, scale=scale))
    finally:
        lib.pg_synth_free(h)
    return w
