"""The native libraries build, load, and export every entry point include/*.h
declares.  No compute call is made (this runs on CPU-only machines too)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    names = set(re.findall(r"\b(pgh?_[a-z0-9_]+)\s*\(", text))
    return names


def test_headers_match_exports(native):
    from pastis_gb300 import capi
    decl = (_declared("pastis_gb300.h") | _declared("pastis_gb300_synth.h")
            | _declared("pastis_gb300_host.h"))
    exported = (set(capi.EXPORTS["libpastis_gb300.so"]) | set(capi.EXPORTS["libpastis_synth.so"])
                | set(capi.EXPORTS["libpastis_host.so"]))
    assert decl == exported, (decl ^ exported)


@pytest.mark.parametrize("lib", ["libpastis_gb300.so", "libpastis_synth.so", "libpastis_host.so"])
def test_library_exports(native, lib):
    from pastis_gb300 import capi
    h = ctypes.CDLL(os.path.join(native, lib))
    for sym in capi.EXPORTS[lib]:
        assert hasattr(h, sym), sym


def test_struct_layouts(native):
    from pastis_gb300 import capi
    from oracle import oracle
    assert capi.PAIR_DTYPE == oracle.PAIR_DTYPE
    assert capi.RESULT_DTYPE == oracle.RESULT_DTYPE
    assert ctypes.sizeof(capi.Config) == 64
    assert ctypes.sizeof(capi.Tuning) == 36


def test_tuning_defaults_without_gpu(native):
    """pg_tuning_default: occupancy-limited grids, bucketed order, 8 rows per
    lane, no graph."""
    from pastis_gb300 import capi
    t = capi.default_tuning()
    assert t.as_dict() == {"dp_blocks_per_sm": 0, "xd_blocks_per_sm": 0, "bucket_order": 1,
                           "rows_max": 8, "graph": 0, "xd_int16": 0, "dp_traceback": 0,
                           "dir_arena_mb": 0, "xd_stepped": -1}


def test_defaults_and_errors_without_gpu(native):
    """pg_config_default mirrors PASTIS's defaults; error strings are defined."""
    from pastis_gb300 import capi
    lib = capi.load()
    c = capi.config(capi.MODE_XDROP)
    assert (c.gap_open, c.gap_ext, c.xdrop, c.seed_len, c.seed_count) == (-11, -2, 49, 6, 2)
    assert (c.ani_thr, c.cov_thr) == (30, 0.7)
    for code in range(0, -8, -1):
        assert lib.pg_strerror(code)
    assert b"sm_103a" in lib.pg_version()
    # the resolved gap model for the reference's constructor order
    assert capi.resolved_gaps(c) == (-2, -11, -11)
    c.gap_semantics = capi.GAPS_NOMINAL
    assert capi.resolved_gaps(c) == (-11, -2, -2)


def test_create_rejects_bad_config(native):
    from pastis_gb300 import capi
    lib = capi.load()
    h = ctypes.c_void_p()
    for field, val in (("mode", 7), ("tie", 9), ("xdrop", -1), ("gap_open", -5000),
                       ("seed_len", 0), ("flags", 64), ("flags", 4)):
        c = capi.config(capi.MODE_XDROP)
        setattr(c, field, val)
        assert lib.pg_create(ctypes.byref(c), ctypes.byref(h)) == capi.PG_ERR_ARG, field
    # the two defined flags pass validation (and then find no device here)
    c = capi.config(capi.MODE_XDROP, flags=capi.F_SKIP_SPURIOUS_SEED | capi.F_XDROP_AFFINE)
    rc = lib.pg_create(ctypes.byref(c), ctypes.byref(h))
    assert rc != capi.PG_ERR_ARG
    if rc == capi.PG_OK:
        lib.pg_destroy(h)


def test_noalloc_argument_checks_without_gpu(native):
    """pg_align_sw_noalloc rejects a batch its 32-bit work counter cannot
    index, and a column bound over 65535, before it touches a device."""
    from pastis_gb300 import capi
    lib = capi.load()
    cfg = capi.config(capi.MODE_SW)
    fake = 4096    # never dereferenced: the checks come first

    def call(max_col, n):
        return lib.pg_align_sw_noalloc(ctypes.byref(cfg), fake, fake, 1, fake, fake, 1, max_col,
                                       fake, n, 0, 0, fake, None)

    assert call(100, 1 << 31) == capi.PG_ERR_ARG
    assert call(65536, 10) == capi.PG_ERR_RANGE
    assert call(100, 0) == capi.PG_OK
