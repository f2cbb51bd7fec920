"""The C-ABI library builds, loads and exports every symbol the header
declares; the ctypes mirror matches the header (CPU only, no compute)."""
import ctypes as C
import os
import re

import pytest

from thindb_gb300 import abi, engine

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "thindb_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^[A-Za-z_][\w \*]*?\b(tgpu_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_operator_entry_points():
    fns = declared_functions()
    for name in ("tgpu_table_register", "tgpu_query_create", "tgpu_query_next", "tgpu_query_cancel",
                 "tgpu_query_destroy", "tgpu_last_error_message"):
        assert name in fns


def test_library_exports_every_declared_symbol():
    lib = engine.lib()
    missing = [f for f in declared_functions() if not hasattr(lib, f)]
    assert not missing, missing


def test_ctypes_mirror_covers_the_header():
    mirrored = {n for n, _, _ in abi.SIGNATURES}
    assert set(declared_functions()) <= mirrored | {"tgpu_group_by_i64_noalloc"}


def test_abi_version_and_build_info():
    lib = engine.lib()
    assert lib.tgpu_abi_version() == abi.ABI_VERSION
    assert b"sm_103a" in lib.tgpu_build_info()


def test_struct_sizes_match_c_layout():
    # sizes the header implies on LP64 (both x86_64 and aarch64)
    assert C.sizeof(abi.ColumnDesc) == 64
    assert C.sizeof(abi.TableDesc) == 40
    assert C.sizeof(abi.AggSpec) == 16
    assert C.sizeof(abi.Predicate) == 40
    assert C.sizeof(abi.Request) == 136
    assert C.sizeof(abi.OutputColumn) == 80
    assert C.sizeof(abi.QueryStats) == 104
    assert C.sizeof(abi.Batch) == 40


def test_no_device_fails_loudly():
    """Without a GPU the engine refuses (no CPU fallback exists)."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    import numpy as np

    cols = [engine.Column("k", abi.BIGINT, np.arange(10, dtype=np.int64))]
    with pytest.raises(engine.EngineError) as ei:
        engine.Table(cols)
    assert ei.value.status in (abi.ERR_NO_DEVICE, abi.ERR_CUDA)
