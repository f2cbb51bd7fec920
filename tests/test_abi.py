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
    assert C.sizeof(abi.AggSpec) == 24
    assert C.sizeof(abi.Predicate) == 40
    assert C.sizeof(abi.Request) == 136
    assert C.sizeof(abi.OutputColumn) == 80
    assert C.sizeof(abi.QueryStats) == 104
    assert C.sizeof(abi.Batch) == 40
    assert C.sizeof(abi.Shape) == 32
    assert C.sizeof(abi.Tuning) == 56


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


def test_tuning_table_round_trip_and_validation():
    """tgpu_tuning_set / _get hold the table on the host (no device work)."""
    lib = engine.lib()
    saved = engine.tuning_entries()
    try:
        arr = (abi.Tuning * 2)()
        arr[0].shape.key_words, arr[0].shape.fold, arr[0].shape.groups_log2 = 1, 3, 21
        arr[0].chunk_rows, arr[0].cache_slots, arr[0].table_load_pct = 1024, -1, 25
        arr[0].flags = abi.FLAG_GATHER_SCAN
        arr[1].shape.batched, arr[1].chunk_rows = 1, 4096
        assert lib.tgpu_tuning_set(arr, 2) == abi.OK
        got = engine.tuning_entries()
        assert len(got) == 2
        assert got[0]["shape"]["groups_log2"] == 21 and got[0]["cache_slots"] == -1
        assert got[1]["shape"]["batched"] == 1 and got[1]["chunk_rows"] == 4096
        bad = (abi.Tuning * 1)()
        bad[0].chunk_rows = 300  # not a multiple of 256
        assert lib.tgpu_tuning_set(bad, 1) == abi.ERR_INVALID_ARGUMENT
        assert len(engine.tuning_entries()) == 2  # a rejected table leaves the old one
        engine.clear_tuning()
        assert engine.tuning_entries() == []
    finally:
        arr = (abi.Tuning * max(1, len(saved)))()
        lib.tgpu_tuning_set(arr, 0)
        if saved:
            import json
            import tempfile

            with tempfile.NamedTemporaryFile("w", suffix=".json", delete=False) as f:
                json.dump({"entries": saved}, f)
            engine.load_tuning(f.name)
            os.unlink(f.name)


def test_committed_tuning_table_parses():
    """The measured table that ships with the package is well formed."""
    import json

    if not os.path.exists(engine.TUNING_PATH):
        pytest.skip("no tuning table committed")
    doc = json.load(open(engine.TUNING_PATH))
    fields = {f for f, _ in abi.Shape._fields_}
    for e in doc["entries"]:
        assert set(e["shape"]) == fields
        assert e["chunk_rows"] % 256 == 0 and e["table_load_pct"] in (0, 25, 50, 70)


def test_tuning_merge_keeps_untouched_shapes():
    """--merge: a shape tuned again takes its new entry, other shapes keep
    theirs, and the provenance lists both runs."""
    from thindb_gb300.autotune import merge_tables

    def entry(groups_log2, chunk):
        shape = {f: 0 for f, _ in abi.Shape._fields_}
        shape["groups_log2"] = groups_log2
        return {"shape": shape, "chunk_rows": chunk}

    old = {"generated_by": "python -m thindb_gb300.autotune --workloads plain --reps 3", "seconds": 10.0,
           "entries": [entry(10, 512), entry(20, 1024)]}
    entries, by, seconds = merge_tables(old, [entry(20, 4096), entry(22, 2048)],
                                        "python -m thindb_gb300.autotune --workloads distinct --reps 3", 5.0)
    assert [(e["shape"]["groups_log2"], e["chunk_rows"]) for e in entries] == [(10, 512), (20, 4096), (22, 2048)]
    assert by == [old["generated_by"], "python -m thindb_gb300.autotune --workloads distinct --reps 3 --merge <this file>"]
    assert seconds == 15.0
    # a second merge appends to the list
    _, by2, _ = merge_tables({"generated_by": by, "seconds": seconds, "entries": entries}, [], "cmd", 1.0)
    assert by2[:2] == by and by2[2] == "cmd --merge <this file>"


def test_aggregate_registry_names():
    """thinDB's registerAggregate rules: case-insensitive names, built-in names
    and repeats refused (no device needed)."""
    assert not engine.aggregate_registered("geo_mean")
    engine.register_aggregate("Geo_Mean")
    try:
        assert engine.aggregate_registered("geo_mean") and engine.aggregate_registered("GEO_MEAN")
        with pytest.raises(engine.EngineError) as e:
            engine.register_aggregate("geo_mean")
        assert e.value.status == abi.ERR_INVALID_ARGUMENT
    finally:
        engine.unregister_aggregate("GEO_MEAN")
    assert not engine.aggregate_registered("geo_mean")
    for bad in ("sum", "COUNT", "", "9lives", "has space", "x" * 64):
        with pytest.raises(engine.EngineError):
            engine.register_aggregate(bad)
    with pytest.raises(engine.EngineError):
        engine.unregister_aggregate("never_registered")


def test_debug_hooks_validate_their_bounds():
    """The test hooks take effect for queries planned later and refuse values
    out of range (no device needed)."""
    for bits in (8, 63, 0):
        engine.set_digest_bits(bits)
    with pytest.raises(engine.EngineError) as e:
        engine.set_digest_bits(64)
    assert e.value.status == abi.ERR_INVALID_ARGUMENT
    engine.set_device_wait_limit(0)
    with pytest.raises(engine.EngineError):
        engine.set_device_wait_limit((1 << 40) + 1)
