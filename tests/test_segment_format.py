"""Segment images (CPU only): the restated writer's images read back through a
plain Python restatement of thinDB's block decoding, and the library's
segment walker rejects malformed or unsupported images before any device
work (segment_reader.zig decodeColumnPayload :1730, forBlockOf :1809,
rleBlockOf :2098)."""
import struct

import numpy as np
import pytest

from golden.segments import ENC_FOR, ENC_RAW, ENC_RLE, NATIVE, write_segment
from thindb_gb300 import abi
from thindb_gb300.engine import Column, EngineError, Table


def read_segment(image: bytes, types):
    """Values and validity per column (NOT NULL columns: validity None)."""
    assert image[:4] == b"tDBS" and image[-4:] == b"tDBS"
    n = struct.unpack_from("<Q", image, 24)[0]
    vals = [[] for _ in types]
    valid = [[] for _ in types]
    nullable = [False] * len(types)
    pos, done, encs = 32, 0, []
    while done < n:
        rows = struct.unpack_from("<I", image, pos)[0]
        pos += 8
        for c, ty in enumerate(types):
            comp, flags, enc, _, usize, ssize = struct.unpack_from("<BBBBII", image, pos)
            assert comp == 0 and usize == ssize
            p = image[pos + 12:pos + 12 + ssize]
            pos += 12 + ssize
            encs.append(enc)
            dt = np.dtype(NATIVE[ty]).newbyteorder("<")
            off = 0
            if flags & 1:
                nullable[c] = True
                bm = np.frombuffer(p, np.uint8, (rows + 7) // 8)
                valid[c].append(np.unpackbits(bm, bitorder="little")[:rows].astype(bool))
                off = (rows + 7) // 8
            else:
                valid[c].append(np.ones(rows, bool))
            if enc == ENC_RAW:
                v = np.frombuffer(p, dt, rows, off)
            elif enc == ENC_FOR:
                base = int.from_bytes(p[off:off + 16], "little", signed=True)
                w = p[off + 16]
                codes = np.frombuffer(p, np.dtype(f"<u{w}") if w > 1 else np.uint8, rows, off + 20)
                v = np.array([(base + int(x)) for x in codes], dtype=object)
                bits = 8 * dt.itemsize
                v = np.array([((x + (1 << bits)) % (1 << bits)) for x in v], dtype=np.uint64)
                v = v.astype(f"<u{dt.itemsize}").view(dt)
            else:
                assert enc == ENC_RLE
                runs = struct.unpack_from("<I", p, off)[0]
                w = p[off + 4]
                rv = np.frombuffer(p, np.dtype(NATIVE[ty]).newbyteorder("<"), runs, off + 8)
                rl = np.frombuffer(p, "<u4", runs, off + 8 + runs * w)
                v = np.repeat(rv, rl)
            vals[c].append(v)
        done += rows
    return ([np.concatenate(v) for v in vals], [np.concatenate(v) if nb else None for v, nb in zip(valid, nullable)],
            encs)


def check_round_trip(types, values, validity, **kw):
    image, _ = write_segment(types, values, validity, **kw)
    got, ok, encs = read_segment(image, types)
    for c in range(len(types)):
        want_ok = np.ones(len(values[c]), bool) if validity[c] is None else np.asarray(validity[c])
        if validity[c] is None:
            assert ok[c] is None
        else:
            assert np.array_equal(ok[c], want_ok)
        w = np.asarray(values[c], NATIVE[types[c]])
        assert np.array_equal(got[c][want_ok], w[want_ok])
    return encs


def test_writer_picks_rle_for_runs_for_for_narrow_ranges_raw_otherwise():
    rng = np.random.default_rng(3)
    n = 10_000
    runny = np.repeat(rng.integers(-9, 9, 100), 100).astype(np.int64)
    narrow = (1_000_000 + rng.integers(0, 200, n)).astype(np.int64)
    wide = rng.integers(-2**62, 2**62, n).astype(np.int64)
    flt = rng.random(n)
    tiny = rng.integers(-128, 127, n).astype(np.int8)
    types = [abi.BIGINT, abi.BIGINT, abi.BIGINT, abi.DOUBLE, abi.TINYINT]
    encs = check_round_trip(types, [runny, narrow, wide, flt, tiny], [None] * 5, row_group_rows=n)
    assert encs == [ENC_RLE, ENC_FOR, ENC_RAW, ENC_RAW, ENC_RAW]


@pytest.mark.parametrize("encoding", [None, "raw", "for", "for8", "rle"])
def test_round_trip_each_encoding_with_nulls_and_a_partial_last_group(encoding):
    rng = np.random.default_rng(4)
    n = 5_003
    types = [abi.INT, abi.SMALLINT, abi.DATE, abi.DATETIME, abi.DECIMAL64, abi.BOOLEAN]
    values = [rng.integers(-5, 5, n).astype(np.int32), rng.integers(-30000, 30000, n).astype(np.int16),
              np.repeat(rng.integers(18000, 20000, n // 7 + 1), 7)[:n].astype(np.int32),
              rng.integers(0, 2**40, n).astype(np.int64), rng.integers(-10**12, 10**12, n).astype(np.int64),
              (rng.random(n) > 0.5).astype(np.uint8)]
    validity = [rng.random(n) > 0.1, None, rng.random(n) > 0.5, None, rng.random(n) > 0.3, None]
    check_round_trip(types, values, validity, row_group_rows=1024, encoding=encoding)


def test_for_clamps_null_placeholders_outside_the_range():
    v = np.array([5, -2**63, 7, 2**63 - 1, 6], np.int64)
    ok = np.array([True, False, True, False, True])
    check_round_trip([abi.BIGINT], [v], [ok], encoding="for")


def register(image, types):
    cols = [Column(f"c{i}", t, None) for i, t in enumerate(types)]
    return Table.from_segment(image, cols)


def good_image():
    v = np.arange(300, dtype=np.int64) // 7
    return write_segment([abi.BIGINT, abi.INT], [v, v.astype(np.int32)], [None, v % 5 != 0], row_group_rows=128)


def patched(image: bytes, at: int, data: bytes) -> bytes:
    b = bytearray(image)
    b[at:at + len(data)] = data
    return bytes(b)


@pytest.mark.parametrize("what", ["magic", "tail_magic", "truncated", "block_size", "rg_rows", "for_width",
                                  "rle_lengths"])
def test_malformed_images_are_invalid(what):
    image, heads = good_image()
    types = [abi.BIGINT, abi.INT]
    if what == "magic":
        image = b"XDBS" + image[4:]
    elif what == "tail_magic":
        image = image[:-4] + b"tDBX"
    elif what == "truncated":
        image = image[:200] + image[-8:]
    elif what == "block_size":
        image = patched(image, heads[0] + 8, struct.pack("<I", 1 << 30))
        image = patched(image, heads[0] + 4, struct.pack("<I", 1 << 30))
    elif what == "rg_rows":
        image = patched(image, 32, struct.pack("<I", 10_000))
    elif what in ("for_width", "rle_lengths"):
        image, heads = write_segment(types, [np.arange(300, dtype=np.int64) // (1 if what == "for_width" else 50),
                                             np.zeros(300, np.int32)], [None, None], row_group_rows=300,
                                     encoding="for" if what == "for_width" else "rle")
        if what == "for_width":
            image = patched(image, heads[0] + 12 + 16, bytes([3]))
        else:
            image = patched(image, heads[0] + 12 + 8 + 6 * 8, struct.pack("<I", 51))
    with pytest.raises(EngineError) as e:
        register(image, types)
    assert e.value.status == abi.ERR_INVALID_ARGUMENT, str(e.value)


@pytest.mark.parametrize("what", ["zstd", "lz4", "int_streams", "dict", "fsst", "version", "string_column"])
def test_unsupported_blocks_are_reported(what):
    image, heads = good_image()
    types = [abi.BIGINT, abi.INT]
    if what in ("zstd", "lz4"):
        image = patched(image, heads[1], bytes([1 if what == "zstd" else 2]))
    elif what == "int_streams":
        image = patched(image, heads[1] + 1, bytes([3]))
    elif what in ("dict", "fsst"):
        image = patched(image, heads[0] + 2, bytes([2 if what == "dict" else 4]))
    elif what == "version":
        image = patched(image, 4, struct.pack("<H", 8))
    else:
        types = [abi.VARCHAR, abi.INT]
    with pytest.raises(EngineError) as e:
        register(image, types)
    assert e.value.status == abi.ERR_UNSUPPORTED_TYPE, str(e.value)


@pytest.mark.parametrize("encoding", [None, "raw", "for", "for8", "rle"])
@pytest.mark.parametrize("rg", [1024, 1000])
def test_oracle_decode_matches_the_writer_input(encoding, rg):
    import oracle
    rng = np.random.default_rng(5)
    n = 7_777
    types = [abi.INT, abi.BIGINT, abi.DOUBLE, abi.TINYINT, abi.DATETIME]
    values = [np.repeat(rng.integers(-3, 3, n // 10 + 1), 10)[:n].astype(np.int32),
              rng.integers(-2**63, 2**63 - 1, n, dtype=np.int64), rng.random(n),
              rng.integers(-128, 127, n).astype(np.int8), (10**12 + rng.integers(0, 10**6, n)).astype(np.int64)]
    validity = [rng.random(n) > 0.3, None, rng.random(n) > 0.5, rng.random(n) > 0.9, None]
    image, _ = write_segment(types, values, validity, row_group_rows=rg, encoding=encoding)
    for threads in (1, 4):
        got = oracle.decode_segment(image, types, [v is not None for v in validity], threads=threads)
        for c, (vals, ok) in enumerate(got):
            want_ok = np.ones(n, bool) if validity[c] is None else validity[c]
            if validity[c] is None:
                assert ok is None
            else:
                assert np.array_equal(ok, want_ok)
            assert np.array_equal(vals[want_ok], np.asarray(values[c])[want_ok])


def test_replicated_image_repeats_the_rows():
    import oracle
    from golden.segments import replicate, sample_table
    names, types, values, validity = sample_table(3_000)
    image, _ = write_segment(types, values, validity, row_group_rows=1024)
    big = replicate(image, len(types), 3)
    got = oracle.decode_segment(big, types, [v is not None for v in validity])
    for c, (vals, ok) in enumerate(got):
        want_ok = np.ones(3_000, bool) if validity[c] is None else validity[c]
        okr = np.tile(want_ok, 3)
        assert np.array_equal(vals[okr], np.tile(values[c], 3)[okr])
        if validity[c] is not None:
            assert np.array_equal(ok, okr)
    # the footer's size and trailing magic
    assert big[-4:] == b"tDBS"
    fsize = struct.unpack_from("<I", big, len(big) - 8)[0]
    assert struct.unpack_from("<I", big, len(big) - fsize)[0] == 9  # row groups: 3 x 3


def _rows_equal(dec, values, validity):
    for c, (vals, ok) in enumerate(dec):
        want = np.asarray(values[c])
        mask = np.ones(want.size, bool) if validity[c] is None else validity[c]
        if validity[c] is None:
            assert ok is None
        else:
            assert np.array_equal(ok, mask), c
        assert np.array_equal(vals[mask], want[mask]), c


def test_reference_for_table_round_trips():
    """for_encoding_test.zig:8-48: 2,500 rows in 256-row groups; `k` (200
    values above 1,000,000) and `neg` (a negative base, both bounds present)
    narrow to FOR, `wide` cannot narrow and stays raw, `solo` is one value,
    `maybe_null` is NULL every 4th row; every value decodes exactly."""
    import oracle
    i = np.arange(2500, dtype=np.int64)
    neg = -30_000 + (i * 7) % 5_001
    neg[0], neg[1] = -30_000, -25_000
    types = [abi.BIGINT, abi.BIGINT, abi.BIGINT, abi.BIGINT, abi.INT]
    values = [1_000_000 + i % 200, neg, (i * 2_400_000_000_007) % (2**63 - 1), np.full(2500, 12_345, np.int64),
              (500 + i % 50).astype(np.int32)]
    validity = [None, None, None, None, i % 4 != 0]
    image, _ = write_segment(types, values, validity, row_group_rows=256)
    _, _, encs = read_segment(image, types)
    enc = np.array(encs).reshape(-1, len(types))
    assert (enc[:, 0] == ENC_FOR).all() and (enc[:, 1] == ENC_FOR).all() and (enc[:, 2] == ENC_RAW).all()
    assert (enc[:, 4] == ENC_FOR).all()
    _rows_equal(oracle.decode_segment(image, types, [v is not None for v in validity]), values, validity)


def test_reference_rle_table_known_answers():
    """rle_encoding_test.zig:17-45, :128-166: 2,500 rows in 256-row groups;
    the long-run columns take RLE (runs straddle row groups), the alternating
    one does not; every value decodes exactly and the test's aggregates over
    the decoded table hold."""
    import oracle
    from thindb_gb300.engine import AggSpec, Pred, Request
    i = np.arange(2500, dtype=np.int64)
    types = [abi.BIGINT, abi.TINYINT, abi.INT, abi.BIGINT]
    values = [7_000_000_000 + i // 100, np.where(i % 250 == 249, 1, 0).astype(np.int8),
              (100 + i % 2).astype(np.int32), 40_000 + i // 50]
    validity = [None, None, None, i % 4 != 0]
    image, _ = write_segment(types, values, validity, row_group_rows=256)
    _, _, encs = read_segment(image, types)
    enc = np.array(encs).reshape(-1, len(types))
    assert (enc[:, 0] == ENC_RLE).all() and (enc[:, 1] == ENC_RLE).all() and (enc[:, 2] != ENC_RLE).all()
    dec = oracle.decode_segment(image, types, [v is not None for v in validity])
    _rows_equal(dec, values, validity)
    cols = [Column("runs", abi.BIGINT, dec[0][0]), Column("flag", abi.TINYINT, dec[1][0]),
            Column("alt", abi.INT, dec[2][0]), Column("runs_null", abi.BIGINT, dec[3][0], validity=dec[3][1])]
    t = oracle.HostTable(cols)

    def count(where):
        return int(oracle.run(t, Request([], [AggSpec("count", None, "c")], where=[where]))["c"][0][0])

    assert count(Pred("runs", "=", 7_000_000_003)) == 100
    assert count(Pred("flag", "!=", 0)) == 10
    assert count(Pred("flag", "=", 0)) == 2490
    assert count(Pred("runs", ">", 7_000_000_010)) == 1400
    assert count(Pred("runs", "<=", 7_000_000_010)) == 1100
    sums = oracle.run(t, Request([], [AggSpec("sum", "flag", "f"), AggSpec("sum", "runs", "r")]))
    assert int(sums["f"][0][0]) == 10
    assert int(sums["r"][0][0]) == sum(7_000_000_000 + k // 100 for k in range(2500))
