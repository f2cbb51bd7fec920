"""Test infrastructure: a restatement of thinDB's segment writer, so the
segment reader can be checked on images laid out as thinDB writes them.

Layout (thinDB src/storage/format.zig:1-38, version 17 at :85):
  header   "tDBS", u16 version, u16 flags (0), u64 schema fingerprint,
           u64 segment id, u64 row count                          (32 bytes)
  row groups, each: u32 row count, u32 padding, then per column a 12-byte
           block header (u8 compression, u8 flags: bit 0 has_nulls, bit 1
           int_streams; u8 encoding, u8 reserved, u32 uncompressed size,
           u32 stored size; format.zig:201-228) and the payload
  footer   u32 row-group count; per row group u64 offset, u32 length, u32 row
           count, 56 bytes of statistics per column, a u64 block offset per
           column, a u32 block length per column; u32 string-table count; u32
           footer size (itself and the trailing magic included); "tDBS"

Payload (segment_writer.zig writeColumnBlock :1141-1188): a nullable column
prefixes every block with its validity bitmap (bit set = value,
writeValidityBitmap :1839), then one of
  RLE (rleEncode :1289): u32 runs, u8 value width (the native width), 3 pad,
      run values, u32 run lengths — chosen only when smaller than both raw and
      this block's FOR body; NULL placeholders are part of the runs;
  FOR (forEncode :1408): i128 base (the minimum non-null value), u8 width
      (the narrowest of 1/2/4/8 holding max - base, taken only below the
      native width and when the body is smaller than raw), 3 pad, one LE
      delta per row (NULL rows 0, out-of-range placeholders clamped);
  raw: the native little-endian values.
Only integer-family columns (BOOLEAN, TINYINT, SMALLINT, INT, DATE, BIGINT,
DATETIME, DECIMAL64) take RLE; FOR also skips 1-byte types.  The footer's
statistics are written as zeros here: the reader under test does not use them.

`encoding` forces one encoding for every integer column's blocks (e.g. FOR
width 8, which thinDB's writer never picks) so each decoder branch is reached;
FLOAT and DOUBLE blocks stay raw.
"""
from __future__ import annotations

import struct
from typing import Optional, Sequence

import numpy as np

from thindb_gb300 import abi

NATIVE = {abi.BOOLEAN: np.uint8, abi.TINYINT: np.int8, abi.SMALLINT: np.int16, abi.INT: np.int32,
          abi.DATE: np.int32, abi.BIGINT: np.int64, abi.DATETIME: np.int64, abi.DECIMAL64: np.int64,
          abi.FLOAT: np.float32, abi.DOUBLE: np.float64}
INTEGER = {abi.BOOLEAN, abi.TINYINT, abi.SMALLINT, abi.INT, abi.DATE, abi.BIGINT, abi.DATETIME, abi.DECIMAL64}
ENC_RAW, ENC_FOR, ENC_RLE = 0, 1, 3
FOOTER_STATS_BYTES = 56


def _for_width(span: int) -> int:
    return 1 if span <= 0xFF else 2 if span <= 0xFFFF else 4 if span <= 0xFFFFFFFF else 8


def _runs(vals: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Run values and lengths of the stored stream (placeholders included)."""
    if vals.size == 0:
        return vals[:0], np.zeros(0, np.uint32)
    change = np.flatnonzero(vals[1:] != vals[:-1]) + 1
    starts = np.concatenate(([0], change))
    lens = np.diff(np.concatenate((starts, [vals.size]))).astype(np.uint32)
    return vals[starts], lens


def _for_body(vals: np.ndarray, valid: np.ndarray, width: Optional[int] = None) -> Optional[bytes]:
    if not valid.any():
        if width is None:
            return None                     # all-null block: stays raw
        lo, hi = 0, 0
    else:
        live = vals[valid].astype(np.int64)
        lo, hi = int(live.min()), int(live.max())
    span = hi - lo
    w = width or _for_width(span)
    if width is None and w >= vals.dtype.itemsize:
        return None
    # v - lo in [0, span] fits u64 for every in-range value; the subtraction wraps mod 2^64
    wide = vals.astype(np.int64)
    deltas = wide.view(np.uint64) - np.uint64(lo & 0xFFFFFFFFFFFFFFFF)
    deltas = np.where(~valid | (wide < lo), np.uint64(0), deltas)
    deltas = np.where(valid & (wide > hi), np.uint64(span), deltas)
    codes = (deltas & np.uint64((1 << (8 * w)) - 1 if w < 8 else 0xFFFFFFFFFFFFFFFF)).astype(
        f"<u{w}" if w > 1 else np.uint8)
    return lo.to_bytes(16, "little", signed=True) + bytes([w, 0, 0, 0]) + codes.tobytes()


def _rle_body(vals: np.ndarray) -> bytes:
    rv, rl = _runs(vals)
    return (struct.pack("<I", rv.size) + bytes([vals.dtype.itemsize, 0, 0, 0]) +
            rv.astype(vals.dtype.newbyteorder("<")).tobytes() + rl.astype("<u4").tobytes())


def encode_block(ty: int, vals: np.ndarray, valid: np.ndarray, nullable: bool,
                 encoding: Optional[str] = None) -> tuple[int, bytes]:
    """(encoding byte, payload) for one column block, choosing as
    writeColumnBlock does unless `encoding` forces "raw" / "for" / "for8" /
    "rle"."""
    vals = np.ascontiguousarray(vals, dtype=NATIVE[ty])
    n = vals.size
    native = vals.dtype.itemsize
    head = np.packbits(valid, bitorder="little").tobytes() if nullable else b""
    raw = vals.astype(vals.dtype.newbyteorder("<")).tobytes()
    if encoding == "raw" or ty not in INTEGER:
        return ENC_RAW, head + raw
    if encoding == "rle":
        return ENC_RLE, head + _rle_body(vals)
    if encoding in ("for", "for8"):
        return ENC_FOR, head + _for_body(vals, valid, 8 if encoding == "for8" else
                                         _for_width(_span(vals, valid)))
    if ty in INTEGER and n:
        nruns = _runs(vals)[0].size
        rle_size = 8 + nruns * (native + 4)
        if rle_size < n * native:
            fb = _for_body(vals, valid) if native > 1 else None
            if fb is None or rle_size < len(fb):
                return ENC_RLE, head + _rle_body(vals)
        if native > 1:
            fb = _for_body(vals, valid)
            if fb is not None and len(fb) < n * native:
                return ENC_FOR, head + fb
    return ENC_RAW, head + raw


def _span(vals: np.ndarray, valid: np.ndarray) -> int:
    if not valid.any():
        return 0
    live = vals[valid].astype(np.int64)
    return int(live.max()) - int(live.min())


def write_segment(types: Sequence[int], values: Sequence[np.ndarray],
                  validity: Sequence[Optional[np.ndarray]], row_group_rows: int = 65536,
                  version: int = 17, segment_id: int = 1, encoding: Optional[str] = None,
                  fingerprint: int = 0x5EED) -> tuple[bytes, list[int]]:
    """A segment image of the columns (`validity[c]` None = NOT NULL) and the
    byte offset of every block header, row group by row group."""
    n = int(values[0].size) if len(values) else 0
    out = bytearray(b"tDBS" + struct.pack("<HHQQQ", version, 0, fingerprint, segment_id, n))
    headers: list[int] = []
    groups = []
    for r0 in range(0, n, row_group_rows):
        r1 = min(n, r0 + row_group_rows)
        g0 = len(out)
        out += struct.pack("<II", r1 - r0, 0)
        offs, lens = [], []
        for c, ty in enumerate(types):
            vals = np.asarray(values[c])[r0:r1]
            valid = (np.ones(r1 - r0, bool) if validity[c] is None
                     else np.asarray(validity[c], bool)[r0:r1])
            enc, payload = encode_block(ty, vals, valid, validity[c] is not None, encoding)
            headers.append(len(out))
            offs.append(len(out))
            flags = 1 if validity[c] is not None else 0
            out += struct.pack("<BBBBII", 0, flags, enc, 0, len(payload), len(payload)) + payload
            lens.append(len(out) - offs[-1])
        groups.append((g0, len(out) - g0, r1 - r0, offs, lens))
    return bytes(out + _footer(groups, len(types))), headers


def _footer(groups, n_cols: int) -> bytes:
    foot = bytearray(struct.pack("<I", len(groups)))
    for g0, glen, grows, offs, lens in groups:
        foot += struct.pack("<QII", g0, glen, grows)
        foot += bytes(FOOTER_STATS_BYTES * n_cols)
        foot += b"".join(struct.pack("<Q", o) for o in offs)
        foot += b"".join(struct.pack("<I", ln) for ln in lens)
    foot += struct.pack("<I", 0)                      # no string tables
    foot += struct.pack("<I", len(foot) + 8) + b"tDBS"
    return bytes(foot)


def _groups(image: bytes, n_cols: int) -> list:
    """(offset, length, rows, block offsets, block lengths) of every row group."""
    n = struct.unpack_from("<Q", image, 24)[0]
    pos, done, groups = 32, 0, []
    while done < n:
        g0 = pos
        rows = struct.unpack_from("<I", image, pos)[0]
        pos += 8
        offs, lens = [], []
        for _ in range(n_cols):
            size = struct.unpack_from("<I", image, pos + 8)[0]
            offs.append(pos)
            lens.append(12 + size)
            pos += 12 + size
        groups.append((g0, pos - g0, rows, offs, lens))
        done += rows
    return groups


def replicate(image: bytes, n_cols: int, times: int) -> bytes:
    """The segment with its row groups repeated `times` times (a large image
    from a small one; the footer is rebuilt)."""
    groups = _groups(image, n_cols)
    body = image[32:groups[-1][0] + groups[-1][1]] if groups else b""
    n = struct.unpack_from("<Q", image, 24)[0]
    head = bytearray(image[:32])
    struct.pack_into("<Q", head, 24, n * times)
    shifted = []
    for k in range(times):
        d = k * len(body)
        shifted += [(g0 + d, gl, gr, [o + d for o in offs], lens) for g0, gl, gr, offs, lens in groups]
    return bytes(head) + body * times + _footer(shifted, n_cols)


def concat(images: Sequence[bytes], n_cols: int) -> bytes:
    """One segment holding the row groups of several (same schema), in order:
    row groups of differing sizes for the reader."""
    head = bytearray(images[0][:32])
    body, groups, total = bytearray(), [], 0
    for im in images:
        gs = _groups(im, n_cols)
        if not gs:
            continue
        d = 32 + len(body) - gs[0][0]
        body += im[gs[0][0]:gs[-1][0] + gs[-1][1]]
        groups += [(g0 + d, gl, gr, [o + d for o in offs], lens) for g0, gl, gr, offs, lens in gs]
        total += struct.unpack_from("<Q", im, 24)[0]
    struct.pack_into("<Q", head, 24, total)
    return bytes(head) + bytes(body) + _footer(groups, n_cols)


def sample_table(n: int, seed: int = 7) -> tuple:
    """An eight-column table of the encodings a thinDB table stores: names,
    types, values and validity (None = NOT NULL).  region SMALLINT (runs of
    500: RLE), day DATE (sorted: RLE), user BIGINT over 50k (FOR width 2),
    amount BIGINT +-1e9 (FOR width 4), price DOUBLE (raw), flag BOOLEAN,
    tiny TINYINT (raw), cents DECIMAL64 +-1e6 (FOR width 4); day, user, price
    and tiny are nullable."""
    rng = np.random.default_rng(seed)
    names = ["region", "day", "user", "amount", "price", "flag", "tiny", "cents"]
    types = [abi.SMALLINT, abi.DATE, abi.BIGINT, abi.BIGINT, abi.DOUBLE, abi.BOOLEAN, abi.TINYINT, abi.DECIMAL64]
    values = [np.repeat(rng.integers(0, 6, n // 500 + 1), 500)[:n].astype(np.int16),
              (19000 + np.arange(n) // 997).astype(np.int32),
              rng.integers(0, 50_000, n).astype(np.int64),
              rng.integers(-10**9, 10**9, n).astype(np.int64),
              np.round(rng.random(n) * 1000, 2),
              (rng.random(n) > 0.7).astype(np.uint8),
              rng.integers(-100, 100, n).astype(np.int8),
              rng.integers(-10**6, 10**6, n).astype(np.int64)]
    validity = [None, rng.random(n) > 0.02, rng.random(n) > 0.05, None, rng.random(n) > 0.1, None,
                rng.random(n) > 0.2, None]
    return names, types, values, validity
