"""The allocation-free GROUP BY entry point, through the C ABI.

tgpu_group_by_i64_noalloc exists for callers that cannot let a library
allocate device memory (a host that pre-reserves the GPU's memory for its own
arena, a plugin inside another runtime's pool, a latency-critical loop that
must not block in cudaMalloc/cudaFree).  It keeps its group table in a fixed
device array inside the library.  This test checks it against the regular
operator (tgpu_query_create / tgpu_query_next) and against the oracle on two
calls in a row, which also shows the shared array is left ready for the next
call.  The first call of the file runs on a non-blocking stream (the call may
not rely on the legacy default stream to order its clearing), then come an
empty input and the largest result the fixed buffers hold.  The file sorts
last so a stop-at-first-failure run has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from thindb_gb300 import abi
from thindb_gb300.engine import AggSpec, Column, Request, Table, lib, try_build_group_topn

pytestmark = pytest.mark.gpu

MAX_GROUPS = 65536


def noalloc_fn():
    fn = lib().tgpu_group_by_i64_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64] + [C.c_void_p] * 6 + [C.c_void_p]
    return fn


def regular(keys, values):
    t = Table([Column("k", abi.BIGINT, keys), Column("v", abi.BIGINT, values)])
    q = try_build_group_topn(t, Request(["k"], [AggSpec("count", None, "c"), AggSpec("sum", "v", "s"),
                                                 AggSpec("min", "v", "mn"), AggSpec("max", "v", "mx")]))
    r = q.collect()
    q.close()
    t.close()
    order = np.argsort(r["k"][0], kind="stable")
    return [r[n][0][order] for n in ("k", "c", "s", "mn", "mx")]


def by_oracle(keys, values):
    import oracle

    cols = [Column("k", abi.BIGINT, keys), Column("v", abi.BIGINT, values)]
    req = Request(["k"], [AggSpec("count", None, "c"), AggSpec("sum", "v", "s"), AggSpec("min", "v", "mn"),
                          AggSpec("max", "v", "mx")])
    r = oracle.run(oracle.HostTable(cols), req, threads=4)
    order = np.argsort(r["k"][0], kind="stable")
    return [np.asarray(r[n][0])[order] for n in ("k", "c", "s", "mn", "mx")]


def run_noalloc(torch, keys, values, stream=None):
    dk = torch.from_numpy(keys).cuda()
    dv = torch.from_numpy(values).cuda()
    outs = [torch.zeros(MAX_GROUPS, dtype=torch.int64, device="cuda") for _ in range(5)]
    ng = torch.zeros(1, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()  # inputs and outputs are ready before a call on another stream
    handle = stream.cuda_stream if stream is not None else None
    st = noalloc_fn()(dk.data_ptr() if len(keys) else None, dv.data_ptr() if len(keys) else None, len(keys),
                      *[o.data_ptr() for o in outs], ng.data_ptr(), handle)
    assert st == abi.OK, lib().tgpu_last_error_message()
    n = int(ng.item())
    cols = [o[:n].cpu().numpy() for o in outs]
    order = np.argsort(cols[0], kind="stable")
    return [c[order] for c in cols]


def check(got, keys, values, call):
    want = regular(keys, values)
    ref = by_oracle(keys, values)
    for g, w, o, name in zip(got, want, ref, ("k", "count", "sum", "min", "max")):
        assert np.array_equal(g, w), (call, name, "regular operator")
        assert np.array_equal(g, o), (call, name, "oracle")


def test_noalloc_matches_regular_operator_twice():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2026)
    side = torch.cuda.Stream()  # non-blocking: no implicit order with the legacy default stream
    for call, (n, groups) in enumerate([(1_000_000, 5_000), (300_000, 40_000)]):
        domain = rng.integers(-(1 << 62), 1 << 62, groups, dtype=np.int64)
        domain[0] = 0  # the all-zero key takes the table's extra slot
        keys = domain[rng.integers(0, groups, n)]
        values = rng.integers(-(1 << 62), 1 << 62, n, dtype=np.int64)  # BIGINT sums wrap
        got = run_noalloc(torch, keys, values, stream=side if call == 0 else None)
        check(got, keys, values, call)


def test_noalloc_empty_and_largest_result():
    torch = pytest.importorskip("torch")
    empty = np.zeros(0, dtype=np.int64)
    got = run_noalloc(torch, empty, empty)
    assert all(len(c) == 0 for c in got)
    # exactly TGPU_NOALLOC_MAX_GROUPS distinct keys: every output slot used
    rng = np.random.default_rng(7)
    domain = rng.choice(np.arange(-(1 << 40), 1 << 40, 9973, dtype=np.int64), MAX_GROUPS, replace=False)
    keys = np.concatenate([domain, domain[rng.integers(0, MAX_GROUPS, 200_000)]])
    values = rng.integers(-(1 << 40), 1 << 40, len(keys), dtype=np.int64)
    got = run_noalloc(torch, keys, values)
    assert len(got[0]) == MAX_GROUPS
    check(got, keys, values, "max")


def test_noalloc_rejects_too_many_groups():
    torch = pytest.importorskip("torch")
    keys = np.arange(1, MAX_GROUPS + 100, dtype=np.int64)
    values = np.ones_like(keys)
    dk = torch.from_numpy(keys).cuda()
    dv = torch.from_numpy(values).cuda()
    outs = [torch.zeros(MAX_GROUPS, dtype=torch.int64, device="cuda") for _ in range(5)]
    ng = torch.zeros(1, dtype=torch.int64, device="cuda")
    st = noalloc_fn()(dk.data_ptr(), dv.data_ptr(), len(keys), *[o.data_ptr() for o in outs], ng.data_ptr(), None)
    assert st == abi.ERR_INVALID_ARGUMENT
    assert b"65,536" in lib().tgpu_last_error_message()
    # the scratch is still usable afterwards
    keys2 = np.array([3, 1, 3], dtype=np.int64)
    got = run_noalloc(torch, keys2, np.array([10, 20, 30], dtype=np.int64))
    assert [list(c) for c in got] == [[1, 3], [1, 2], [20, 40], [20, 10], [20, 30]]
