"""The entry point that allocates nothing (dcns_semiglobal_noalloc) against the allocating one
(dcns_semiglobal_batch): same score and end positions, bit-exact, on calls in a row.  Its callers are the ones that
cannot allocate device memory at call time (memory owned by another allocator, or threads that cannot take
cudaMalloc's device-wide synchronisation), so the test allocates the input and output buffers itself and hands them
over.  Collected last so that a stop at the first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_LEN = 16384  # the fixed scratch array's limit per sequence


def _bind():
    import dcns_gb300
    L = dcns_gb300.library()
    L.dcns_semiglobal_noalloc.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.POINTER(dcns_gb300.Params),
                                          C.c_void_p, C.c_void_p]
    L.dcns_semiglobal_noalloc.restype = C.c_int
    return L


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.int8)).cuda()


def _call(L, da, na, db, nb, p, out, stream):
    return L.dcns_semiglobal_noalloc(da.data_ptr(), na, db.data_ptr(), nb, C.byref(p), out.data_ptr(), stream)


def test_noalloc_matches_allocating_entry_point(lib):
    import torch

    import dcns_gb300
    from dcns_gb300 import workloads as W
    L = _bind()
    rng = np.random.default_rng(8)
    pairs = []
    for n1, n2 in ((2400, 2100), (900, 3000)):
        x, y = W.planted_pair(rng, n1, n2, 4, 40, 200, 0.8, 0.95, 0.01, 0.0)
        pairs.append((W.prepare(x), W.prepare(y)))
    stream = torch.cuda.current_stream()
    for kw in (dict(), dict(bandwidth=60, zdrop=30, open2=-20, ext2=-1)):
        exp, _ = lib.SemiGlobal(pairs, cigar=False, **kw)
        p = dcns_gb300.params(**kw)
        for k, (a, b) in enumerate(pairs):  # two calls in a row share the scratch array
            da, db = _dev(a), _dev(b)
            out = torch.full((4,), -7, dtype=torch.int32, device="cuda")
            assert _call(L, da, len(a), db, len(b), p, out, stream.cuda_stream) == 0
            torch.cuda.synchronize()
            got = [int(v) for v in out.cpu()]
            assert got[3] == 0
            assert tuple(got[:3]) == tuple(int(v) for v in exp[k, :3]), (k, kw)


def test_noalloc_at_the_size_limit_and_back_to_back_on_one_stream(lib):
    """Pairs at the 16,384-base limit (full and one-column DPs), issued back to back on one stream with one
    synchronisation at the end: calls ordered on a stream reuse the shared array without a host sync."""
    import torch

    import dcns_gb300
    from dcns_gb300 import workloads as W
    L = _bind()
    rng = np.random.default_rng(11)
    x, y = W.planted_pair(rng, MAX_LEN, MAX_LEN, 12, 60, 400, 0.8, 0.95, 0.01, 0.0)
    big = (W.prepare(x)[:MAX_LEN], W.prepare(y)[:MAX_LEN])
    pad = lambda s: np.concatenate([s, rng.integers(0, 5, MAX_LEN - len(s)).astype(np.int8)])  # noqa: E731
    big = (pad(big[0]), pad(big[1]))
    one = (big[0], big[1][:1])
    small = (big[0][:700], big[1][100:900])
    pairs = [big, one, small, big]
    exp, _ = lib.SemiGlobal(pairs, cigar=False)
    p = dcns_gb300.params()
    stream = torch.cuda.Stream()
    ins = [(_dev(a), _dev(b)) for a, b in pairs]
    outs = [torch.full((4,), -7, dtype=torch.int32, device="cuda") for _ in pairs]
    torch.cuda.synchronize()
    for (a, b), (da, db), out in zip(pairs, ins, outs):
        assert _call(L, da, len(a), db, len(b), p, out, stream.cuda_stream) == 0
    stream.synchronize()
    for k, out in enumerate(outs):
        got = [int(v) for v in out.cpu()]
        assert got[3] == 0, k
        assert tuple(got[:3]) == tuple(int(v) for v in exp[k, :3]), k


def test_noalloc_bad_code_status_then_next_call_exact(lib):
    """A code outside 0..4 is reported in the status word (the host never sees the device sequence), and the next
    call on the same array is still exact."""
    import torch

    import dcns_gb300
    L = _bind()
    rng = np.random.default_rng(12)
    a = rng.integers(0, 5, 500).astype(np.int8)
    b = rng.integers(0, 5, 400).astype(np.int8)
    bad = a.copy()
    bad[123] = 7
    p = dcns_gb300.params()
    out = torch.full((4,), -7, dtype=torch.int32, device="cuda")
    assert _call(L, _dev(bad), len(bad), _dev(b), len(b), p, out, None) == 0
    torch.cuda.synchronize()
    assert [int(v) for v in out.cpu()] == [-1, -1, -1, 1]
    exp, _ = lib.SemiGlobal([(a, b)], cigar=False)
    assert _call(L, _dev(a), len(a), _dev(b), len(b), p, out, None) == 0
    torch.cuda.synchronize()
    got = [int(v) for v in out.cpu()]
    assert got[3] == 0 and tuple(got[:3]) == tuple(int(v) for v in exp[0, :3])


def test_noalloc_rejects_oversize_inputs_and_bad_parameters(lib):
    import torch

    import dcns_gb300
    L = _bind()
    a = torch.zeros(MAX_LEN + 1, dtype=torch.int8, device="cuda")
    out = torch.zeros(4, dtype=torch.int32, device="cuda")
    p = dcns_gb300.params()
    assert _call(L, a, MAX_LEN + 1, a, 10, p, out, None) == -1  # DCNS_ERR_INVALID: beyond the fixed scratch
    # the allocating entry point's parameter checks: a positive gap opening, an out-of-range second opening, a
    # negative z-drop are all rejected before anything is queued
    for kw in (dict(open1=1), dict(open2=-200000), dict(zdrop=-1), dict(bandwidth=0)):
        assert _call(L, a, 10, a, 10, dcns_gb300.params(**kw), out, None) == -1, kw
        with pytest.raises(dcns_gb300.DcnsError):
            lib.SemiGlobal([(np.zeros(10, np.int8), np.zeros(10, np.int8))], **kw)
