"""The entry point that allocates nothing (dcns_semiglobal_noalloc) against the allocating one
(dcns_semiglobal_batch): same score and end positions, bit-exact, on two calls in a row.  Its callers are the ones
that cannot allocate device memory at call time (memory owned by another allocator, or threads that cannot take
cudaMalloc's device-wide synchronisation), so the test allocates the input and output buffers itself and hands them
over.  Collected last so that a stop at the first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bind():
    import dcns_gb300
    L = dcns_gb300.library()
    L.dcns_semiglobal_noalloc.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.POINTER(dcns_gb300.Params),
                                          C.c_void_p, C.c_void_p]
    L.dcns_semiglobal_noalloc.restype = C.c_int
    return L


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
            da = torch.from_numpy(a.astype(np.int8)).cuda()
            db = torch.from_numpy(b.astype(np.int8)).cuda()
            out = torch.full((4,), -7, dtype=torch.int32, device="cuda")
            rc = L.dcns_semiglobal_noalloc(da.data_ptr(), len(a), db.data_ptr(), len(b), C.byref(p), out.data_ptr(),
                                           stream.cuda_stream)
            assert rc == 0
            torch.cuda.synchronize()
            got = [int(v) for v in out.cpu()]
            assert got[3] == 0
            assert tuple(got[:3]) == tuple(int(v) for v in exp[k, :3]), (k, kw)


def test_noalloc_rejects_oversize_inputs(lib):
    import torch

    import dcns_gb300
    L = _bind()
    a = torch.zeros(16385, dtype=torch.int8, device="cuda")
    out = torch.zeros(4, dtype=torch.int32, device="cuda")
    p = dcns_gb300.params()
    rc = L.dcns_semiglobal_noalloc(a.data_ptr(), 16385, a.data_ptr(), 10, C.byref(p), out.data_ptr(), None)
    assert rc == -1  # DCNS_ERR_INVALID: beyond the fixed scratch
