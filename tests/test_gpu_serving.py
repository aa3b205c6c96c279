"""The serving loop's admission and failure paths (all made on the host: small device budgets, short waits,
cancellations, requests the host rejects), each followed by results that stay bit-exact: served results are
compared with the oracle restatement, or with the same context's batch call where the oracle's run would be long."""
import threading

import numpy as np
import pytest

import dcns_gb300
from dcns_gb300 import workloads as W

pytestmark = pytest.mark.gpu

NOMEM, TIMEOUT, NOTFOUND, INVALID = -2, -4, -5, -1


def keys(frs):
    return [f.key() for f in frs]


@pytest.fixture(scope="module")
def requests_small():
    return W.batched_pairs(n_pairs=24, seed=31)


def test_admission_by_predicted_work_and_bytes(lib, oracle, requests_small):
    """A tight scan-cell cap and the predicted-bytes cap make the loop admit the queue in several batches."""
    lib.serve_start(1, max_inflight=64, workers=2, batch_cells=2 * 10 ** 8)
    try:
        tickets = [lib.submit(a, b) for a, b in requests_small]
        served = [lib.wait(t) for t in tickets]
        st = lib.serve_stats()
    finally:
        lib.serve_stop()
    assert st["completed"] == len(requests_small) and st["failed"] == 0
    assert st["batches"] > 1 and st["max_batch"] < len(requests_small), st
    for k, (a, b) in enumerate(requests_small):
        assert keys(served[k]) == keys(oracle.find(a, b)[0]), k


def test_device_budget_splits_batches_exactly(oracle, requests_small):
    """A context budget that one request fits and the whole queue does not: with the predicted-bytes cap lifted,
    the device budget's own check rejects the batch (DCNS_ERR_NOMEM) and the loop halves it until each part fits;
    every result is still the oracle's, and the same context aligns exactly afterwards."""
    budget = None
    for mb in (12, 16, 24, 32, 48, 64, 96, 128, 192, 256):
        # every request alone fits: run one after another on one context (its buffers only grow, so each call had
        # at most the budget), then the whole queue on a fresh context
        e = dcns_gb300.Engine(0, mem_budget=mb << 20)
        try:
            for p in requests_small:
                e.align_pairs([p], 1)
        except dcns_gb300.DcnsError as err:
            assert err.code == NOMEM
            continue
        finally:
            e.close()
        e = dcns_gb300.Engine(0, mem_budget=mb << 20)
        try:
            e.align_pairs(requests_small, 1)
            fits_all = True
        except dcns_gb300.DcnsError as err:
            assert err.code == NOMEM
            fits_all = False
        finally:
            e.close()
        if not fits_all:
            budget = mb << 20
        break
    if budget is None:
        pytest.skip("no probed budget fits one request but not the whole queue")
    eng = dcns_gb300.Engine(0, mem_budget=budget)
    try:
        eng.serve_start(1, max_inflight=64, workers=1, batch_cells=10 ** 15, admit_bytes=1 << 50)
        try:
            tickets = [eng.submit(a, b) for a, b in requests_small]
            served = [eng.wait(t) for t in tickets]
            st = eng.serve_stats()
        finally:
            eng.serve_stop()
        assert st["nomem_splits"] > 0 and st["failed"] == 0, st
        for k, (a, b) in enumerate(requests_small):
            assert keys(served[k]) == keys(oracle.find(a, b)[0]), k
        a, b = requests_small[3]
        assert keys(eng.align_pairs([(a, b)], 1)[0]) == keys(oracle.find(a, b)[0])
    finally:
        eng.close()


def test_wait_timeout_then_result(lib):
    """A 1 ms wait on a long request returns DCNS_ERR_TIMEOUT; waiting again returns the result."""
    rng = np.random.default_rng(5)
    long = []
    for _ in range(3):
        x, y = W.planted_pair(rng, 30000, 30000, 40, 60, 300, 0.8, 0.95, 0.01, 0.0)
        long.append((W.prepare(x), W.prepare(y)))
    lib.serve_start(1, max_inflight=8, workers=1)
    try:
        tickets = [lib.submit(a, b) for a, b in long]
        with pytest.raises(dcns_gb300.DcnsError) as ei:
            lib.wait(tickets[-1], timeout_ms=1)
        assert ei.value.code == TIMEOUT
        served = [lib.wait(t) for t in tickets]
    finally:
        lib.serve_stop()
    batch = lib.align_pairs(long, 1)
    for k in range(len(long)):
        assert keys(served[k]) == keys(batch[k]), k


def test_cancel_and_rejected_requests(lib, requests_small):
    """Cancelled tickets (queued or being aligned) report DCNS_ERR_NOTFOUND; codes outside 0..4 are rejected at
    submission; an unknown ticket is DCNS_ERR_NOTFOUND; the other requests are exact."""
    lib.serve_start(1, max_inflight=4, workers=1, batch_cells=10 ** 9)
    try:
        bad = requests_small[0][0].copy()
        bad[7] = 9
        with pytest.raises(dcns_gb300.DcnsError) as ei:
            lib.submit(bad, requests_small[0][1])
        assert ei.value.code == INVALID
        tickets = [lib.submit(a, b) for a, b in requests_small]
        gone = {tickets[0], tickets[-1], tickets[-2]}
        for t in gone:
            lib.cancel(t)
        for t in gone:
            with pytest.raises(dcns_gb300.DcnsError) as ei:
                lib.wait(t)
            assert ei.value.code == NOTFOUND
        with pytest.raises(dcns_gb300.DcnsError) as ei:
            lib.wait(10 ** 9)
        assert ei.value.code == NOTFOUND
        served = {t: lib.wait(t) for t in tickets if t not in gone}
        st = lib.serve_stats()
    finally:
        lib.serve_stop()
    assert st["cancelled"] == 3 and st["failed"] == 0
    batch = lib.align_pairs(requests_small, 1)
    for k, t in enumerate(tickets):
        if t not in gone:
            assert keys(served[t]) == keys(batch[k]), k


def test_failing_request_fails_alone(lib, oracle, requests_small):
    """A request the pipeline rejects (a sequence of 2^24 bases, beyond its 16 M limit) admitted into one batch with
    others: the batch is retried one request at a time, that request alone fails (DCNS_ERR_INVALID) and the rest
    are the oracle's."""
    huge = np.zeros(1 << 24, np.int8)
    reqs = list(requests_small[:6]) + [(huge, requests_small[0][1])] + list(requests_small[6:12])
    lib.serve_start(1, max_inflight=64, workers=1, batch_cells=10 ** 18, admit_bytes=1 << 60)
    try:
        tickets = [lib.submit(a, b) for a, b in reqs]
        results = {}
        for k, t in enumerate(tickets):
            try:
                results[k] = lib.wait(t)
            except dcns_gb300.DcnsError as err:
                results[k] = err.code
        st = lib.serve_stats()
    finally:
        lib.serve_stop()
    assert results[6] == INVALID
    assert st["solo_retries"] > 0 and st["failed"] == 1, st
    for k, (a, b) in enumerate(reqs):
        if k != 6:
            assert keys(results[k]) == keys(oracle.find(a, b)[0]), k


def test_stop_overlapping_waiters(lib, requests_small):
    """dcns_serve_stop while other threads wait: it aligns what is queued and wakes every waiter, which returns its
    result (or DCNS_ERR_NOTFOUND for a ticket it does not hold); nothing is freed under them."""
    lib.serve_start(1, max_inflight=8, workers=2)
    tickets = [lib.submit(a, b) for a, b in requests_small]
    got, errs = {}, []

    def waiter(ts):
        for t in ts:
            try:
                got[t] = lib.wait(t)
            except dcns_gb300.DcnsError as err:
                errs.append(err.code)

    ths = [threading.Thread(target=waiter, args=(tickets[k::3],)) for k in range(3)]
    for th in ths:
        th.start()
    lib.serve_stop()
    for th in ths:
        th.join(timeout=600)
    assert not any(th.is_alive() for th in ths)
    assert all(c in (NOTFOUND, INVALID) for c in errs)
    batch = lib.align_pairs(requests_small, 1)
    for k, t in enumerate(tickets):
        if t in got:
            assert keys(got[t]) == keys(batch[k]), k
