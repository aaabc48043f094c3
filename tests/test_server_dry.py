"""CPU tests of the request loop's scheduling (dry mode: no device work).

A server created without a handle runs every admitted request for a time proportional to its
bytes instead of launching kernels, so admission by memory budget, the in-flight limit, arrival
order, tickets, rejection and the statistics are exercised here without a GPU."""
import time

import numpy as np

from skinny_matmul_gb300 import build
from skinny_matmul_gb300 import lib as L
from skinny_matmul_gb300.api import Server


def _server(budget, streams=2, inflight=4):
    build.build()
    return Server(None, budget, streams, inflight)


def test_dry_admission_respects_budget_and_slots():
    budget = 4 << 20
    s = _server(budget, inflight=3)
    bufs = []
    tickets = []
    for i in range(40):
        K = 20000 + 1000 * i
        A = np.zeros(K * 8)
        C = np.zeros(64)
        bufs.append((A, C))
        st, t = s.submit("tsmttsm", "float64", 8, 8, K, A, 8, A, 8, C, 8)
        assert st == L.OK
        tickets.append(t)
    s.drain(60)
    for t in tickets:
        st, res = s.poll(t)
        assert st == L.OK and res == L.OK
    stats = s.stats()
    assert stats["completed"] == 40 and stats["failed"] == 0
    assert 0 < stats["peak_bytes_in_use"] <= budget
    assert 1 <= stats["max_inflight_seen"] <= 3
    assert stats["p99_latency_us"] >= stats["p50_latency_us"] > 0
    s.close()


def test_dry_rejects_oversized_and_malformed():
    s = _server(1 << 20)
    A = np.zeros(10)
    st, t = s.submit("tsmm", "float64", 8, 8, 1 << 20, A, 8, A, 8, A, 8)  # needs far more than 1 MiB
    assert st == L.NO_MEM
    st2, res = s.poll(t)
    assert st2 == L.OK and res == L.NO_MEM
    st, t = s.submit("svqb", "float32", 4, 4, 100, A, 4)  # SVQB is FP64 only
    assert st == L.BAD_ARG
    assert s.stats()["rejected"] == 2
    s.close()


def test_dry_requests_arriving_during_execution_are_admitted():
    """Continuous batching: requests submitted while others run are admitted as memory frees up,
    and in arrival order of admission."""
    s = _server(2 << 20, inflight=8)
    keep = []
    first = []
    for i in range(4):
        A = np.zeros(60000 * 2)
        keep.append(A)
        first.append(s.submit("tsmttsm", "float64", 2, 2, 60000, A, 2, A, 2, np.zeros(4), 2)[1])
    time.sleep(0.001)
    late = []
    for i in range(6):
        A = np.zeros(30000 * 2)
        keep.append(A)
        late.append(s.submit("tsmm", "float64", 2, 2, 30000, A, 2, np.zeros(4), 2, A, 2)[1])
    for t in first + late:
        st, res = s.wait(t, 30)
        assert st == L.OK and res == L.OK
    assert s.stats()["completed"] == 10
    s.close()


def test_dry_wait_timeout_and_unknown_ticket():
    s = _server(1 << 30)
    st, res = s.wait(123456, timeout_s=0.01)
    assert st == L.TIMEOUT
    st, res = s.poll(999)
    assert st == L.NOT_READY
    s.close()
