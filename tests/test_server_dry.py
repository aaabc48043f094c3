"""CPU tests of the request loop's scheduling (dry mode: no device work).

A server created without a handle runs every admitted request for a time proportional to its
bytes instead of launching kernels, so admission by memory budget, the in-flight limit, arrival
order, tickets, rejection and the statistics are exercised here without a GPU."""
import time

import numpy as np

from skinny_matmul_gb300 import build
from skinny_matmul_gb300 import lib as L
from skinny_matmul_gb300.api import Server


def _server(budget, streams=2, inflight=4, group_bytes=0):
    """Dry server; grouping off unless asked (these tests exercise the in-flight slots)."""
    build.build()
    return Server(None, budget, streams, inflight, group_bytes=group_bytes)


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


FAKE = 1 << 40  # host "addresses" for dry mode, which never dereferences them


def test_dry_small_requests_are_grouped():
    """Small requests collect while a grouped batch runs and go out together: far fewer launches
    than requests."""
    s = _server(1 << 30, group_bytes=32 << 20)
    # FP64 8 x 8, K = 30000: 3.8 MB of operands, 1.9 M FMAs ~ 22 MB-equivalent of cost
    tickets = [s.submit("tsmttsm", "float64", 8, 8, 30000, FAKE, 8, FAKE + 8, 8, FAKE + 16, 8)[1]
               for _ in range(200)]
    s.drain(60)
    for t in tickets:
        assert s.poll(t) == (L.OK, L.OK)
    st = s.stats()
    assert st["completed"] == 200 and st["grouped"] == 200
    assert 1 <= st["group_launches"] <= 100
    assert st["max_inflight_seen"] == 0  # no in-flight slot was used
    s.close()


def test_dry_grouping_threshold_and_ops():
    """Above the cost threshold, SVQB and the dd / split methods run on their own; the cost of an
    FP64 product counts its FMAs (~11 bytes-equivalent each), not only its bytes."""
    s = _server(1 << 40, group_bytes=1 << 20)
    t_small = s.submit("tsmm", "float64", 4, 4, 1000, FAKE, 4, FAKE, 4, FAKE, 4)[1]
    t_big = s.submit("tsmm", "float64", 4, 4, 1 << 20, FAKE, 4, FAKE, 4, FAKE, 4)[1]
    t_dd = s.submit("tsmttsm", "float64", 4, 4, 1000, FAKE, 4, FAKE, 4, FAKE, 4, acc="dd")[1]
    t_sv = s.submit("svqb", "float64", 4, 4, 1000, FAKE, 4, None, 0, FAKE, 4)[1]
    t_wide = s.submit("tsmttsm", "float64", 65, 4, 100, FAKE, 65, FAKE, 4, FAKE, 65)[1]
    # 32 x 32 FP64, K = 4000: 2 MB of operands (under the threshold) but 4 M FMAs (over it)
    t_fma = s.submit("tsmttsm", "float64", 32, 32, 4000, FAKE, 32, FAKE + 8, 32, FAKE + 16, 32)[1]
    # the same shape in FP32 is priced by its bytes (1 MB): grouped
    t_f32 = s.submit("tsmttsm", "float32", 32, 32, 4000, FAKE, 32, FAKE + 8, 32, FAKE + 16, 32)[1]
    s.drain(60)
    for t in (t_small, t_big, t_dd, t_sv, t_wide, t_fma, t_f32):
        assert s.poll(t) == (L.OK, L.OK)
    st = s.stats()
    assert st["grouped"] == 2 and st["completed"] == 7
    s.close()


def test_dry_small_passes_large_waiting_for_a_slot():
    """One in-flight slot: a small request behind a large one that waits for the slot runs first."""
    s = _server(1 << 40, inflight=1, group_bytes=32 << 20)
    K = 1 << 20  # TSMM 64 x 64 FP64: ~1 GB, ~20 ms of dry time each
    t1 = s.submit("tsmm", "float64", 64, 64, K, FAKE, 64, FAKE + 8, 64, FAKE + 16, 64)[1]
    t2 = s.submit("tsmm", "float64", 64, 64, K, FAKE, 64, FAKE + 8, 64, FAKE + 16, 64)[1]
    ts = s.submit("tsmttsm", "float64", 4, 4, 1000, FAKE, 4, FAKE + 8, 4, FAKE + 16, 4)[1]
    assert s.wait(ts, 10) == (L.OK, L.OK)
    assert s.poll(t2)[0] == L.NOT_READY
    s.drain(60)
    assert s.poll(t1) == (L.OK, L.OK) and s.poll(t2) == (L.OK, L.OK)
    s.close()


def test_dry_small_never_passes_a_memory_wait():
    """A small request behind a large one that waits for memory waits too (strict memory order)."""
    K = 1 << 20
    need = 2 * K * 64 * 8 + 64 * 64 * 8  # A and C of the large TSMM, B rounded below
    s = _server(need + (1 << 20), inflight=4, group_bytes=32 << 20)
    t1 = s.submit("tsmm", "float64", 64, 64, K, FAKE, 64, FAKE + 8, 64, FAKE + 16, 64)[1]
    t2 = s.submit("tsmm", "float64", 64, 64, K, FAKE, 64, FAKE + 8, 64, FAKE + 16, 64)[1]
    ts = s.submit("tsmttsm", "float64", 4, 4, 1000, FAKE, 4, FAKE + 8, 4, FAKE + 16, 4)[1]
    assert s.wait(ts, 30) == (L.OK, L.OK)
    assert s.poll(t1) == (L.OK, L.OK)  # the small request could only start after t1 freed memory
    s.drain(60)
    assert s.poll(t2) == (L.OK, L.OK)
    s.close()
