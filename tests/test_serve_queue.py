"""The native serving queue as a drop-in for the reference W3C service's
batcher (crates/cubbs-w3c-service/src/batcher.rs): the six batcher tests
(batcher.rs:325-500) restated against ServeQueue with a host processor, plus
the queue bound, the shared slot cap over per-queue limits, reply callbacks
that submit again, draining on close and a failing processor.  CPU
only: a server with a caller processor makes no CUDA call."""
import threading
import time

import pytest

from conftest import load_package


@pytest.fixture(scope="module")
def pkg():
    p = load_package()
    p.build()
    return p


def identity(queue, items):
    return [(0, v % 256, v) for v in items]


def values(recs, timeout=5):
    return [r.receive(timeout)[2] for r in recs]


def test_coalesces_requests_within_the_interval(pkg):
    # batcher.rs:325-347: a lone request waits out the window, five quick
    # ones share the next batch
    with pkg.ServeQueue(identity, max_inflight=1) as q:
        q.configure_batcher(0, interval_ms=20, max_batch_size=16, queue_capacity=32, pipelines=1)
        t = time.monotonic()
        assert q.submit(0, 1, timeout=5) == (0, 1, 1)
        assert time.monotonic() - t >= 0.019
        recs = [q.enqueue(0, v) for v in range(2, 7)]
        assert values(recs) == list(range(2, 7))
        s = q.snapshot(0)
        assert (s["dispatches"], s["last_batch_size"], s["max_observed_batch"]) == (2, 5, 5)
        assert s["batch_size_counts"][1] == 1 and s["batch_size_counts"][5] == 1
        assert len(s["batch_size_counts"]) == 17


def test_keeps_backlog_for_later_dispatches(pkg):
    # batcher.rs:349-370: nine requests at batch size 4 leave as 4, 4, 1
    with pkg.ServeQueue(identity, max_inflight=1) as q:
        q.configure_batcher(0, interval_ms=50, max_batch_size=4, queue_capacity=32, pipelines=1)
        assert q.submit(0, 0, timeout=5)[2] == 0
        recs = [q.enqueue(0, v) for v in range(1, 10)]
        assert values(recs) == list(range(1, 10))
        s = q.snapshot(0)
        assert (s["dispatched_items"], s["dispatches"], s["max_observed_batch"]) == (10, 4, 4)
        assert s["queued"] == 0 and s["inflight_batches"] == 0


def test_complete_batches_bypass_the_interval(pkg):
    # batcher.rs:372-394
    with pkg.ServeQueue(identity, max_inflight=1) as q:
        q.configure_batcher(0, interval_ms=100, max_batch_size=4, queue_capacity=32, pipelines=1)
        assert q.submit(0, 0, timeout=5)[2] == 0
        t = time.monotonic()
        recs = [q.enqueue(0, v) for v in range(1, 9)]
        assert values(recs) == list(range(1, 9))
        assert time.monotonic() - t < 0.08, "two complete batches must not wait for the 100 ms window"


def test_dispatches_as_soon_as_a_staggered_batch_is_full(pkg):
    # batcher.rs:396-421
    with pkg.ServeQueue(identity, max_inflight=1) as q:
        q.configure_batcher(0, interval_ms=100, max_batch_size=4, queue_capacity=32, pipelines=1)
        assert q.submit(0, 0, timeout=5)[2] == 0
        t = time.monotonic()
        first = q.enqueue(0, 1)
        time.sleep(0.005)
        rest = [q.enqueue(0, v) for v in range(2, 5)]
        assert values([first] + rest) == [1, 2, 3, 4]
        assert time.monotonic() - t < 0.08
        assert q.snapshot(0)["last_batch_size"] == 4


def test_partial_batch_gets_a_fresh_window_after_a_slow_dispatch(pkg):
    # batcher.rs:423-449
    def slow_first(queue, items):
        if items == [0]:
            time.sleep(0.03)
        return identity(queue, items)

    with pkg.ServeQueue(slow_first, max_inflight=1) as q:
        q.configure_batcher(0, interval_ms=20, max_batch_size=4, queue_capacity=32, pipelines=1)
        assert q.submit(0, 0, timeout=5)[2] == 0
        first = q.enqueue(0, 1)
        time.sleep(0.005)
        rest = [q.enqueue(0, v) for v in range(2, 5)]
        assert values([first] + rest) == [1, 2, 3, 4]
        s = q.snapshot(0)
        assert (s["dispatches"], s["last_batch_size"]) == (2, 4)


def _concurrency_probe(sleep_s):
    lock = threading.Lock()
    state = {"active": 0, "max": 0, "per_queue": {}}

    def proc(queue, items):
        with lock:
            state["active"] += 1
            state["max"] = max(state["max"], state["active"])
            pq = state["per_queue"].setdefault(queue, [0, 0])
            pq[0] += 1
            pq[1] = max(pq[1], pq[0])
        time.sleep(sleep_s)
        with lock:
            state["active"] -= 1
            state["per_queue"][queue][0] -= 1
        return identity(queue, items)

    return proc, state


def test_overlaps_batches_with_two_pipelines(pkg):
    # batcher.rs:451-489
    proc, state = _concurrency_probe(0.02)
    with pkg.ServeQueue(proc, max_inflight=2) as q:
        q.configure_batcher(0, interval_ms=0, max_batch_size=2, queue_capacity=32, pipelines=2)
        recs = [q.enqueue(0, v) for v in range(8)]
        assert values(recs) == list(range(8))
    assert state["max"] == 2


def test_shared_slots_cap_per_queue_pipelines(pkg):
    """Per-queue pipelines under a shared slot count (main.rs spawn_with_slots):
    two queues with two pipelines each never run more than the server's three
    batches at once, and each queue never more than its own two."""
    proc, state = _concurrency_probe(0.02)
    with pkg.ServeQueue(proc, max_inflight=3) as q:
        for queue in (0, 1):
            q.configure_batcher(queue, interval_ms=0, max_batch_size=1, queue_capacity=64, pipelines=2)
        recs = [q.enqueue(v % 2, v) for v in range(24)]
        assert values(recs) == list(range(24))
        s = q.snapshot(-1)
        assert s["dispatched_items"] == 24 and s["dispatches"] == 24
        assert q.snapshot(0)["dispatched_items"] == 12 == q.snapshot(1)["dispatched_items"]
    assert state["max"] == 3
    assert max(v[1] for v in state["per_queue"].values()) == 2


def test_queue_capacity_holds_back_submitters(pkg):
    gate = threading.Event()

    def blocked(queue, items):
        gate.wait(5)
        return identity(queue, items)

    with pkg.ServeQueue(blocked, max_inflight=1) as q:
        q.configure(0, max_batch_items=1, queue_capacity=2)
        first = q.enqueue(0, 0)        # taken by the slot, which blocks
        deadline = time.monotonic() + 5
        while q.snapshot(0)["inflight_batches"] != 1 and time.monotonic() < deadline:
            time.sleep(0.001)
        q.enqueue(0, 1)
        q.enqueue(0, 2)                # the queue is now full
        entered = threading.Event()
        third = []

        def late():
            entered.set()
            third.append(q.enqueue(0, 3))

        t = threading.Thread(target=late)
        t.start()
        entered.wait(5)
        time.sleep(0.05)
        assert not third, "a submit into a full queue must wait for room"
        assert q.snapshot(0)["queued"] == 2
        gate.set()
        t.join(5)
        assert third and third[0].receive(5)[2] == 3
        assert first.receive(5)[2] == 0


def test_reply_callback_may_submit_again(pkg):
    """A reply callback runs on the dispatch thread outside the queue's lock
    and can enqueue the next request."""
    with pkg.ServeQueue(identity, max_inflight=1) as q:
        q.configure(0, max_batch_items=8, coalesce_us=1000)
        seen = []
        done = threading.Event()

        def step(reply):
            seen.append(reply[2])
            if len(seen) < 6:
                q.enqueue(0, 100 + len(seen), callback=step)
            else:
                done.set()

        q.enqueue(0, 100, callback=step)
        assert done.wait(5)
        assert seen == list(range(100, 106))
        assert q.snapshot(0)["dispatches"] == 6


def test_close_serves_queued_requests(pkg):
    """Requests still queued when the server closes are served, not dropped."""
    q = pkg.ServeQueue(identity, max_inflight=2)
    q.configure(1, max_batch_items=1000, coalesce_us=10_000_000)
    late = [q.enqueue(1, v) for v in range(40)]
    assert q.snapshot(1)["queued"] == 40
    t = time.monotonic()
    q.close()
    assert time.monotonic() - t < 5
    assert all(r.done() for r in late)
    assert values(late) == list(range(40))


def test_failing_processor_fails_its_batch(pkg):
    def flaky(queue, items):
        if 13 in items:
            raise RuntimeError("processor failure")
        return identity(queue, items)

    with pkg.ServeQueue(flaky, max_inflight=1) as q:
        q.configure(0, max_batch_items=1)
        recs = [q.enqueue(0, v) for v in (12, 13, 14)]
        out = [r.receive(5) for r in recs]
    assert out[0] == (0, 12, 12) and out[2] == (0, 14, 14)
    assert out[1][0] == pkg.ERR_INTERNAL


def test_snapshot_queue_wait_and_config(pkg):
    with pkg.ServeQueue(identity, max_inflight=1, max_batch_items=64) as q:
        assert q.config(3) == {"max_batch_items": 64, "max_inflight": 0, "coalesce_us": 0, "queue_capacity": 0}
        eff = q.configure_batcher(3, interval_ms=10, max_batch_size=8, queue_capacity=100, pipelines=4)
        assert eff == {"max_batch_items": 8, "max_inflight": 4, "coalesce_us": 10000, "queue_capacity": 100}
        assert q.config(3) == eff
        recs = [q.enqueue(3, v) for v in range(3)]
        values(recs)
        s = q.snapshot(3)
        assert s["dispatched_items"] == 3
        # each request waited out (most of) the 10 ms window before dispatch
        assert s["total_queue_wait_ms"] >= 3 * 5
        assert s["average_queue_wait_ms"] == pytest.approx(s["total_queue_wait_ms"] / 3)
        empty = q.snapshot(5)
        assert empty["dispatches"] == 0 and empty["average_queue_wait_ms"] == 0.0


def test_invalid_arguments(pkg):
    import ctypes
    lib = pkg.lib()
    h = ctypes.c_void_p()
    assert lib.cubbs_bbs_gpu_serve_create_with_processor(
        pkg.ABI_VERSION, None, pkg._SERVE_PROCESSOR(), None, ctypes.addressof(h)) \
        == pkg.ERR_INVALID_INPUT
    with pkg.ServeQueue(identity) as q:
        with pytest.raises(ValueError):
            q.enqueue(pkg.SERVE_MAX_QUEUES, 1)
        with pytest.raises(ValueError):
            q.configure(-1)
        snap = pkg.ServeSnapshot()
        assert lib.cubbs_bbs_gpu_serve_snapshot(q._handle, 0, ctypes.byref(snap), None, ctypes.c_size_t(4)) \
            == pkg.ERR_INVALID_INPUT
