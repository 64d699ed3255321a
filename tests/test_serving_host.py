"""Host logic of the serving loop (no GPU): admission by HBM footprint,
continuous batching over stream slots, result routing, cancellation, library
errors and timeouts, with a fake device backend."""
import threading
import time

import numpy as np
import pytest

from jax_cosmo_gb300.serving import Server, _Arena

P0 = [0.2589, 0.0486, 0.6774, 0.9667, 0.8159, 0.0, -1.0, 0.0]


class FakeModel:
    def __init__(self, footprint, tag=0.0):
        self.footprint = footprint
        self.tag = tag


class FakeBackend:
    """Batches complete when the test releases them (or at once if auto)."""

    def __init__(self, n_slots, auto=False, fail_launch=None):
        self.auto = auto
        self.fail_launch = fail_launch
        self.gates = [threading.Event() for _ in range(n_slots)]
        self.out = [None] * n_slots
        self.batches = []
        self.lock = threading.Lock()
        self.in_flight_bytes = 0
        self.max_in_flight_bytes = 0
        self.nbytes = [0] * n_slots

    def plan(self, models):
        s = sum(m.footprint for m in models)
        return s, s

    def launch(self, slot, reqs, off, nbytes):
        if self.fail_launch is not None and any(r.model.tag == self.fail_launch for r in reqs):
            raise ValueError("library refused the batch")
        with self.lock:
            self.batches.append([r.model.tag for r in reqs])
            self.in_flight_bytes += nbytes
            self.max_in_flight_bytes = max(self.max_in_flight_bytes, self.in_flight_bytes)
        self.nbytes[slot] = nbytes
        # result of a request: a function of its own inputs only
        self.out[slot] = np.array([[r.model.tag + np.sum(r.params)] + list(r.params * r.model.tag)
                                   for r in reqs])
        self.gates[slot].clear()
        if self.auto:
            self.gates[slot].set()

    def ready(self, slot):
        done = self.gates[slot].is_set()
        if done:
            with self.lock:
                self.in_flight_bytes -= self.nbytes[slot]
                self.nbytes[slot] = 0
        return done

    def fetch(self, slot, n):
        return self.out[slot][:n]

    def release_all(self):
        for g in self.gates:
            g.set()


def wait_until(cond, timeout=5.0):
    t0 = time.time()
    while not cond():
        if time.time() - t0 > timeout:
            raise AssertionError("condition not reached")
        time.sleep(0.001)


def test_arena_first_fit_and_coalesce():
    a = _Arena(10 * 256)
    o1 = a.alloc(300)   # 512
    o2 = a.alloc(256)
    o3 = a.alloc(1024)
    assert (o1, o2, o3) == (0, 512, 768)
    assert a.alloc(2048) is None
    a.release(o2, 256)
    a.release(o1, 300)
    assert a.free[0] == (0, 768)
    a.release(o3, 1024)
    assert a.free == [(0, 2560)] and a.used == 0 and a.peak == 1792


def test_results_routed_to_their_requests():
    be = FakeBackend(2, auto=True)
    with Server(hbm_budget=1 << 20, backend=be, n_streams=2) as srv:
        futs = []
        for k in range(50):
            p = np.array(P0) + 0.001 * k
            futs.append((k, p, srv.submit(FakeModel(1024, tag=float(k % 7 + 1)), p)))
        for k, p, f in futs:
            r = f.result(timeout=5)
            tag = float(k % 7 + 1)
            assert r.loglike == pytest.approx(tag + p.sum())
            np.testing.assert_allclose(r.grad, p * tag)
    st = srv.stats()
    assert st["completed"] == 50 and st["failed"] == 0
    assert st["p50_ms"] is not None and st["p99_ms"] >= st["p50_ms"]


def test_continuous_batching_one_slot():
    be = FakeBackend(1)
    srv = Server(hbm_budget=1 << 20, backend=be, n_streams=1).start()
    f1 = srv.submit(FakeModel(256, 1.0), P0)
    wait_until(lambda: len(be.batches) == 1)
    # arrivals while the first batch is on the device join the next launch
    later = [srv.submit(FakeModel(256, 2.0), P0) for _ in range(4)]
    time.sleep(0.05)
    assert len(be.batches) == 1
    be.gates[0].set()
    f1.result(timeout=5)
    wait_until(lambda: len(be.batches) == 2)
    assert be.batches[1] == [2.0] * 4
    be.release_all()
    for f in later:
        f.result(timeout=5)
    srv.stop()


def test_two_slots_overlap():
    be = FakeBackend(2)
    srv = Server(hbm_budget=1 << 20, backend=be, n_streams=2).start()
    srv.submit(FakeModel(256, 1.0), P0)
    wait_until(lambda: len(be.batches) == 1)
    srv.submit(FakeModel(256, 2.0), P0)
    # the second request does not wait for the first batch: second slot
    wait_until(lambda: len(be.batches) == 2)
    be.release_all()
    srv.stop()


def test_admission_by_footprint():
    be = FakeBackend(2)
    fp = 4 * 1024
    srv = Server(hbm_budget=10 * 1024, backend=be, n_streams=2, max_batch=64).start()
    futs = [srv.submit(FakeModel(fp, 1.0), P0) for _ in range(5)]
    wait_until(lambda: len(be.batches) == 1)
    time.sleep(0.05)
    # two requests fit in 10 KiB; the rest wait for memory, not for a slot
    assert be.batches == [[1.0, 1.0]]
    assert be.max_in_flight_bytes <= 10 * 1024
    for _ in range(3):
        be.release_all()
        time.sleep(0.02)
    for f in futs:
        f.result(timeout=5)
    srv.stop()
    assert be.max_in_flight_bytes <= 10 * 1024
    assert srv.stats()["arena_peak_bytes"] <= 10 * 1024


def test_refusals_at_submit():
    srv = Server(hbm_budget=4096, backend=FakeBackend(1, auto=True), n_streams=1)
    with pytest.raises(MemoryError):
        srv.submit(FakeModel(8192), P0)
    with pytest.raises(ValueError):
        srv.submit(FakeModel(256), [np.nan] + P0[1:])
    with pytest.raises(ValueError):
        srv.submit(FakeModel(256), P0[:7])


def test_cancelled_request_is_not_launched():
    be = FakeBackend(1)
    srv = Server(hbm_budget=1 << 20, backend=be, n_streams=1).start()
    srv.submit(FakeModel(256, 1.0), P0)
    wait_until(lambda: len(be.batches) == 1)
    f_cancel = srv.submit(FakeModel(256, 5.0), P0)
    f_keep = srv.submit(FakeModel(256, 6.0), P0)
    assert f_cancel.cancel()
    be.release_all()
    wait_until(lambda: len(be.batches) == 2)
    be.release_all()
    f_keep.result(timeout=5)
    srv.stop()
    assert [5.0] not in be.batches and all(5.0 not in b for b in be.batches)


def test_launch_error_fails_only_its_batch():
    be = FakeBackend(1, auto=True, fail_launch=9.0)
    with Server(hbm_budget=1 << 20, backend=be, n_streams=1) as srv:
        bad = srv.submit(FakeModel(256, 9.0), P0)
        with pytest.raises(ValueError):
            bad.result(timeout=5)
        good = srv.submit(FakeModel(256, 1.0), P0)
        assert good.result(timeout=5).loglike == pytest.approx(1.0 + sum(P0))


def test_timeout_retires_slot():
    be = FakeBackend(2)  # never released
    srv = Server(hbm_budget=1 << 20, backend=be, n_streams=2, timeout_s=0.2).start()
    f1 = srv.submit(FakeModel(256, 1.0), P0)
    with pytest.raises(TimeoutError):
        f1.result(timeout=5)
    # the other slot still serves (and times out in turn); then nothing is left
    f2 = srv.submit(FakeModel(256, 2.0), P0)
    with pytest.raises(TimeoutError):
        f2.result(timeout=5)
    f3 = srv.submit(FakeModel(256, 3.0), P0)
    with pytest.raises(RuntimeError):
        f3.result(timeout=5)
    srv.stop()
