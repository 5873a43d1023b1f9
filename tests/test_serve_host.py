"""Serving loop host logic (no GPU): the seeded request mix and the
first-in first-out admission under an HBM budget, with a stand-in solver."""
import threading
import time

import pytest

import x2dhf_gb300 as xg
from conftest import golden_deck
from x2dhf_gb300 import serve

TEMPLATES = {n: golden_deck(n + "_set01") for n in ("h2", "lih", "fh", "co", "n2")}


def test_requests_are_reproducible_and_valid():
    a = serve.make_requests(TEMPLATES, 40, rate=5.0, seed=42)
    b = serve.make_requests(TEMPLATES, 40, rate=5.0, seed=42)
    assert [(q.template, q.arrival, q.r, q.nnu, q.nmu) for q in a] == [(q.template, q.arrival, q.r, q.nnu, q.nmu)
                                                                          for q in b]
    assert all(x.arrival < y.arrival for x, y in zip(a, a[1:]))
    assert {q.template for q in a} == set(TEMPLATES)
    electrons = {"h2": 2, "lih": 4, "fh": 10, "co": 14, "n2": 14}
    for q in a:
        c = xg.parse_deck(q.deck)
        assert (c.nnu, c.nmu) == (q.nnu, q.nmu)
        assert (q.nnu - 1) % 30 == 0 and (q.nmu - 1) % 30 == 0
        assert 151 <= q.nnu <= 481 and 241 <= q.nmu <= 721
        r0 = {"h2": 1.4, "lih": 3.015, "fh": 1.7328, "co": 2.132, "n2": 2.068}[q.template]
        assert max(1.5, 0.8 * r0) <= q.r <= min(5.0, 1.5 * r0)
        assert round(c.z1 + c.z2) == electrons[q.template] and max(c.z1, c.z2) <= 9
        assert sum(c.occ[i] for i in range(c.norb)) == electrons[q.template]
        assert q.bytes > 0


class FakeBackend:
    """Sleeps for a duration derived from the request and records the
    footprint in flight at every start."""

    def __init__(self):
        self.lock = threading.Lock()
        self.order = []

    def open(self):
        return object()

    def solve(self, h, q):
        with self.lock:
            self.order.append(q.rid)
        time.sleep(0.002 * (1 + q.rid % 3))
        return 10 + q.rid, 1, -float(q.rid), (-0.5,) * q.norb

    def close(self, h):
        pass


@pytest.mark.parametrize("slots,budget_factor", [(1, 100.0), (4, 100.0), (4, 2.5)])
def test_admission_fifo_and_budget(slots, budget_factor):
    reqs = serve.make_requests(TEMPLATES, 30, rate=0.0, seed=7)
    budget = int(budget_factor * max(q.bytes for q in reqs))
    be = FakeBackend()
    srv = serve.Server(slots=slots, hbm_budget=budget, backend=be)
    done, wall = srv.run(reqs, realtime=False)
    assert [c.rid for c in done] == [q.rid for q in reqs]
    assert be.order == sorted(be.order)  # first in, first out
    assert srv.peak_bytes <= budget
    assert (srv.budget_waits > 0) == (slots > 1 and budget_factor < 10)
    assert all(c.iterations == 10 + c.rid and c.total_energy == -float(c.rid) for c in done)
    s = serve.summary(done, wall)
    assert s["requests"] == 30 and s["latency_p99_s"] >= s["latency_p50_s"] > 0


def test_arrivals_are_honoured():
    reqs = serve.make_requests(TEMPLATES, 8, rate=200.0, seed=3)
    done, wall = serve.Server(slots=2, backend=FakeBackend()).run(reqs)
    for q, c in zip(reqs, done):
        assert c.start >= q.arrival - 1e-6 and c.latency >= c.end - c.start


class FailingBackend(FakeBackend):
    """FakeBackend whose every fifth request fails the way a library call
    reports a NaN."""

    def solve(self, h, q):
        if q.rid % 5 == 2:
            raise xg.X2GError(5, "NaN in orbital energy")
        return super().solve(h, q)


def test_failed_requests_are_recorded_and_serving_continues():
    reqs = serve.make_requests(TEMPLATES, 20, rate=0.0, seed=9)
    done, wall = serve.Server(slots=3, backend=FailingBackend()).run(reqs, realtime=False)
    assert [c.rid for c in done] == [q.rid for q in reqs]
    for c in done:
        if c.rid % 5 == 2:
            assert "NaN" in c.error and not c.converged and c.total_energy != c.total_energy
        else:
            assert not c.error and c.iterations == 10 + c.rid
    s = serve.summary(done, wall)
    assert s["failed"] == 4 and s["converged"] == 16 and s["unconverged"] == 0


def test_other_errors_stop_the_run():
    class Broken(FakeBackend):
        def solve(self, h, q):
            raise RuntimeError("backend bug")

    with pytest.raises(RuntimeError):
        serve.Server(slots=2, backend=Broken()).run(serve.make_requests(TEMPLATES, 4, rate=0.0, seed=1),
                                                   realtime=False)
