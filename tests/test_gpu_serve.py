"""Serving loop on the GPU: a request's results do not depend on what else
is being served (alone vs mixed with other requests, bit for bit)."""
import pytest

from conftest import golden_deck
from x2dhf_gb300 import serve

pytestmark = pytest.mark.gpu


def test_alone_equals_mixed():
    templates = {n: golden_deck(n + "_set01") for n in ("h2", "lih")}
    reqs = serve.make_requests(templates, 6, rate=0.0, seed=11)
    alone, _ = serve.Server(slots=1).run(reqs, realtime=False)
    mixed, _ = serve.Server(slots=3).run(reqs, realtime=False)
    for a, b in zip(alone, mixed):
        assert a.rid == b.rid and a.iterations == b.iterations
        assert a.total_energy == b.total_energy
        assert a.orbital_energies == b.orbital_energies
    assert all(a.converged for a in alone)


class _ShortSolves(serve.GpuBackend):
    """A fixed number of SCF iterations per request: many fresh solves (new
    buffers, grid tables and initial guesses) start while other slots'
    kernels run."""

    def solve(self, ctx, q):
        from x2dhf_gb300 import SCF, parse_deck
        s = SCF(ctx, parse_deck(q.deck, precision=self.precision, batch_mode=self.batch_mode))
        try:
            res = s.run(40)
            return res.iterations, res.converged, res.total_energy, tuple(float(res.ee[i]) for i in range(q.norb))
        finally:
            s.close()


def test_concurrent_starts_equal_alone():
    # every buffer a solve allocates and every table it uploads is ordered on
    # its context's stream, so solves starting beside others (small ones
    # beside N2 and CO, whose kernels keep the SMs busy) see the same state
    # as alone
    templates = {n: golden_deck(n + "_set01") for n in ("h2", "lih", "co", "n2")}
    reqs = serve.make_requests(templates, 32, rate=0.0, seed=5)
    alone, _ = serve.Server(slots=1, backend=_ShortSolves()).run(reqs, realtime=False)
    for _ in range(2):
        mixed, _ = serve.Server(slots=4, backend=_ShortSolves()).run(reqs, realtime=False)
        for a, b in zip(alone, mixed):
            assert a.rid == b.rid and a.iterations == b.iterations == 40
            assert a.total_energy == b.total_energy
            assert a.orbital_energies == b.orbital_energies
    assert all(e == e for a in alone for e in a.orbital_energies)
