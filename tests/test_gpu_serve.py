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
