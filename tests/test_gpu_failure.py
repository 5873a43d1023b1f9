"""Failure detection of the persistent sweeps, tested without a GPU fault.

Every device-side wait of the cooperative FP64 sweep (its grid barrier) and
of the persistent-band FP32 sweep of the mixed form (its neighbours' phase
counts) is bounded by the context's wait limit.  With the limit set to 0 a
wait that is not met at once fails: the waiting block records
X2G_ERR_TIMEOUT and every block of the launch returns.  Nothing hangs,
nothing traps.  These tests check that

* the timeout reaches the caller as error code 4 at the next synchronisation;
* the error of one call survives a second, normal call queued behind it
  before the host reads it (the error word is not cleared between launches:
  the second call's launches leave at their first wait);
* the next call on the same context succeeds and gives the same bits as a
  context that never timed out.

Each call relaxes 40 potentials of the Ne grid, so the FP64 sweep runs as two
launches (32 + 8 jobs) and the error of the first launch must outlive the
second.
"""
import numpy as np
import pytest

import x2dhf_gb300 as xg
from conftest import golden_deck
from oracle.pyoracle import Case

pytestmark = pytest.mark.gpu

NJOBS = 40


@pytest.fixture(scope="module")
def ne():
    torch = pytest.importorskip("torch")
    deck = golden_deck("ne_set01")
    oc = Case(deck)
    c = xg.parse_deck(deck)
    specs = []
    iorb = 1
    while len(specs) < NJOBS:
        for k in range(1, oc.npots(iorb) + 1):
            in1, in2, idel, isym = oc.pot_info(iorb, k)
            specs.append((in1, in2, idel, isym, oc.putin(isym, oc.pot(iorb, k))))
        iorb = iorb % oc.norb + 1
    specs = specs[:NJOBS]
    orbs = {i: oc.putin(1 if c.m[i - 1] % 2 == 0 else -1, oc.orbital(i)) for i in range(1, oc.norb + 1)}
    return torch, c, orbs, specs, oc.omega()[1]


def _batch(ne):
    """Fresh device copies of the 40 potentials and their jobs."""
    torch, c, orbs, specs, omega = ne
    dev = torch.device("cuda:0")
    dorbs = {i: torch.tensor(v, device=dev) for i, v in orbs.items()}
    bufs = [torch.tensor(s[4], device=dev) for s in specs]
    jobs = [xg.Job(u=u.data_ptr(), psa=dorbs[a].data_ptr(), psb=dorbs[b].data_ptr(), omega=omega, isym=isym,
                   idel=idel, kind=1) for u, (a, b, idel, isym, _) in zip(bufs, specs)]
    torch.cuda.synchronize()
    return dorbs, bufs, jobs


def _reference(ne, precision, on_chip=True):
    """The same batch on a context that never timed out."""
    torch, c = ne[0], ne[1]
    ctx = xg.Context(0)
    ctx.set_mixed_on_chip(on_chip)
    g = xg.Grid(ctx, c.nnu, c.nmu, c.r, c.rinf, c.z1, c.z2)
    keep, bufs, jobs = _batch(ne)
    xg.relax(ctx, g, jobs, 10, precision)
    ctx.synchronize()
    out = [b.cpu().numpy() for b in bufs]
    g.close()
    ctx.close()
    return out


@pytest.mark.parametrize("precision,on_chip", [(xg.FP64, True), (xg.MIXED, False)],
                         ids=["fp64-grid-barrier", "mixed-persistent-band"])
def test_timeout_is_reported_and_context_recovers(ne, precision, on_chip):
    c = ne[1]
    ref = _reference(ne, precision, on_chip)
    ctx = xg.Context(0)
    ctx.set_mixed_on_chip(on_chip)
    g = xg.Grid(ctx, c.nnu, c.nmu, c.r, c.rinf, c.z1, c.z2)
    # call 1 times out; call 2, with the normal limit, is queued before the
    # host reads the error word and must not wipe it
    k1 = _batch(ne)
    ctx.set_wait_limit(0.0)
    xg.relax(ctx, g, k1[2], 10, precision)
    k2 = _batch(ne)
    ctx.set_wait_limit(2.0)
    xg.relax(ctx, g, k2[2], 10, precision)
    with pytest.raises(xg.X2GError) as ei:
        ctx.synchronize()
    assert ei.value.code == 4, str(ei.value)
    # the context is usable again and bit-identical to an untouched one
    keep, bufs, jobs = _batch(ne)
    xg.relax(ctx, g, jobs, 10, precision)
    ctx.synchronize()
    for k, (b, r) in enumerate(zip(bufs, ref)):
        assert np.array_equal(b.cpu().numpy(), r), k
    g.close()
    ctx.close()


def test_wait_limit_argument_checked():
    ctx = xg.Context(0)
    with pytest.raises(xg.X2GError) as ei:
        ctx.set_wait_limit(-1.0)
    assert ei.value.code == 1
    ctx.set_wait_limit(2.0)
    ctx.close()
