"""The relaxation entry point that allocates nothing.

x2g_relax_noalloc exists for callers that must not allocate device memory
while they run (x2g_relax grows its workspace with cudaMalloc when a larger
batch arrives).  It keeps its scratch in a fixed library-resident device
array instead.  This test checks it against x2g_relax on the same inputs:
all Coulomb and exchange potentials of one Ne orbital (right-hand sides
built on the device in that scratch), two calls in a row, FP64 results
bit for bit equal as in the other sweep tests.  It also checks that a batch
larger than the fixed scratch is refused with an error.

This file is collected last on purpose (test_zz_*).
"""
import pytest

import x2dhf_gb300 as xg
from conftest import golden_deck
from oracle.pyoracle import Case

pytestmark = pytest.mark.gpu


def _potential_jobs(torch, oc, c, iorb, dev):
    orbs = {i: torch.tensor(oc.putin(1 if c.m[i - 1] % 2 == 0 else -1, oc.orbital(i)), device=dev)
            for i in range(1, oc.norb + 1)}
    omega = oc.omega()[1]
    bufs, specs = [], []
    for k in range(1, oc.npots(iorb) + 1):
        in1, in2, idel, isym = oc.pot_info(iorb, k)
        bufs.append(torch.tensor(oc.putin(isym, oc.pot(iorb, k)), device=dev))
        specs.append((in1, in2, idel, isym))
    return orbs, bufs, specs, omega


def _jobs(xg, orbs, bufs, specs, omega):
    return [xg.Job(u=u.data_ptr(), psa=orbs[a].data_ptr(), psb=orbs[b].data_ptr(), omega=omega, isym=s, idel=d, kind=1)
            for u, (a, b, d, s) in zip(bufs, specs)]


def test_noalloc_matches_relax_two_calls():
    torch = pytest.importorskip("torch")
    deck = golden_deck("ne_set01")
    oc = Case(deck)
    c = xg.parse_deck(deck)
    ctx = xg.Context(0)
    grid = xg.Grid(ctx, c.nnu, c.nmu, c.r, c.rinf, c.z1, c.z2)
    dev = torch.device("cuda:0")
    orbs, ref_bufs, specs, omega = _potential_jobs(torch, oc, c, 1, dev)
    new_bufs = [b.clone() for b in ref_bufs]
    ref_jobs = _jobs(xg, orbs, ref_bufs, specs, omega)
    new_jobs = _jobs(xg, orbs, new_bufs, specs, omega)
    torch.cuda.synchronize()
    for call in range(2):
        xg.relax(ctx, grid, ref_jobs, 10, xg.FP64)
        ctx.synchronize()
        xg.relax_noalloc(ctx, grid, new_jobs, 10)
        for k, (a, b) in enumerate(zip(ref_bufs, new_bufs)):
            assert torch.equal(a, b), (call, k, (a - b).abs().max().item())
    grid.close()
    ctx.close()


def test_noalloc_rejects_oversized_batch():
    torch = pytest.importorskip("torch")
    deck = golden_deck("ne_set01")
    c = xg.parse_deck(deck)
    ctx = xg.Context(0)
    grid = xg.Grid(ctx, c.nnu, c.nmu, c.r, c.rinf, c.z1, c.z2)
    u = torch.zeros((c.nmu + 8) * (c.nnu + 8), dtype=torch.float64, device="cuda:0")
    job = xg.Job(u=u.data_ptr(), psa=u.data_ptr(), psb=u.data_ptr(), omega=1.9, isym=1, idel=0, kind=1)
    # one right-hand side of this grid is 151*181*8 bytes: 200 jobs exceed 32 MiB
    with pytest.raises(xg.X2GError) as ei:
        xg.relax_noalloc(ctx, grid, [job] * 200, 10)
    assert ei.value.code == 1 and "scratch" in str(ei.value)
    grid.close()
    ctx.close()
