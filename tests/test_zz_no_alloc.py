"""The relaxation entry point that allocates nothing.

x2g_relax_noalloc exists for callers that must not allocate device memory
while they run (x2g_relax grows its workspace with cudaMalloc when a larger
batch arrives).  It keeps its scratch in a fixed library-resident device
array instead.  These tests check it against x2g_relax on the same inputs,
FP64 results bit for bit equal as in the other sweep tests:

* all Coulomb and exchange potentials of one Ne orbital (right-hand sides
  built on the device in that scratch), two calls in a row;
* 72 potentials, which run as three launches of at most 32 jobs in the
  scratch (the per-launch barrier reset and the right-hand-side offsets of
  the later launches);
* the largest batch that fits the 32 MiB array is accepted, one more job is
  refused with an error;
* a device wait timeout in any launch of a call is returned, and the next
  call succeeds.

This file is collected last on purpose (test_zz_*).
"""
import numpy as np
import pytest

import x2dhf_gb300 as xg
from conftest import golden_deck
from oracle.pyoracle import Case

pytestmark = pytest.mark.gpu

SCRATCH = 32 << 20   # bytes of the library-resident array
JOB_ENTRY = 112      # bytes per job-table entry (documented in include/x2dhf_gpu.h)


def _potential_specs(oc, c, n=None, iorb=1):
    """(in1, in2, idel, isym, initial extended potential) of orbital iorb's
    potentials, or, with n, of n potentials taken round the orbitals."""
    specs = []
    while True:
        for k in range(1, oc.npots(iorb) + 1):
            in1, in2, idel, isym = oc.pot_info(iorb, k)
            specs.append((in1, in2, idel, isym, oc.putin(isym, oc.pot(iorb, k))))
        if n is None:
            return specs
        if len(specs) >= n:
            return specs[:n]
        iorb = iorb % oc.norb + 1


def _device_batch(torch, oc, c, specs, omega):
    dev = torch.device("cuda:0")
    orbs = {i: torch.tensor(oc.putin(1 if c.m[i - 1] % 2 == 0 else -1, oc.orbital(i)), device=dev)
            for i in range(1, oc.norb + 1)}
    bufs = [torch.tensor(s[4], device=dev) for s in specs]
    jobs = [xg.Job(u=u.data_ptr(), psa=orbs[a].data_ptr(), psb=orbs[b].data_ptr(), omega=omega, isym=s, idel=d, kind=1)
            for u, (a, b, d, s, _) in zip(bufs, specs)]
    return orbs, bufs, jobs


def _setup():
    torch = pytest.importorskip("torch")
    deck = golden_deck("ne_set01")
    oc = Case(deck)
    c = xg.parse_deck(deck)
    ctx = xg.Context(0)
    grid = xg.Grid(ctx, c.nnu, c.nmu, c.r, c.rinf, c.z1, c.z2)
    return torch, oc, c, ctx, grid


def _scratch_need(c, njobs):
    plain = (c.nnu * c.nmu * 8 + 255) // 256 * 256
    return 256 + (JOB_ENTRY * njobs + 255) // 256 * 256 + plain * njobs


def test_noalloc_matches_relax_two_calls():
    torch, oc, c, ctx, grid = _setup()
    specs = _potential_specs(oc, c)
    omega = oc.omega()[1]
    orbs, ref_bufs, ref_jobs = _device_batch(torch, oc, c, specs, omega)
    orbs2, new_bufs, new_jobs = _device_batch(torch, oc, c, specs, omega)
    torch.cuda.synchronize()
    for call in range(2):
        xg.relax(ctx, grid, ref_jobs, 10, xg.FP64)
        ctx.synchronize()
        xg.relax_noalloc(ctx, grid, new_jobs, 10)
        for k, (a, b) in enumerate(zip(ref_bufs, new_bufs)):
            assert torch.equal(a, b), (call, k, (a - b).abs().max().item())
    grid.close()
    ctx.close()


def test_noalloc_multi_launch_batch_matches_relax():
    torch, oc, c, ctx, grid = _setup()
    specs = _potential_specs(oc, c, n=72)
    omega = oc.omega()[1]
    orbs, ref_bufs, ref_jobs = _device_batch(torch, oc, c, specs, omega)
    orbs2, new_bufs, new_jobs = _device_batch(torch, oc, c, specs, omega)
    torch.cuda.synchronize()
    xg.relax(ctx, grid, ref_jobs, 10, xg.FP64)
    ctx.synchronize()
    xg.relax_noalloc(ctx, grid, new_jobs, 10)
    for k, (a, b) in enumerate(zip(ref_bufs, new_bufs)):
        assert torch.equal(a, b), (k, (a - b).abs().max().item())
    grid.close()
    ctx.close()


def test_noalloc_size_limit_exact_fit():
    torch, oc, c, ctx, grid = _setup()
    nfit = 1
    while _scratch_need(c, nfit + 1) <= SCRATCH:
        nfit += 1
    assert nfit > 72
    specs = _potential_specs(oc, c, n=nfit + 1)
    omega = oc.omega()[1]
    orbs, bufs, jobs = _device_batch(torch, oc, c, specs, omega)
    torch.cuda.synchronize()
    with pytest.raises(xg.X2GError) as ei:
        xg.relax_noalloc(ctx, grid, jobs, 10)
    assert ei.value.code == 1 and "scratch" in str(ei.value)
    xg.relax_noalloc(ctx, grid, jobs[:nfit], 10)
    grid.close()
    ctx.close()


def test_noalloc_reports_timeout_then_recovers():
    torch, oc, c, ctx, grid = _setup()
    specs = _potential_specs(oc, c, n=40)
    omega = oc.omega()[1]
    orbs, ref_bufs, ref_jobs = _device_batch(torch, oc, c, specs, omega)
    torch.cuda.synchronize()
    xg.relax(ctx, grid, ref_jobs, 10, xg.FP64)
    ctx.synchronize()
    orbs1, bufs1, jobs1 = _device_batch(torch, oc, c, specs, omega)
    torch.cuda.synchronize()
    ctx.set_wait_limit(0.0)
    with pytest.raises(xg.X2GError) as ei:
        xg.relax_noalloc(ctx, grid, jobs1, 10)
    assert ei.value.code == 4, str(ei.value)
    ctx.set_wait_limit(2.0)
    orbs2, bufs2, jobs2 = _device_batch(torch, oc, c, specs, omega)
    torch.cuda.synchronize()
    xg.relax_noalloc(ctx, grid, jobs2, 10)
    for k, (a, b) in enumerate(zip(ref_bufs, bufs2)):
        assert torch.equal(a, b), (k, (a - b).abs().max().item())
    grid.close()
    ctx.close()
