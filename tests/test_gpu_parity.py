"""GPU parity: the CUDA path against the CPU oracle on the same inputs.

Sweeps are compared bit for bit (the FP64 kernel reproduces the
single-thread MCSOR order and the reference's unfused arithmetic); SCF
results within the stated tolerances (reduction order differs)."""
import numpy as np
import pytest

import x2dhf_gb300 as xg
from conftest import golden_deck, golden_json
from oracle.pyoracle import Case, with_hydrogen0

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = xg.Context(0)
    yield c
    c.close()


def _all_mcsor(deck):
    """The GPU relaxes orbitals and potentials with MCSOR; the oracle does the
    same with the mcsor and mcsor-ce cards."""
    lines = [ln for ln in deck.splitlines() if not ln.strip().lower().startswith(("mcsor", "stop"))]
    return "\n".join(lines + ["mcsor", "mcsor-ce", "stop"]) + "\n"


def _grid(ctx, deck):
    c = xg.parse_deck(deck)
    return c, xg.Grid(ctx, c.nnu, c.nmu, c.r, c.rinf, c.z1, c.z2)


ORB_CASES = [("he_set01", 1), ("h2_set01", 1), ("ne_set01", 1), ("ne_set01", 4), ("h_set04", 1)]


@pytest.mark.parametrize("name,iorb", ORB_CASES)
@pytest.mark.parametrize("nsweeps", [1, 10])
def test_orbital_mcsor_bitexact(ctx, name, iorb, nsweeps):
    deck = golden_deck(name)
    oc = Case(deck)
    c, g = _grid(ctx, deck)
    f1, f2 = oc.fock(iorb)
    diag = oc.coeffs()[5]
    lhs, rhs = f1 + diag, f2.copy()
    isym = 1 if c.m[iorb - 1] % 2 == 0 else -1
    uext = oc.putin(isym, oc.orbital(iorb))
    omega = oc.omega()[0]
    ref = oc.sweep(1, isym, nsweeps, omega, uext, lhs, rhs, oc.suppl(0), oc.suppl(2))
    got = xg.mcsor_host(ctx, g, isym, 0, omega, nsweeps, uext.copy(), lhs, rhs)
    assert np.array_equal(got, ref), np.abs(got - ref).max()


@pytest.mark.parametrize("name,iorb", [("he_set01", 1), ("ne_set01", 1), ("ne_set01", 2)])
def test_potential_mcsor_bitexact(ctx, name, iorb):
    deck = golden_deck(name)
    oc = Case(deck)
    c, g = _grid(ctx, deck)
    e, f3, gg = oc.suppl(3), oc.suppl(7), oc.suppl(9)
    for k in range(1, oc.npots(iorb) + 1):
        in1, in2, idel, isym = oc.pot_info(iorb, k)
        rhs = (oc.orbital(in1) * oc.orbital(in2)) * gg
        lhs = f3.copy() if idel == 0 else f3 + float(idel * idel) * e
        uext = oc.putin(isym, oc.pot(iorb, k))
        omega = oc.omega()[1]
        ref = oc.sweep(1, isym, 10, omega, uext, lhs, rhs, oc.suppl(1), oc.suppl(2))
        got = xg.mcsor_host(ctx, g, isym, 1, omega, 10, uext.copy(), lhs, rhs)
        assert np.array_equal(got, ref), (k, np.abs(got - ref).max())


def test_batched_potentials_from_orbitals_bitexact(ctx):
    """All potentials of one orbital in one launch, rhs built on the device."""
    torch = pytest.importorskip("torch")
    deck = golden_deck("ne_set01")
    oc = Case(deck)
    c, g = _grid(ctx, deck)
    iorb = 1
    dev = torch.device("cuda:0")
    orbs = {i: torch.tensor(oc.putin(1 if c.m[i - 1] % 2 == 0 else -1, oc.orbital(i)), device=dev)
            for i in range(1, oc.norb + 1)}
    jobs, bufs, refs = [], [], []
    omega = oc.omega()[1]
    for k in range(1, oc.npots(iorb) + 1):
        in1, in2, idel, isym = oc.pot_info(iorb, k)
        u = torch.tensor(oc.putin(isym, oc.pot(iorb, k)), device=dev)
        bufs.append(u)
        jobs.append(xg.Job(u=u.data_ptr(), psa=orbs[in1].data_ptr(), psb=orbs[in2].data_ptr(), omega=omega,
                           isym=isym, idel=idel, kind=1))
        oc.relax_pot(iorb, k, 1)
        refs.append(oc.putin(isym, oc.pot(iorb, k)))
    torch.cuda.synchronize()
    xg.relax(ctx, g, jobs, 10)
    ctx.synchronize()
    n8 = c.nnu + 8
    for k, (u, ref) in enumerate(zip(bufs, refs)):
        got = u.cpu().numpy().reshape(c.nmu + 8, n8)[4:c.nmu + 4, 4:c.nnu + 4]
        exp = ref.reshape(c.nmu + 8, n8)[4:c.nmu + 4, 4:c.nnu + 4]
        assert np.array_equal(got, exp), (k, np.abs(got - exp).max())


def test_mixed_relaxation_tracks_fp64(ctx):
    """FP32 sweeps + FP64 defect correction stay within FP32 rounding of the FP64 result."""
    deck = golden_deck("he_set01")
    oc = Case(deck)
    c, g = _grid(ctx, deck)
    f1, f2 = oc.fock(1)
    lhs, rhs = f1 + oc.coeffs()[5], f2.copy()
    uext = oc.putin(1, oc.orbital(1))
    omega = oc.omega()[0]
    exact = xg.mcsor_host(ctx, g, 1, 0, omega, 10, uext.copy(), lhs, rhs)
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    u = torch.tensor(uext, device=dev)
    dl, dr = torch.tensor(lhs, device=dev), torch.tensor(rhs, device=dev)
    torch.cuda.synchronize()  # the context's stream is not ordered after torch's
    xg.relax(ctx, g, [xg.Job(u=u.data_ptr(), lhs=dl.data_ptr(), rhs=dr.data_ptr(), omega=omega, isym=1, kind=0)],
             10, xg.MIXED)
    ctx.synchronize()
    got = u.cpu().numpy()
    change = np.abs(exact - uext).max()
    assert np.abs(got - exact).max() <= 1e-5 * change + 1e-14


@pytest.mark.parametrize("name", ["he_set01", "ne_set01", "h2_set01"])
def test_mixed_on_chip_matches_persistent_band_path(ctx, name):
    """The cluster (distributed shared memory) FP32 sweep and the
    persistent-band FP32 sweep run the same schedule on the same (residual,
    omega/lhs) pairs, so they agree to FP32 rounding of the correction (the
    same bound as mixed vs FP64 above)."""
    torch = pytest.importorskip("torch")
    deck = golden_deck(name)
    oc = Case(deck)
    c, g = _grid(ctx, deck)
    f1, f2 = oc.fock(1)
    lhs, rhs = f1 + oc.coeffs()[5], f2.copy()
    isym = 1 if c.m[0] % 2 == 0 else -1
    uext = oc.putin(isym, oc.orbital(1))
    omega = oc.omega()[0]
    dev = torch.device("cuda:0")
    dl, dr = torch.tensor(lhs, device=dev), torch.tensor(rhs, device=dev)
    out = []
    for on_chip in (True, False):
        ctx.set_mixed_on_chip(on_chip)
        u = torch.tensor(uext, device=dev)
        torch.cuda.synchronize()
        xg.relax(ctx, g, [xg.Job(u=u.data_ptr(), lhs=dl.data_ptr(), rhs=dr.data_ptr(), omega=omega, isym=isym,
                                 kind=0)], 10, xg.MIXED)
        ctx.synchronize()
        out.append(u.cpu().numpy())
    ctx.set_mixed_on_chip(True)
    change = np.abs(out[1] - uext).max()
    assert np.abs(out[0] - out[1]).max() <= 1e-5 * change


@pytest.mark.parametrize("name", ["ne_set01", "h2_set01"])
def test_potential_cluster_variant_tracks_fp64(ctx, name):
    """Every potential of the case in one mixed-form launch, through the
    cluster kernel and through its potentials' variant (two CTAs per SM,
    residual only on chip, omega/lhs from the row term f3 + idel^2 e_mu and
    the column term idel^2 e_nu): both stay within FP32 rounding of the FP64
    sweep's change, Coulomb (idel 0) and exchange (idel > 0) potentials
    alike.  The start is one FP64 sweep from the deck's initial potentials,
    so that the axis values are the extrapolation of the interior, as after
    any relaxation: the mixed form extrapolates the correction on the axis,
    which equals extrapolating u only for such a start."""
    torch = pytest.importorskip("torch")
    deck = golden_deck(name)
    oc = Case(deck)
    c, g = _grid(ctx, deck)
    dev = torch.device("cuda:0")
    orbs = {i: torch.tensor(oc.putin(1 if c.m[i - 1] % 2 == 0 else -1, oc.orbital(i)), device=dev)
            for i in range(1, oc.norb + 1)}
    omega = oc.omega()[1]
    specs = []
    for iorb in range(1, oc.norb + 1):
        for k in range(1, oc.npots(iorb) + 1):
            in1, in2, idel, isym = oc.pot_info(iorb, k)
            specs.append((in1, in2, idel, isym, oc.putin(isym, oc.pot(iorb, k))))
    assert len({s[2] for s in specs}) >= (2 if name == "ne_set01" else 1)

    def run(precision, variant, start=None, nsweeps=10):
        bufs = [torch.tensor(s[4], device=dev) for s in specs] if start is None else \
            [torch.tensor(x, device=dev) for x in start]
        jobs = [xg.Job(u=u.data_ptr(), psa=orbs[a].data_ptr(), psb=orbs[b].data_ptr(), omega=omega, isym=sy,
                       idel=d, kind=1) for u, (a, b, d, sy, _) in zip(bufs, specs)]
        ctx.set_potential_clusters(variant)
        torch.cuda.synchronize()
        xg.relax(ctx, g, jobs, nsweeps, precision)
        ctx.synchronize()
        return [u.cpu().numpy() for u in bufs]

    def grid_part(x):
        # the nu x mu points the caller reads back (putout): the ghost cells
        # are refreshed from the interior at the start of an FP64 call, and
        # only read as mirrored interior values by the mixed form
        return x.reshape(c.nmu + 8, c.nnu + 8)[4:c.nmu + 4, 4:c.nnu + 4]

    start = run(xg.FP64, False, nsweeps=1)
    exact = [grid_part(x) for x in run(xg.FP64, False, start)]
    plain = [grid_part(x) for x in run(xg.MIXED, False, start)]
    pair = [grid_part(x) for x in run(xg.MIXED, True, start)]
    ctx.set_potential_clusters("auto")
    for k, (e, a, b, u0, s) in enumerate(zip(exact, plain, pair, [grid_part(x) for x in start], specs)):
        change = np.abs(e - u0).max()
        assert change > 0
        assert np.abs(a - e).max() <= 1e-5 * change + 1e-14, (k, s[2], np.abs(a - e).max() / change)
        assert np.abs(b - e).max() <= 1e-5 * change + 1e-14, (k, s[2], np.abs(b - e).max() / change)


@pytest.mark.parametrize("variant", [False, True])
def test_free_colouring_tracks_oracle_sweep(ctx, variant):
    """The seam-free colouring of the mixed form's cluster sweep, plain kernel
    and potentials' variant, against the oracle's FP64 sweep in the same
    colouring (mode 2): every potential of Ne (idel 0, 1 and 2), one launch,
    within FP32 rounding of the change; a start from one FP64 sweep (axis
    consistent with the interior), the nu x mu points compared."""
    torch = pytest.importorskip("torch")
    deck = golden_deck("ne_set01")
    oc = Case(deck)
    c, g = _grid(ctx, deck)
    dev = torch.device("cuda:0")
    orbs = {i: torch.tensor(oc.putin(1 if c.m[i - 1] % 2 == 0 else -1, oc.orbital(i)), device=dev)
            for i in range(1, oc.norb + 1)}
    omega = oc.omega()[1]
    e, f3, gg = oc.suppl(3), oc.suppl(7), oc.suppl(9)
    specs, starts, refs = [], [], []
    for iorb in range(1, oc.norb + 1):
        for k in range(1, oc.npots(iorb) + 1):
            in1, in2, idel, isym = oc.pot_info(iorb, k)
            rhs = (oc.orbital(in1) * oc.orbital(in2)) * gg
            lhs = f3.copy() if idel == 0 else f3 + float(idel * idel) * e
            u1 = oc.sweep(1, isym, 1, omega, oc.putin(isym, oc.pot(iorb, k)), lhs, rhs, oc.suppl(1), oc.suppl(2))
            # ghosts refreshed from the swept interior, as every relaxation starts
            u1 = oc.putin(isym, u1.reshape(c.nmu + 8, c.nnu + 8)[4:c.nmu + 4, 4:c.nnu + 4].ravel())
            specs.append((in1, in2, idel, isym))
            starts.append(u1)
            refs.append(oc.sweep(2, isym, 10, omega, u1, lhs, rhs, oc.suppl(1), oc.suppl(2)))
    bufs = [torch.tensor(x, device=dev) for x in starts]
    jobs = [xg.Job(u=u.data_ptr(), psa=orbs[a].data_ptr(), psb=orbs[b].data_ptr(), omega=omega, isym=sy, idel=d,
                   kind=1) for u, (a, b, d, sy) in zip(bufs, specs)]
    ctx.set_mixed_colouring("free")
    ctx.set_potential_clusters(variant)
    torch.cuda.synchronize()
    try:
        xg.relax(ctx, g, jobs, 10, xg.MIXED)
        ctx.synchronize()
    finally:
        ctx.set_mixed_colouring("reference")
        ctx.set_potential_clusters("auto")

    def part(x):
        return x.reshape(c.nmu + 8, c.nnu + 8)[4:c.nmu + 4, 4:c.nnu + 4]

    for k, (u, ref, u0, sp) in enumerate(zip(bufs, refs, starts, specs)):
        got, exp, st = part(u.cpu().numpy()), part(ref), part(u0)
        change = np.abs(exp - st).max()
        assert change > 0
        assert np.abs(got - exp).max() <= 1e-5 * change + 1e-14, (k, sp[2], np.abs(got - exp).max() / change)


def test_residual_overlap_is_bit_identical(ctx):
    """A potential batch larger than one wave of the potentials' cluster
    variant (32 seeded Slater-product sources on 331x481, where 14 such
    clusters are co-resident: waves of 14, 14 and 4): with the overlap, the
    later waves' FP64 residuals run on the auxiliary stream beside the
    earlier waves' sweeps; the kernels and their inputs are the same, so
    every result equals the batch without it bit for bit."""
    torch = pytest.importorskip("torch")
    import bench

    nnu, nmu, r, rinf = 331, 481, 2.0, 40.0
    g = xg.Grid(ctx, nnu, nmu, r, rinf, 1.0, 1.0)
    plain, pot = g.cluster_occupancy()
    B = 32
    assert 0 < pot < B
    dev = torch.device("cuda:0")
    n8, m8 = nnu + 8, nmu + 8
    omega = bench.C_double_pair(xg, nnu, nmu)[1]
    pairs = []
    for pa, pb in bench.slater_sources(rinf, nnu, nmu, r, B):
        ua = torch.zeros(m8, n8, dtype=torch.float64, device=dev)
        ub = torch.zeros_like(ua)
        ua[4:nmu + 4, 4:nnu + 4] = torch.from_numpy(pa[0])
        ub[4:nmu + 4, 4:nnu + 4] = torch.from_numpy(pb[0])
        pairs.append((ua, ub, abs(pa[1] - pb[1])))

    def run(overlap):
        us = [torch.zeros(m8, n8, dtype=torch.float64, device=dev) for _ in pairs]
        jobs = [xg.Job(u=u.data_ptr(), psa=ua.data_ptr(), psb=ub.data_ptr(), omega=omega,
                       isym=1 if d % 2 == 0 else -1, idel=d, kind=1) for u, (ua, ub, d) in zip(us, pairs)]
        ctx.set_residual_overlap(overlap)
        torch.cuda.synchronize()
        for _ in range(3):
            xg.relax(ctx, g, jobs, 10, xg.MIXED)
        ctx.synchronize()
        return us

    try:
        a = run(False)
        b = run(True)
    finally:
        ctx.set_residual_overlap(True)
    assert max(float(x.abs().max()) for x in a) > 0
    for k, (x, y) in enumerate(zip(a, b)):
        assert torch.equal(x, y), k
    g.close()


def _scf_records_match(name, niter, transform=None, tol=1e-11, batch_mode=0):
    deck = golden_deck(name)
    if transform:
        deck = transform(deck)
    deck = _all_mcsor(deck)
    oc = Case(deck)
    oc.set_batch_potentials(batch_mode)
    oc.steps(niter)
    ctx = xg.Context(0)
    s = xg.SCF(ctx, xg.parse_deck(deck, batch_mode=batch_mode))
    s.run(niter)
    ro, rg = oc.records(), s.records()
    assert len(ro) == len(rg)
    for a, b in zip(ro, rg):
        assert a[:2] == b[:2]
        assert abs(a[2] - b[2]) <= tol * max(1.0, abs(a[2])), (a, b)
    s.close()
    ctx.close()


def test_scf_he_trajectory_matches_oracle():
    _scf_records_match("he_set02", 40, with_hydrogen0)


def test_scf_h2_trajectory_matches_oracle():
    _scf_records_match("h2_set01", 40)


def test_scf_ne_trajectory_matches_oracle():
    _scf_records_match("ne_set01", 25)


def _kf_small(deck):
    """KF (Z=19,9, R=4.1035, 3 pi + 8 sigma) on a 241x301 grid, R_inf=60
    (coarser grids let the first iterations from the hydrogenic start blow
    up to 1e+250, where no two summation orders agree)."""
    out = []
    for ln in deck.splitlines():
        key = ln.strip().lower()
        if key.startswith("grid"):
            ln = "grid 241 301 60.0"
        if key.startswith(("mmoments", "conv", "!")):
            continue
        out.append(ln)
    return "\n".join(out) + "\n"


def test_scf_kf_trajectory_matches_oracle():
    """11 orbitals incl. pi-pi exchange pairs (two potentials each),
    heteronuclear: 72 potentials per SCF iteration."""
    _scf_records_match("kf_set01", 5, _kf_small)


@pytest.mark.parametrize("batch_mode", [1, 2])
def test_scf_batched_trajectory_matches_oracle(batch_mode):
    """All potentials of an iteration in one launch (1), and all orbitals in
    one more (2): the GPU follows the oracle's run of the same mode."""
    _scf_records_match("ne_set01", 25, batch_mode=batch_mode)


@pytest.mark.parametrize("batch_mode", [1, 2])
def test_scf_kf_batched_trajectory_matches_oracle(batch_mode):
    """KF's 72 potentials in one call (three launches of at most 32 jobs)
    and its 11 orbitals in one launch."""
    _scf_records_match("kf_set01", 5, _kf_small, batch_mode=batch_mode)


def test_gram_orthonormalise_matches_rounds():
    """Batch mode 2 orthonormalises an iteration's orbitals in rounds with
    the loop's own sums by default, or through their Gram matrix.  Equal in
    exact arithmetic: N2 (331x481, mixed) solved both ways lands on the same
    energies, and Ne in FP64 follows the same trajectory for 60 iterations
    past its frozen-orbital start."""
    import bench

    ctx = xg.Context(0)
    out = {}
    for gram in (True, False):
        ctx.set_gram_orthonormalise(gram)
        s = xg.SCF(ctx, xg.parse_deck(bench.n2_deck(), precision=xg.MIXED, batch_mode=2))
        r = s.run()
        out[gram] = (r.iterations, r.total_energy, [r.ee[i] for i in range(6)])
        s.close()
    # each exits at its own iteration of the same converging trajectory: the
    # energies agree to the exit's own accuracy, and both lie within the
    # tolerance of the FP64 oracle solved to 1000 iterations
    ref = golden_json("n2_331x481_oracle")["total_energy"]
    for gram in (True, False):
        assert abs(out[gram][1] - ref) < 1e-9, (gram, out[gram][1], ref)
    assert abs(out[True][1] - out[False][1]) < 5e-10, out
    assert max(abs(a - b) for a, b in zip(out[True][2], out[False][2])) < 5e-10, out
    assert abs(out[True][0] - out[False][0]) <= 30, out
    recs = {}
    deck = _all_mcsor(golden_deck("ne_set01"))
    for gram in (True, False):
        ctx.set_gram_orthonormalise(gram)
        s = xg.SCF(ctx, xg.parse_deck(deck, batch_mode=2))
        s.run(80)
        recs[gram] = s.records()
        s.close()
    ctx.set_gram_orthonormalise(False)
    assert len(recs[True]) == len(recs[False]) > 0
    for a, b in zip(recs[True], recs[False]):
        assert a[:2] == b[:2]
        assert abs(a[2] - b[2]) <= 1e-11 * max(1.0, abs(a[2])), (a, b)
    ctx.close()


def test_scf_he_converged_energy_vs_golden():
    """He MCSOR converged to 1e-12: the reference's own final energy."""
    deck = _all_mcsor(with_hydrogen0(golden_deck("he_set02")))
    ctx = xg.Context(0)
    s = xg.SCF(ctx, xg.parse_deck(deck))
    res = s.run()
    g = golden_json("he_set02")
    assert abs(res.total_energy - g["total_energy"]) < 1e-10
    s.close()
    ctx.close()


def test_scf_he_mixed_converges_to_fp64():
    deck = _all_mcsor(with_hydrogen0(golden_deck("he_set02")))
    ctx = xg.Context(0)
    e = {}
    for prec in (xg.FP64, xg.MIXED):
        s = xg.SCF(ctx, xg.parse_deck(deck, precision=prec))
        e[prec] = s.run().total_energy
        s.close()
    assert abs(e[xg.MIXED] - e[xg.FP64]) < 1e-9
    ctx.close()


def test_integer_pipe_conversions_match_hardware(ctx):
    """The mixed form narrows its FP64 residual and widens its FP32 correction
    with integer operations; they equal the hardware conversions bit for bit
    (NaN to NaN) on edge cases and 16M hashed bit patterns, outside the float
    subnormal range that they flush to zero."""
    assert ctx.convert_selftest(1 << 24, seed=12345) == 0


def _initial_functions_match(deck, rtol=1e-13):
    """Every orbital, Coulomb and exchange potential of the hydrogenic /
    Thomas-Fermi start (initOrbitalsPotentials.F90:714-934,
    coulombExchangePotentials.f90:14-239), evaluated on the device, against
    the oracle's start on the same grid; device exp/pow may differ from the
    host's in the last bit, so the bound is relative to each function's
    largest value."""
    oc = Case(deck)
    ctx = xg.Context(0)
    s = xg.SCF(ctx, xg.parse_deck(_all_mcsor(deck)))
    m = [int(s.case.m[i]) for i in range(s.case.norb)]
    checked = 0
    for i in range(1, s.case.norb + 1):
        ref, got = oc.orbital(i), s.function(0, i)
        assert np.max(np.abs(got - ref)) <= rtol * np.max(np.abs(ref)), ("orbital", i)
        checked += 1
    for iorb in range(1, s.case.norb + 1):
        for k in range(1, oc.npots(iorb) + 1):
            in1, in2, idel, _ = oc.pot_info(iorb, k)
            if in1 == in2 and idel == 0:
                got = s.function(1, in1)
            else:
                a, b = min(in1, in2), max(in1, in2)
                second = a != b and m[a - 1] > 0 and m[b - 1] > 0 and idel == m[a - 1] + m[b - 1]
                got = s.function(2, a, b, 1 if second else 0)
            ref = oc.pot(iorb, k)
            assert np.max(np.abs(got - ref)) <= rtol * max(np.max(np.abs(ref)), 1e-300), (iorb, k, in1, in2, idel)
            checked += 1
    assert checked > s.case.norb
    s.close()
    ctx.close()


def test_initial_guess_n2_matches_oracle():
    """N2: sigma and pi orbitals on both centres, pi-pi exchange pairs."""
    _initial_functions_match(golden_deck("n2_set01"))


def test_initial_guess_kf_matches_oracle():
    """KF: heteronuclear, 3 pi + 8 sigma, n up to 4 (Laguerre and Legendre
    series of several terms)."""
    _initial_functions_match(_kf_small(golden_deck("kf_set01")))


def test_initial_guess_lih_matches_oracle():
    _initial_functions_match(golden_deck("lih_set01"))


def test_mixed_persistent_sweep_scf_matches_on_chip():
    """KF on 241x301 in the mixed form, once with the cluster sweep and once
    with the persistent-band sweep (batches of 32 potentials in bands of
    several tiles per block, single orbitals one tile per block): both sweep
    the same schedule, so the SCF records agree to the FP32 rounding of the
    corrections, far below the FP64 defect-corrected energies."""
    deck = _all_mcsor(_kf_small(golden_deck("kf_set01")))
    ctx = xg.Context(0)
    recs = []
    for on_chip in (True, False):
        ctx.set_mixed_on_chip(on_chip)
        s = xg.SCF(ctx, xg.parse_deck(deck, precision=xg.MIXED))
        s.run(4)
        recs.append(s.records())
        s.close()
    ctx.set_mixed_on_chip(True)
    assert len(recs[0]) == len(recs[1]) > 0
    for a, b in zip(*recs):
        assert a[:2] == b[:2]
        assert abs(a[2] - b[2]) <= 1e-9 * max(1.0, abs(a[2])), (a, b)
    ctx.close()


def test_mixed_persistent_sweep_batches_track_fp64():
    """20 potentials on 541x721 (no cluster plan): the persistent-band sweep
    takes them in two launches of at most 16 (the most whose bands fit the
    GPU's shared memory two blocks per SM), and every result stays within
    FP32 rounding of the FP64 sweep's change, as for a single job."""
    torch = pytest.importorskip("torch")
    import bench

    nnu, nmu, r, rinf = 541, 721, 2.0, 40.0
    assert xg.host_cluster_plan(nnu, nmu)[0] == 0
    ctx = xg.Context(0)
    g = xg.Grid(ctx, nnu, nmu, r, rinf, 1.0, 1.0)
    dev = torch.device("cuda:0")
    n8, m8 = nnu + 8, nmu + 8
    keep, out = [], {}
    for prec in (xg.FP64, xg.MIXED):
        jobs, us = [], []
        for pa, pb in bench.slater_sources(rinf, nnu, nmu, r, 20):
            ua = torch.zeros(m8, n8, dtype=torch.float64, device=dev)
            ub = torch.zeros_like(ua)
            ua[4:nmu + 4, 4:nnu + 4] = torch.from_numpy(pa[0])
            ub[4:nmu + 4, 4:nnu + 4] = torch.from_numpy(pb[0])
            u = torch.zeros_like(ua)
            idel = abs(pa[1] - pb[1])
            keep += [ua, ub]
            us.append(u)
            jobs.append(xg.Job(u=u.data_ptr(), psa=ua.data_ptr(), psb=ub.data_ptr(), omega=1.95,
                               isym=1 if idel % 2 == 0 else -1, idel=idel, kind=1))
        torch.cuda.synchronize()
        xg.relax(ctx, g, jobs, 10, prec)
        ctx.synchronize()
        out[prec] = [u.cpu().numpy() for u in us]
    for a, b in zip(out[xg.FP64], out[xg.MIXED]):
        change = np.abs(a).max()
        assert change > 0
        assert np.abs(a - b).max() <= 1e-5 * change
    ctx.close()




def test_gpu_start_matches_printed_initial_energies():
    """The GPU's hydrogenic start and prepSCF (device-evaluated LCAO
    orbitals and potential guesses, norms, orthogonalisation, moments,
    orbital energies, total energy) against the total energy the reference
    printed after its own start, for the closed-shell outputs of the current
    program version: He, Ne, Ca atoms and H2, He2, LiH, AlF, GaF (9 to 15
    orbitals for the fluorides)."""
    g = golden_json("initial_energies")
    ctx = xg.Context(0)
    checked = 0
    for rel, v in g.items():
        if v["group"] != "current":
            continue
        case = xg.parse_deck(_all_mcsor(v["deck"]))
        if any(case.occ[i] not in (2.0, 4.0) for i in range(case.norb)) and case.norb > 1:
            continue  # open shells: outside the closed-shell GPU path
        s = xg.SCF(ctx, case)
        e, ref = s.run(0).total_energy, v["initial_total_energy"]
        assert abs(e - ref) <= 2e-11 * abs(ref) + 1e-13, (rel, e, ref)
        s.close()
        checked += 1
    assert checked == 8
    ctx.close()


@pytest.mark.parametrize("name,iorb,kind", [("he_set01", 1, 0), ("h2_set01", 1, 0), ("ne_set01", 1, 0),
                                            ("ne_set01", 4, 0), ("ne_set01", 2, 1), ("ne_set01", 1, 1)])
@pytest.mark.parametrize("nsweeps", [1, 10])
def test_sor_bitexact(ctx, name, iorb, kind, nsweeps):
    """List-order SOR on the GPU (pipelined wavefront) against the oracle's
    sequential SOR over the middle list, orbitals (kind 0, explicit lhs/rhs)
    and potentials (kind 1, rhs = psa psb g formed on the device)."""
    torch = pytest.importorskip("torch")
    deck = golden_deck(name)
    oc = Case(deck)
    c, g = _grid(ctx, deck)
    dev = torch.device("cuda:0")
    if kind == 0:
        f1, f2 = oc.fock(iorb)
        lhs, rhs = f1 + oc.coeffs()[5], f2.copy()
        isym = -1 if c.m[iorb - 1] % 2 else 1
        uext = oc.putin(isym, oc.orbital(iorb))
        omega = oc.omega()[0]
        ref = oc.sweep(0, isym, nsweeps, omega, uext, lhs, rhs, oc.suppl(0), oc.suppl(2))
        u, dl, dr = (torch.tensor(x, device=dev) for x in (uext, lhs, rhs))
        jobs = [xg.Job(u=u.data_ptr(), lhs=dl.data_ptr(), rhs=dr.data_ptr(), omega=omega, isym=isym, kind=0)]
    else:
        in1, in2, idel, isym = oc.pot_info(iorb, 1)
        rhs = (oc.orbital(in1) * oc.orbital(in2)) * oc.suppl(9)
        lhs = oc.suppl(7).copy() if idel == 0 else oc.suppl(7) + float(idel * idel) * oc.suppl(3)
        uext = oc.putin(isym, oc.pot(iorb, 1))
        omega = oc.omega()[1]
        ref = oc.sweep(0, isym, nsweeps, omega, uext, lhs, rhs, oc.suppl(1), oc.suppl(2))
        orbs = {i: torch.tensor(oc.putin(1 if c.m[i - 1] % 2 == 0 else -1, oc.orbital(i)), device=dev)
                for i in (in1, in2)}
        u = torch.tensor(uext, device=dev)
        jobs = [xg.Job(u=u.data_ptr(), psa=orbs[in1].data_ptr(), psb=orbs[in2].data_ptr(), omega=omega, isym=isym,
                       idel=idel, kind=1)]
    torch.cuda.synchronize()
    xg.relax(ctx, g, jobs, nsweeps, xg.SOR)
    ctx.synchronize()
    got = u.cpu().numpy()
    n8 = c.nnu + 8
    # the relaxed function: interior, axis rows/columns and the fixed rows
    sl = np.s_[4:c.nmu + 4, 4:c.nnu + 4]
    a, b = got.reshape(c.nmu + 8, n8)[sl], ref.reshape(c.nmu + 8, n8)[sl]
    assert np.abs(b - uext.reshape(c.nmu + 8, n8)[sl]).max() > 0
    assert np.array_equal(a, b), np.abs(a - b).max()


# the reference's own SOR decks, run on the GPU as the reference ran them
SOR_GOLDEN = [("h2_set01", None), ("he_set01", with_hydrogen0), ("he_set02", with_hydrogen0)]


@pytest.mark.parametrize("name,transform", SOR_GOLDEN)
def test_scf_sor_decks_reproduce_reference_trajectory(name, transform):
    """Decks without the mcsor-ce card relax potentials (and, without mcsor,
    orbitals) with list-order SOR, as the reference does; the GPU run
    reproduces every orbital-energy line the reference printed, its
    iteration count, its sweep count and its final energy (he/set-02: MCSOR
    orbitals, SOR potentials)."""
    deck = golden_deck(name)
    if transform:
        deck = transform(deck)
    g = golden_json(name)
    ctx = xg.Context(0)
    s = xg.SCF(ctx, xg.parse_deck(deck))
    r = s.run()
    recs = s.records()
    assert len(recs) == len(g["records"]), (len(recs), len(g["records"]))
    for (it, io, ee, dee, dn), gr in zip(recs, g["records"]):
        assert it == gr[0]
        assert abs(ee - gr[2]) <= 1e-11 * max(1.0, abs(gr[2])), (it, ee, gr)
    assert abs(r.total_energy - g["total_energy"]) <= 1e-12 * abs(g["total_energy"])
    assert r.sweeps == g["sweeps"]
    s.close()
    ctx.close()


def test_scf_ne_sor_reproduces_reference_trajectory():
    """Ne (ne/set-01): 4 orbitals incl. 1pi, SOR for orbitals and potentials,
    1432 printed orbital-energy lines and 52540 sweeps."""
    test_scf_sor_decks_reproduce_reference_trajectory("ne_set01", None)
