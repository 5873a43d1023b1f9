"""CPU checks of the library's host-side setup (no GPU): operator tables
against the oracle, grid rounding, and the colour/level sweep schedule."""
import numpy as np
import pytest

import x2dhf_gb300 as xg
from conftest import golden_deck
from oracle.pyoracle import Case


@pytest.mark.parametrize("name", ["h2_set01", "he_set01", "ne_set01"])
def test_tables_bitwise_equal_oracle(name):
    oc = Case(golden_deck(name))
    c = xg.parse_deck(golden_deck(name))
    assert (c.nnu, c.nmu) == (oc.nni, oc.nmu)
    # table index map: library -> oracle (borb bpot d e f0 f1 f2 f3 f4 g wgt1 wgt2)
    omap = {0: 0, 1: 1, 2: 2, 3: 3, 4: 4, 5: 5, 6: 6, 7: 7, 8: 8, 9: 9, 10: 12, 11: 13}
    for which, ow in omap.items():
        a = xg.host_table(c.nnu, c.nmu, c.r, c.rinf, c.z1, c.z2, which)
        b = oc.suppl(ow)
        assert np.array_equal(a, b), which


def test_grid_rounding():
    assert [xg.round_grid(n) for n in (169, 241, 337, 481, 793, 1201, 505, 721)] == \
        [151, 241, 331, 481, 781, 1201, 481, 721]


def _check_schedule(nnu, nmu):
    order, pts, tile, col, lev = xg.host_schedule(nnu, nmu)
    n8 = nnu + 8
    npts = (nnu - 2) * (nmu - 5)
    assert order.size == npts == pts.size
    assert sorted(pts.tolist()) == sorted(order.tolist())
    pos = np.full(n8 * (nmu + 8), -1)
    pos[order] = np.arange(npts)
    # per point schedule data indexed by list position
    t_of = np.empty(npts, int); c_of = np.empty(npts, int); l_of = np.empty(npts, int)
    t_of[pos[pts]] = tile; c_of[pos[pts]] = col; l_of[pos[pts]] = lev
    assert (c_of == np.arange(npts) % 5).all()  # colour = list index mod 5
    # every same-colour stencil pair: same tile, later point has higher level
    npairs = 0
    for off in [1, 2, 3, 4, n8, 2 * n8, 3 * n8, 4 * n8]:
        q = order + off
        ok = q < pos.size
        pq = np.full(npts, -1)
        pq[ok] = pos[q[ok]]
        p = np.arange(npts)
        m = (pq >= 0) & (pq % 5 == p % 5)
        a, b = p[m], pq[m]
        first, second = np.minimum(a, b), np.maximum(a, b)
        assert (t_of[first] == t_of[second]).all()
        assert (l_of[second] > l_of[first]).all()
        npairs += m.sum()
    # tiles are row bands in ext rows [4, nmu); band 0 holds rows 4..9
    rows = order // n8
    assert rows.min() == 5 and rows.max() == nmu - 1
    return npairs


@pytest.mark.parametrize("nnu,nmu", [(31, 31), (91, 121), (151, 211), (151, 241), (331, 481), (781, 1201)])
def test_schedule_reproduces_single_thread_mcsor_order(nnu, nmu):
    npairs = _check_schedule(nnu, nmu)
    assert npairs > 0  # the "middle" ordering has seam conflicts to order


@pytest.mark.parametrize("nnu,nmu", [(31, 31), (91, 121), (151, 211), (151, 241), (331, 481)])
def test_cluster_plan_bands(nnu, nmu):
    """On-chip sweep plan: contiguous bands covering ext rows [4, nmu), band 0
    holds rows 4..9 (the mu=1 extrapolation), every band >= 4 rows (its halo
    is fed by the adjacent band only), shared memory within one SM."""
    C, maxrows, smem, row0 = xg.host_cluster_plan(nnu, nmu)
    assert 2 <= C <= 16
    assert row0[0] == 4 and row0[-1] == nmu
    heights = [b - a for a, b in zip(row0[:-1], row0[1:])]
    assert min(heights) >= 4 and row0[1] >= 10 and max(heights) == maxrows
    ch, off = xg.host_cluster_chunks(nnu, nmu)
    nseg = (off.size - 1) // (5 * C)
    maxchunks = max(off[(k + 1) * 5 * nseg] - off[k * 5 * nseg] for k in range(C))
    assert smem == (((maxrows + 8) + 2 * maxrows) * (nnu + 8) + maxrows + nnu + 8 + 5 * nseg + 1 + maxchunks) * 4
    assert smem <= 200 * 1024
    # every same-colour dependency lies inside one band (bands are unions of tiles)
    order, pts, tile, col, lev = xg.host_schedule(nnu, nmu)
    rows = pts // (nnu + 8)
    band = np.searchsorted(np.array(row0), rows, side="right") - 1
    for t in np.unique(tile):
        assert np.unique(band[tile == t]).size == 1


@pytest.mark.parametrize("nnu,nmu", [(31, 31), (91, 121), (151, 241), (331, 481)])
def test_free_colouring_chunks_cover_grid(nnu, nmu):
    """The seam-free plan of the mixed form's cluster sweep: every interior
    point exactly once, in its CTA's band, in the segment of its colour
    (col - row) mod 5 and kind (off the shared band edges, within 4 rows of
    one; the seam segment empty), chunks of up to 4 points of one row at
    stride 5; no two points of one colour are neighbours on the stencil's
    cross, so each colour is one parallel step."""
    C, maxrows, smem, row0 = xg.host_cluster_plan(nnu, nmu)
    ch, off = xg.host_cluster_chunks(nnu, nmu, colouring="free")
    S = 3
    assert off.size == C * 5 * S + 1 and off[-1] == ch.size
    n8 = nnu + 8
    seen = {}
    for k in range(C):
        for c in range(5):
            assert off[(k * 5 + c) * S + 2] == off[(k * 5 + c) * S + 3]
            for seg in range(2):
                o = (k * 5 + c) * S + seg
                for q in ch[off[o]:off[o + 1]]:
                    lr, cl, n = int(q >> 19), int((q >> 2) & 0x1FFFF), int(q & 3) + 1
                    row = row0[k] + lr
                    assert row0[k] <= row < row0[k + 1]
                    edge = (k > 0 and row < row0[k] + 4) or (k < C - 1 and row >= row0[k + 1] - 4)
                    assert edge == (seg == 1)
                    for j in range(n):
                        col = cl + 5 * j
                        assert (col - row) % 5 == c and (row, col) not in seen
                        seen[(row, col)] = c
    interior = {(r, q) for r in range(5, nmu) for q in range(5, nnu + 3)}
    assert set(seen) == interior
    for (r, q), c in seen.items():
        for d in range(1, 5):
            for nb in ((r + d, q), (r, q + d)):
                assert seen.get(nb, -1) != c


def test_schedule_cache_returns_the_built_schedules():
    """The sweep schedules depend on the grid size only and are kept in a
    process-wide cache of recent sizes: a size built again (after others in
    between, and more sizes than the cache holds) gives the same schedules."""
    first = {n: xg.host_cluster_chunks(*n) for n in [(151, 241), (331, 481)]}
    sor_first = xg.host_sor_schedule(331, 481)
    for n in [(91, 121), (121, 181), (181, 241), (211, 301), (241, 331), (271, 361), (301, 421), (361, 481),
              (331, 481), (151, 241)]:
        xg.host_cluster_chunks(*n)
    for n, (ch, off) in first.items():
        ch2, off2 = xg.host_cluster_chunks(*n)
        assert np.array_equal(ch, ch2) and np.array_equal(off, off2)
    for a, b in zip(sor_first[:4], xg.host_sor_schedule(331, 481)[:4]):
        assert np.array_equal(a, b)


def test_large_grid_has_no_cluster_plan():
    assert xg.host_cluster_plan(781, 1201)[0] == 0


@pytest.mark.parametrize("nnu,nmu", [(31, 31), (91, 121), (151, 241), (331, 481)])
def test_cluster_chunks_cover_schedule(nnu, nmu):
    """The on-chip sweep's chunks hold every scheduled point exactly once, in
    its CTA's band and in the segment of its colour and kind: level-0 points
    off the shared band edges, level-0 points within 4 rows of one, level-0
    seam points (a same-colour stencil neighbour has a higher level), then
    one segment per higher level.  A chunk is up to 4 points of one row at
    stride 5."""
    C, maxrows, smem, row0 = xg.host_cluster_plan(nnu, nmu)
    ch, off = xg.host_cluster_chunks(nnu, nmu)
    order, pts, tile, colour, lev = xg.host_schedule(nnu, nmu)
    nlev = int(lev.max()) + 1
    S = nlev + 2
    assert off.size == C * 5 * S + 1 and off[-1] == ch.size
    n8 = nnu + 8
    info = {int(p): (int(c), int(l)) for p, c, l in zip(pts, colour, lev)}
    offsets = [d for k in range(1, 5) for d in (k, -k, k * n8, -k * n8)]
    seam = set()
    for p, (c, l) in info.items():
        if l == 0 and any(info.get(p + d, (-1, 0))[0] == c and info[p + d][1] > 0 for d in offsets):
            seam.add(p)
    seen = set()
    for k in range(C):
        for c in range(5):
            for seg in range(S):
                o = (k * 5 + c) * S + seg
                for q in ch[off[o]:off[o + 1]]:
                    lr, cl, n = int(q >> 19), int((q >> 2) & 0x1FFFF), int(q & 3) + 1
                    row = row0[k] + lr
                    assert row0[k] <= row < row0[k + 1]
                    edge = (k > 0 and row < row0[k] + 4) or (k < C - 1 and row >= row0[k + 1] - 4)
                    for j in range(n):
                        p = row * n8 + cl + 5 * j
                        assert p in info and p not in seen
                        seen.add(p)
                        assert info[p][0] == c
                        if seg < 3:
                            assert info[p][1] == 0 and (p in seam) == (seg == 2)
                            if seg < 2:
                                assert edge == (seg == 1)
                        else:
                            assert info[p][1] == seg - 2
    assert len(seen) == len(info)


@pytest.mark.parametrize("nnu,nmu", [(31, 31), (91, 121), (241, 301), (331, 481), (541, 721), (781, 1201)])
def test_band_schedule_of_persistent_sweep(nnu, nmu):
    """The persistent-band sweep's schedule: every scheduled point once,
    grouped by colour, level and tile exactly as the sweep schedule assigns
    them; run heights with halos; the 16-byte pieces of a band's halos reach
    into its own rows only on ghost columns; every row inside another band's
    halo lies within 4 rows of its own band's edge (written back each
    phase); at most three runs on either side reach into a band's halos."""
    pts, off, rows, r0, r1, nlev = xg.host_band_schedule(nnu, nmu)
    order, ij, tile, colour, lev = xg.host_schedule(nnu, nmu)
    n8, m8 = nnu + 8, nmu + 8
    nt = len(r0)
    assert r0[0] == 4 and r1[-1] == nmu and (r0[1:] == r1[:-1]).all()
    ext = (pts >> 16) * n8 + (pts & 0xFFFF)
    assert np.array_equal(np.sort(ext), np.sort(ij))
    where = {int(p): (int(t), int(c), int(l)) for p, t, c, l in zip(ij, tile, colour, lev)}
    offs = off.reshape(5, nlev, nt + 1)
    for c in range(5):
        for l in range(nlev):
            for t in range(nt):
                for k in range(offs[c, l, t], offs[c, l, t + 1]):
                    assert where[int(ext[k])] == (t, c, l)
    assert offs[-1, -1, -1] == len(pts) and offs[0, 0, 0] == 0
    for G in range(1, 17):
        runs = [(int(r0[t0]), int(r1[min(t0 + G, nt) - 1])) for t0 in range(0, nt, G)]
        assert rows[G] == max(b - a for a, b in runs) + 8
        for k, (a, b) in enumerate(runs):
            f0, f1 = ((a - 4) * n8) >> 2, ((b + 4) * n8 + 3) >> 2
            fa, fb = (a * n8 + 3) >> 2, (b * n8) >> 2
            assert f0 >= 0 and 4 * f1 <= n8 * m8 and 4 * (f1 - f0) <= rows[G] * n8 + 8
            assert all(q // n8 == a and q % n8 < 4 for q in range(a * n8, 4 * fa))
            assert all(q // n8 == b - 1 and q % n8 >= nnu + 4 for q in range(4 * fb, b * n8))
            lo = a + 4 if k > 0 else a
            hi = b - 4 if k < len(runs) - 1 else b
            for j, (c0, c1) in enumerate(runs):
                if j == k:
                    continue
                for x in list(range(c1, c1 + 4)) + list(range(c0 - 4, c0)):
                    if a <= x < b:
                        assert x < lo or x >= hi
            up = [j for j in range(k) if runs[j][1] > a - 4]
            dn = [j for j in range(k + 1, len(runs)) if runs[j][0] < b + 4]
            assert up == list(range(k - len(up), k)) and dn == list(range(k + 1, k + 1 + len(dn)))
            assert len(up) <= 3 and len(dn) <= 3


@pytest.mark.parametrize("nnu,nmu", [(0, 0), (5, 5), (31, 11), (11, 31)])
def test_degenerate_grids_are_refused(nnu, nmu):
    """Grids too small for the 8th-order stencil's 4-point margins and the
    axis extrapolation are refused with a status code by every host-side
    schedule builder (no exception escapes the C ABI, nothing is built)."""
    for f in (xg.host_schedule, xg.host_band_schedule, xg.host_cluster_chunks):
        with pytest.raises(xg.X2GError) as err:
            f(nnu, nmu)
        assert err.value.code == 6


def test_parse_deck_relaxation_schemes_follow_the_cards():
    """read_mcsor / read_mcsor_o / read_mcsor_ce (inputInterface.F90:
    1910-2028): SOR by default; mcsor and mcsor-o select MCSOR for the
    orbitals, mcsor-ce for the potentials, and a later mcsor card puts the
    potentials back on SOR."""
    def schemes(deck):
        c = xg.parse_deck(deck)
        return c.orb_scheme, c.pot_scheme

    base = [ln for ln in golden_deck("h2_set01").splitlines() if ln.strip().lower() != "stop"]
    assert schemes("\n".join(base + ["stop"])) == (0, 0)
    assert schemes("\n".join(base + ["mcsor", "stop"])) == (1, 0)
    assert schemes("\n".join(base + ["mcsor-o", "stop"])) == (1, 0)
    assert schemes("\n".join(base + ["mcsor-ce", "stop"])) == (0, 1)
    assert schemes("\n".join(base + ["mcsor", "mcsor-ce", "stop"])) == (1, 1)
    assert schemes("\n".join(base + ["mcsor-ce", "mcsor", "stop"])) == (1, 0)
    c = xg.parse_deck("\n".join(base + ["mcsor-ce 1 7", "stop"]))
    assert c.maxsor_pot == 7


def _sor_wavefront(oc, sched, isym, nsweeps, omega, u0, lhs, rhs, b, d):
    """The GPU's list-order SOR schedule run as a parallel machine in numpy:
    every update of a step is computed from the state at the start of the
    step, then all are written (the reference's arithmetic order, no FMA)."""
    pts, off, bpts, boff, D = sched
    nni = oc.nni
    n8 = nni + 8
    dmu1, dmu2, dni1, dni2, ex, _ = oc.coeffs()
    u = u0.copy()
    ij_all = (pts >> 16) * n8 + (pts & 0xffff)
    ik_all = ((pts >> 16) - 4) * nni + ((pts & 0xffff) - 4)
    bij = (bpts >> 16) * n8 + (bpts & 0xffff)
    bst = np.where((bpts & 0xffff) == 4, 1, np.where((bpts & 0xffff) == nni + 3, -1, n8))
    NL, NB = len(off) - 1, len(boff) - 1
    for t in range((nsweeps - 1) * D + max(NL, NB)):
        writes = []
        for s in range(nsweeps):
            lv = t - s * D
            if lv < 0:
                break
            if lv < NL:
                ij, ik = ij_all[off[lv]:off[lv + 1]], ik_all[off[lv]:off[lv + 1]]

                def f(o):
                    return u[ij + o]

                def pair(c, st, sign):
                    a = [f(-k * st) + sign * f(k * st) for k in (4, 3, 2, 1)]
                    return ((c[0] * a[0] + c[1] * a[1]) + c[2] * a[2]) + c[3] * a[3]

                cc = ((pair(dmu2, n8, 1) + b[ik] * pair(dmu1, n8, -1)) + pair(dni2, 1, 1)) + d[ik] * pair(dni1, 1, -1)
                writes.append((ij, (omega * (rhs[ik] - cc)) / lhs[ik] + (1.0 - omega) * u[ij]))
            if lv < NB:
                ij, st = bij[boff[lv]:boff[lv + 1]], bst[boff[lv]:boff[lv + 1]]
                if isym == 1:
                    v = (((ex[0] * u[ij + st] + ex[1] * u[ij + 2 * st]) + ex[2] * u[ij + 3 * st])
                         + ex[3] * u[ij + 4 * st]) + ex[4] * u[ij + 5 * st]
                else:
                    v = np.zeros(ij.size)
                writes.append((ij, v))
        for ij, v in writes:
            u[ij] = v
    return u


@pytest.mark.parametrize("name,iorb,kind", [("he_set01", 1, 0), ("ne_set01", 1, 0), ("ne_set01", 2, 1)])
def test_sor_wavefront_schedule_equals_sequential_sor(name, iorb, kind):
    """The pipelined wavefront of the GPU's list-order SOR (step = level +
    sweep * delta, all updates of a step independent) gives bit for bit the
    oracle's sequential SOR over the "middle" list with the axis
    extrapolated after every sweep (sormcsor.F90:20-132), for an even and an
    odd orbital and a potential, over 3 sweeps."""
    oc = Case(golden_deck(name))
    c = xg.parse_deck(golden_deck(name))
    sched = xg.host_sor_schedule(oc.nni, oc.nmu)
    if kind == 0:
        f1, f2 = oc.fock(iorb)
        lhs, rhs, b = f1 + oc.coeffs()[5], f2, oc.suppl(0)
        isym = -1 if c.m[iorb - 1] % 2 else 1
        u0 = oc.putin(isym, oc.orbital(iorb))
        omega = oc.omega()[0]
    else:
        in1, in2, idel, isym = oc.pot_info(iorb, 1)
        rhs = (oc.orbital(in1) * oc.orbital(in2)) * oc.suppl(9)
        lhs = oc.suppl(7) + float(idel * idel) * oc.suppl(3)
        b = oc.suppl(1)
        u0 = oc.putin(isym, oc.pot(iorb, 1))
        omega = oc.omega()[1]
    d = oc.suppl(2)
    ref = oc.sweep(0, isym, 3, omega, u0, lhs, rhs, b, d)
    got = _sor_wavefront(oc, sched, isym, 3, omega, u0, lhs, rhs, b, d)
    assert np.abs(ref - u0).max() > 0
    assert np.array_equal(got, ref), np.abs(got - ref).max()
