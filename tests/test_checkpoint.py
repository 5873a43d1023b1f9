"""Checkpoint files (<prefix>.dat/.orb/.coul/.exch) against the reference's
own: the be/set-01 files written by x2dhf are read, rewritten byte for byte
(the .dat date line aside), and an `orbpot old` start from them reproduces
the reference's printed SCF trajectory."""
import os

import numpy as np

from conftest import GOLDEN, golden_deck, golden_json
from oracle.pyoracle import Case
from x2dhf_gb300 import checkpoint

BE = os.path.join(GOLDEN, "be_set01", "be-hf")


def test_read_reference_checkpoint():
    ck = checkpoint.read(BE, m=[0, 0])
    assert (ck.nnu, ck.nmu, ck.nel) == (151, 181, 4)
    assert np.allclose([ck.rinf, ck.z1, ck.z2, ck.r], [35.0, 4.0, 0.0, 2.386], rtol=1e-14)
    assert len(ck.orbitals) == 2 and len(ck.coulomb) == 2 and list(ck.exchange) == [(1, 2, 0)]
    # orbital 1 is 2sigma, orbital 2 is 1sigma (the config card's order)
    assert abs(ck.ee[0, 0] + 0.30927) < 1e-4 and abs(ck.ee[1, 1] + 4.73267) < 1e-4
    assert np.all(np.isfinite(ck.orbitals[0])) and np.abs(ck.orbitals[1]).max() > 0.1


def test_rewrite_is_byte_identical(tmp_path):
    """The writer reproduces the reference's records, including initAddr's
    address arrays in the .orb header."""
    ck = checkpoint.read(BE, m=[0, 0])
    out = str(tmp_path / "copy")
    checkpoint.write(out, ck)
    for ext in ("orb", "coul", "exch"):
        with open(BE + "." + ext, "rb") as a, open(out + "." + ext, "rb") as b:
            assert a.read() == b.read(), ext
    with open(BE + ".dat") as a, open(out + ".dat") as b:
        la, lb = a.read().splitlines(), b.read().splitlines()
    assert la[0] == lb[0] and la[2:] == lb[2:]


def test_round_trip_with_pi_orbitals(tmp_path):
    """Two pi and one sigma orbital: pi-pi pairs carry two exchange
    potentials, a pi orbital its self-exchange potential."""
    rng = np.random.default_rng(5)
    nnu, nmu, m = 31, 41, [1, 0, 1]
    f = lambda: rng.standard_normal((nmu, nnu))
    keys = checkpoint.exchange_order(m)
    assert keys == [(1, 1, 0), (1, 2, 0), (1, 3, 0), (1, 3, 1), (2, 3, 0), (3, 3, 0)]
    ck = checkpoint.Checkpoint("test", nnu, nmu, 40.0, 7.0, 8.0, 2.1, 14, m, [f() for _ in m], [f() for _ in m],
                               {k: f() for k in keys}, rng.standard_normal((3, 3)), np.ones(3))
    p = str(tmp_path / "pi")
    checkpoint.write(p, ck)
    back = checkpoint.read(p, m)
    assert (back.nnu, back.nmu, back.norb, back.nel) == (nnu, nmu, 3, 14)
    for a, b in zip(ck.orbitals + ck.coulomb, back.orbitals + back.coulomb):
        assert np.array_equal(a, b)
    for k in keys:
        assert np.array_equal(ck.exchange[k], back.exchange[k])
    assert np.array_equal(ck.ee, back.ee)


def test_oracle_old_start_matches_reference_trajectory():
    """be/set-01: `orbpot old` from the reference's be-hf files, 10 SOR SCF
    iterations, every printed orbital energy and the final energy."""
    c = Case(golden_deck("be_set01"))
    c.load_checkpoint(checkpoint.read(BE, m=[0, 0]))
    c.run()
    g = golden_json("be_set01")
    recs = c.records()
    assert len(recs) == len(g["records"])
    for (it, io, ee, dee, dn), gr in zip(recs, g["records"]):
        assert it == gr[0]
        assert abs(ee - gr[2]) <= 5e-12 * max(1.0, abs(gr[2])), (it, io, ee, gr)
    assert abs(c.total_energy() - g["total_energy"]) <= 2e-13 * abs(g["total_energy"])
