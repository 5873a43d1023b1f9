"""Checkpoint start on the GPU: from the reference's own be/set-01 files
(orbpot old) the device SCF follows the oracle started from the same files;
a device state written with checkpoint.write and read back starts an
identical SCF."""
import os

import numpy as np
import pytest

import x2dhf_gb300 as xg
from conftest import GOLDEN, golden_deck
from oracle.pyoracle import Case
from x2dhf_gb300 import checkpoint

pytestmark = pytest.mark.gpu

BE = os.path.join(GOLDEN, "be_set01", "be-hf")


def _mcsor(deck):
    lines = [ln for ln in deck.splitlines() if not ln.strip().lower().startswith(("mcsor", "stop"))]
    return "\n".join(lines + ["mcsor", "mcsor-ce", "stop"]) + "\n"


def test_old_start_matches_oracle():
    deck = _mcsor(golden_deck("be_set01"))
    ck = checkpoint.read(BE, m=[0, 0])
    oc = Case(deck)
    oc.load_checkpoint(ck)
    oc.steps(10)
    ctx = xg.Context(0)
    s = xg.SCF(ctx, xg.parse_deck(deck))
    s.load_checkpoint(ck)
    s.run(10)
    ro, rg = oc.records(), s.records()
    assert len(ro) == len(rg) == 20
    for a, b in zip(ro, rg):
        assert a[:2] == b[:2]
        assert abs(a[2] - b[2]) <= 1e-11 * max(1.0, abs(a[2])), (a, b)
    s.close()
    ctx.close()


def test_save_and_restart_round_trip(tmp_path):
    """Write the state of a running SCF, read it into a second SCF: every
    function, Lagrange multiplier, norm and moment arrives bit for bit, and
    the restarted SCF runs on."""
    deck = _mcsor(golden_deck("be_set01"))
    ctx = xg.Context(0)
    a = xg.SCF(ctx, xg.parse_deck(deck))
    a.load_checkpoint(checkpoint.read(BE, m=[0, 0]))
    a.run(3)
    prefix = str(tmp_path / "state")
    cka = a.checkpoint(title="Be")
    checkpoint.write(prefix, cka)
    ck = checkpoint.read(prefix, m=[0, 0])
    b = xg.SCF(ctx, xg.parse_deck(deck))
    b.load_checkpoint(ck)
    for kind, i in ((0, 1), (0, 2), (1, 1), (1, 2)):
        assert np.array_equal(a.function(kind, i), b.function(kind, i))
    assert np.array_equal(a.function(2, 1, 2), b.function(2, 1, 2))
    ckb = b.checkpoint(title="Be")
    assert np.array_equal(cka.ee, ckb.ee) and np.array_equal(cka.orbnorm, ckb.orbnorm)
    assert np.array_equal(cka.cmulti, ckb.cmulti) and np.array_equal(cka.exc, ckb.exc)
    res = b.run(2)
    assert res.iterations == 2 and np.isfinite(res.total_energy)
    a.close()
    b.close()
    ctx.close()
