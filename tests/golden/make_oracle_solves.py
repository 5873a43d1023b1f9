#!/usr/bin/env python
"""A full SCF solve of the bench's N2 workload (closed-shell N2, Z=7,7,
R=2.068 bohr, grid 337x481 -> 331x481, R_inf=40, MCSOR for orbitals and
potentials) by the CPU oracle, in the reference's relaxation order: the
fixture tests/golden/n2_331x481_oracle.json that the GPU parity tests
compare a GPU solve of the same deck against.

The deck runs exactly 1000 SCF iterations (the orbital-energy and norm
thresholds 1e-16 are out of reach, and the stagnation check starts only at
iteration 5000), past the 952 iterations after which the bench deck's 1e-12
threshold stops the oracle, so that the GPU's iteration-by-iteration energies
and its final state are compared with the oracle's at the same iteration.

It records every orbital energy of every SCF iteration, the final orbital
and total energies, the sweep count, and the converged orbitals, Coulomb and
exchange potentials at 64 seeded grid points each together with each
function's max-norm.  A full oracle solve of this grid takes minutes on one
core, too long to repeat inside a test.

    python tests/golden/make_oracle_solves.py
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "n2_331x481_oracle.json")
NSAMPLE = 64


def sample_points(mxsize, seed=7):
    return sorted(int(i) for i in np.random.default_rng(seed).choice(mxsize, NSAMPLE, replace=False))


def function_record(v, idx):
    return {"max_abs": float(np.abs(v).max()), "samples": [float(v[i]) for i in idx]}


def main():
    sys.path.insert(0, ROOT)
    import bench
    from oracle.pyoracle import Case

    deck = "\n".join("scf 1000 0 16 16 1" if ln.strip().lower().startswith("scf") else ln
                     for ln in bench.n2_deck().splitlines()) + "\n"
    t0 = time.perf_counter()
    c = Case(deck)
    c.run()
    wall = time.perf_counter() - t0
    recs = c.records()
    norb = c.norb
    idx = sample_points(c.mxsize)
    pots = []
    for iorb in range(1, norb + 1):
        for k in range(1, c.npots(iorb) + 1):
            in1, in2, idel, isym = c.pot_info(iorb, k)
            pots.append(dict(iorb=iorb, k=k, in1=in1, in2=in2, idel=idel, isym=isym,
                             **function_record(c.pot(iorb, k), idx)))
    out = {
        "deck": deck, "grid": [c.nni, c.nmu], "iterations": recs[-1][0], "sweeps": c.sweeps(),
        "total_energy": c.total_energy(), "orbital_energies": [c.ee(i, i) for i in range(1, norb + 1)],
        "records": [[r[0], r[1], r[2]] for r in recs], "sample_index": idx,
        "orbitals": [function_record(c.orbital(i), idx) for i in range(1, norb + 1)], "potentials": pots,
        "oracle_wall_s": round(wall, 1),
    }
    with open(OUT, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print(f"{OUT}: {out['iterations']} iterations, E = {out['total_energy']:.15f}, {wall:.0f} s")


if __name__ == "__main__":
    main()
