"""Extract the reference's own golden vectors for the (MC)SOR/SCF path.

Reads test-sets/<system>/set-NN/{input.data,reference.lst} from an x2dhf
checkout (its root is the required first argument) and writes, per case, the input deck and a
JSON file with every per-iteration orbital-energy line (scf iteration,
orbital label, orbital energy, energy difference, 1-norm), the final total
energy and the (MC)SOR sweep count printed by the reference program.

These files are the pins of the CPU oracle (tests/test_oracle_golden.py).
The reference's own checkpoint files of be/set-01 (be-hf.*) are copied
unchanged: they pin the checkpoint reader and the orbpot old start.
Run:  python tests/golden/make_golden.py [/path/to/x2dhf]
"""
import json
import os
import re
import sys

CASES = {
    # name: (test-set dir, input override applied by the tests)
    "h2_set01": "h2/set-01",   # H2 151x211, SOR, frozen-orbital start
    "he_set01": "he/set-01",   # He 91x121, SOR
    "he_set02": "he/set-02",   # He 91x121, MCSOR (1 thread)
    "ne_set01": "ne/set-01",   # Ne 151x181, 4 orbitals incl. 1pi, SOR
    "h_set04": "h/set-04",     # H 1pi, 131x?, one electron
    "n2_set01": "n2-elprop/set-01",  # N2 421x781 R_inf=200, 6 orbitals, 22 potentials
    "be_set01": "be/set-01",   # Be 151x181, SOR, started from the be-hf checkpoint (orbpot old)
}
# reference checkpoint files (orbpot old starts), copied as they are
CHECKPOINTS = {"be_set01": ("be/set-01", "be-hf")}
# decks whose reference output is not in the distribution: the input only
INPUT_ONLY = {
    "kf_set01": "kf-elprop/set-01",  # KF, 3 pi + 8 sigma, 11 Coulomb + 61 exchange potentials
    "lih_set01": "lih/set-01",       # LiH, 2 sigma (4 electrons)
    "fh_set01": "fh-elprop/set-01",  # FH, 1 pi + 3 sigma (10 electrons)
    "co_set01": "co-elprop/set-01",  # CO, 1 pi + 5 sigma (14 electrons)
}

# outputs whose first run starts from the hydrogenic LCAO guess: the total
# energy the reference prints after initialisation (prepSCF) pins the start
# (orbitals, Thomas-Fermi Coulomb and 1/r exchange guesses, norms,
# orthogonalisation, multipole moments, orbital energies, EtotalHF).  The
# 2023 runs (the *-elprop sets, ne2/set-03) come from an earlier program
# version whose start differs from the sources; they are kept as the
# record of that, n2-elprop/set-01 among them.
INITIAL_ENERGY_SETS = ["h2/set-01", "he/set-01", "ne/set-01", "na/set-01", "al/set-01", "lih/set-01",
                       "alf/set-02", "gaf/set-01", "he2-elprop/set-01", "ca/set-02"]
EARLIER_VERSION_SETS = ["n2-elprop/set-01", "ne-elprop/set-01", "co-elprop/set-01", "fh-elprop/set-01"]


def first_run(lst):
    """(echoed input deck, run date, first printed total energy) of the
    output's first run."""
    body = lst.split("... start of input data ...", 1)[1]
    echo = body.split("... end of input data", 1)[0].splitlines()[1:]
    deck = "\n".join(ln[2:] if ln.startswith("  ") else ln for ln in echo).rstrip() + "\n"
    date = re.search(r"start:\s+(\S+)", lst)
    etot = re.search(r"total energy:\s+(-?\d\.\d+E[+-]\d+)", body)
    return deck, date.group(1) if date else None, float(etot.group(1))


def initial_energies(root):
    out = {}
    for group, sets in (("current", INITIAL_ENERGY_SETS), ("earlier_version", EARLIER_VERSION_SETS)):
        for rel in sets:
            with open(os.path.join(root, "test-sets", rel, "reference.lst"), errors="replace") as f:
                deck, date, etot = first_run(f.read())
            out[rel] = {"deck": deck, "date": date, "initial_total_energy": etot, "group": group}
    return out


LINE = re.compile(r"^\s*(\d+)\s+(\d+)\s+(sigma|pi|delta|phi)\s*([gu]?)\s+"
                  r"(-?\d\.\d+E[+-]\d+)\s+(-?\d\.\d+E[+-]\d+)\s+(-?\d\.\d+E[+-]\d+)")


def extract(lst):
    recs, etot, sweeps = [], None, None
    for ln in lst.splitlines():
        m = LINE.match(ln)
        if m:
            recs.append([int(m.group(1)), f"{m.group(2)} {m.group(3)} {m.group(4)}".strip(),
                         float(m.group(5)), float(m.group(6)), float(m.group(7))])
            continue
        m = re.match(r"^\s+total energy:\s+(-?\d\.\d+E[+-]\d+)\s*$", ln)
        if m:
            etot = float(m.group(1))
        m = re.search(r"\(MC\)SOR iterations:\s+(\d+)", ln)
        if m:
            sweeps = int(m.group(1))
    return recs, etot, sweeps


def main():
    if len(sys.argv) < 2:
        raise SystemExit("usage: make_golden.py <x2dhf source tree>")
    root = sys.argv[1]
    out = os.path.dirname(os.path.abspath(__file__))
    for name, rel in CASES.items():
        d = os.path.join(root, "test-sets", rel)
        with open(os.path.join(d, "input.data")) as f:
            deck = f.read()
        with open(os.path.join(d, "reference.lst")) as f:
            lst = f.read()
        recs, etot, sweeps = extract(lst)
        if len(recs) > 2000:
            # long runs: keep the first 10 SCF iterations only (the final
            # energy pins the converged result)
            recs = [r for r in recs if r[0] <= 10]
        with open(os.path.join(out, name + ".input"), "w") as f:
            f.write(deck)
        with open(os.path.join(out, name + ".json"), "w") as f:
            json.dump({"source": f"test-sets/{rel}/reference.lst", "records": recs,
                       "total_energy": etot, "sweeps": sweeps}, f, indent=0)
        print(f"{name}: {len(recs)} records, E={etot}, sweeps={sweeps}")
    with open(os.path.join(out, "initial_energies.json"), "w") as f:
        json.dump(initial_energies(root), f, indent=1)
    print("initial_energies.json: printed initial total energies")
    for name, (rel, prefix) in CHECKPOINTS.items():
        os.makedirs(os.path.join(out, name), exist_ok=True)
        for ext in ("dat", "orb", "coul", "exch"):
            with open(os.path.join(root, "test-sets", rel, f"{prefix}.{ext}"), "rb") as f:
                blob = f.read()
            with open(os.path.join(out, name, f"{prefix}.{ext}"), "wb") as f:
                f.write(blob)
        print(f"{name}: checkpoint {prefix}.{{dat,orb,coul,exch}}")
    for name, rel in INPUT_ONLY.items():
        with open(os.path.join(root, "test-sets", rel, "input.data")) as f:
            deck = f.read()
        with open(os.path.join(out, name + ".input"), "w") as f:
            f.write(deck)
        print(f"{name}: input deck only")


if __name__ == "__main__":
    main()
