#!/usr/bin/env python
"""Full SCF solves of the bench's SCF workloads by the reference's own C
relaxation kernels (oracle/_ref: sorpt_ on the colour-ordered lists for the
potentials, one thread per potential, and mcsor_pthread_ for the orbitals)
under the oracle's SCF driver, run to the driver's convergence exit
(src/doSCF.F90:540-723).  TEST INFRASTRUCTURE: it writes
oracle/ref_solves.json, the iteration count and energies of each solve,
which bench.py's reference arm uses to scale a bounded sample of SCF
iterations to one solve.

    python oracle/ref_solves.py [workload ...]     (default: h2 n2)

mcsor_pthread_ runs on one thread here: with more threads the reference's
MCSOR races at the colour seams of the "middle" ordering and the iteration
count can move by a few iterations from run to run.
"""
import json
import os
import platform
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "ref_solves.json")


def solve(name, nthreads=1):
    sys.path.insert(0, ROOT)
    import bench
    from oracle import pyoracle, pyref

    pyoracle.build()
    if not pyref.available():
        raise SystemExit("reference C kernels not built (oracle/build_ref.sh)")
    deck = bench.WORKLOADS[name]()
    t0 = time.perf_counter()
    ref = pyref.ReferenceSCF(deck, nthreads=nthreads)
    ref.case.run()
    wall = time.perf_counter() - t0
    recs = ref.records()
    c = ref.case
    return {"iterations": recs[-1][0] if recs else 0, "sweeps": c.sweeps(), "total_energy": c.total_energy(),
            "orbital_energies": [c.ee(i, i) for i in range(1, c.norb + 1)], "grid": [c.nni, c.nmu],
            "mcsor_threads": nthreads, "wall_s": round(wall, 1), "host": f"{platform.machine()}, {os.cpu_count()} cpus"}


def main(names):
    data = {}
    if os.path.exists(OUT):
        with open(OUT) as f:
            data = json.load(f)
    for n in names:
        data[n] = solve(n)
        print(n, data[n], flush=True)
        with open(OUT, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
            f.write("\n")


if __name__ == "__main__":
    main(sys.argv[1:] or ["h2", "n2"])
