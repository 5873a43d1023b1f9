"""Serving loop: independent SCF requests sharing one GPU.

Each request is one closed-shell HF solve of a diatomic molecule, described
by input cards (an x2dhf input deck).  A server runs `slots` host threads;
each owns a library context (its own CUDA stream and workspace), so the
solves of different slots run concurrently on the GPU.  Requests are admitted
first-in first-out at their arrival times, when a slot is free and the
estimated device footprint of all solves in flight stays within the HBM
budget.  A finished slot takes the next waiting request at once (continuous
batching at request granularity).

The solves are deterministic: a request gives bit-identical orbital and
total energies whether it runs alone or next to other requests, since every
reduction sums in a fixed order and no kernel depends on what else shares
the GPU.

The request mix follows the serving configuration of the survey: seeded
Poisson arrivals; closed-shell diatomics with 2, 4, 10 and 14 electrons and
nuclear charges up to 9, each from one of the reference's own input decks
(its hydrogenic LCAO start), with the grid drawn from N_nu in [169, 505] and
N_mu in [241, 721] before the reference's n = 1 (mod 30) rounding, R_inf =
40, and the bond length drawn from U[1.5, 5.0] bohr restricted to [0.8, 1.5]
times the deck's bond length (further out the restricted closed-shell start
dissociates and no longer converges).  Every solve relaxes all potentials
of an SCF iteration in one launch and then all orbitals in one launch
(x2g_case.batch_mode 2).
"""
import dataclasses
import statistics
import threading
import time

import numpy as np

from . import MIXED, SCF, Context, X2GError, parse_deck, round_grid

# cards of the template decks that the served solve does not use
_DROP = ("mmoments", "conv", "stop", "omega", "altsweeps", "lagra", "!", "grid", "scf", "mcsor", "title")


@dataclasses.dataclass
class Request:
    rid: int
    template: str
    arrival: float          # seconds after the start of the run
    r: float                # bond length, bohr
    nnu: int
    nmu: int
    deck: str
    norb: int
    bytes: int              # estimated device footprint of the solve


@dataclasses.dataclass
class Completed:
    rid: int
    template: str
    arrival: float
    start: float
    end: float
    iterations: int
    converged: int
    total_energy: float
    orbital_energies: tuple
    error: str = ""         # the library's message when the solve failed

    @property
    def latency(self):
        return self.end - self.arrival


def request_deck(template_deck, r, nnu, nmu, maxscf=3000):
    """The template's cards with bond length r, grid nnu x nmu (R_inf = 40),
    MCSOR for orbitals and potentials, orbital-energy threshold 1e-11 and
    norm threshold 1e-13 (at 1e-12 the heteronuclear FH and CO requests
    hover at the threshold and leave by the reference's stagnation exit)."""
    out = []
    for ln in template_deck.splitlines():
        key = ln.strip().lower()
        if not key or key.startswith(_DROP):
            continue
        if key.startswith("nuclei"):
            f = ln.split()
            ln = f"nuclei {f[1]} {f[2]} {r:.6f}"
        out.append(ln)
    out = ["title served"] + out
    out += [f"grid {nnu} {nmu} 40.0", f"scf {maxscf} 0 11 13 1", "mcsor", "mcsor-ce", "stop"]
    return "\n".join(out) + "\n"


def footprint_bytes(case):
    """Device bytes of one solve: orbitals, Coulomb and exchange potentials
    and per-orbital work arrays in the extended layout, plus the grid's
    tables (the closed-shell pair rule: one exchange potential per pair, two
    for a pair of non-sigma orbitals, one self-exchange per non-sigma
    orbital)."""
    m = [int(case.m[i]) for i in range(case.norb)]
    n = len(m)
    pots = n + sum(1 + (1 if (m[i] > 0 and m[j] > 0) else 0) for i in range(n) for j in range(i + 1, n))
    pots += sum(1 for x in m if x > 0)
    ext = (case.nnu + 8) * (case.nmu + 8) * 8
    plain = case.nnu * case.nmu * 8
    return (3 * n + pots) * ext + 60 * plain


def make_requests(templates, n, rate, seed=42):
    """n requests with Poisson arrivals at `rate` per second: templates is
    {name: deck text}; the template, bond length and grid of every request
    come from one seeded generator, so the list is reproducible."""
    rng = np.random.default_rng(seed)
    names = sorted(templates)
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate) if rate > 0 else 0.0
        name = names[int(rng.integers(0, len(names)))]
        base = templates[name]
        r0 = next(float(ln.split()[3]) for ln in base.splitlines() if ln.strip().lower().startswith("nuclei"))
        lo, hi = max(1.5, 0.8 * r0), min(5.0, 1.5 * r0)
        r = float(rng.uniform(lo, hi))
        nnu = round_grid(int(rng.integers(169, 506)))
        nmu = round_grid(int(rng.integers(241, 722)))
        deck = request_deck(base, r, nnu, nmu)
        case = parse_deck(deck)
        out.append(Request(i, name, t, r, case.nnu, case.nmu, deck, case.norb, footprint_bytes(case)))
    return out


class GpuBackend:
    """Solves on the GPU: one library context (own stream) per slot."""

    def __init__(self, device=0, precision=MIXED, batch_mode=2):
        self.device = device
        self.precision = precision
        self.batch_mode = batch_mode

    def open(self):
        return Context(self.device)

    def solve(self, ctx, q):
        s = SCF(ctx, parse_deck(q.deck, precision=self.precision, batch_mode=self.batch_mode))
        try:
            res = s.run()
            return res.iterations, res.converged, res.total_energy, tuple(float(res.ee[i]) for i in range(q.norb))
        finally:
            s.close()

    def close(self, ctx):
        ctx.close()


class Server:
    """`slots` concurrent SCF solves under an HBM budget; `backend` opens a
    per-slot handle and solves one request on it (default: the GPU)."""

    def __init__(self, device=0, slots=4, precision=MIXED, hbm_budget=64 << 30, backend=None, batch_mode=2):
        self.slots = slots
        self.budget = hbm_budget
        self.backend = backend or GpuBackend(device, precision, batch_mode)
        self.peak_bytes = 0  # largest footprint in flight during the last run
        self.budget_waits = 0  # admissions the HBM budget delayed during the last run

    def run(self, requests, realtime=True):
        """Serve the requests (sorted by arrival); with realtime=False every
        request is taken to have arrived at time 0.  Returns the completions
        in request order and the run's wall time.  A solve that fails with a
        library status (X2GError) completes with that error and NaN energies
        and its slot goes on serving; any other exception stops the run and
        is raised."""
        reqs = sorted(requests, key=lambda q: (q.arrival, q.rid))
        self.peak_bytes = 0
        self.budget_waits = 0
        waited = set()
        done = {}
        errors = []
        lock = threading.Condition()
        state = {"next": 0, "bytes": 0, "inflight": 0}
        t0 = time.perf_counter()

        def clock():
            return time.perf_counter() - t0

        def take():
            with lock:
                while True:
                    if state["next"] >= len(reqs) or errors:
                        return None
                    q = reqs[state["next"]]
                    wait = (q.arrival - clock()) if realtime else 0.0
                    if wait > 0:
                        lock.wait(wait)
                        continue
                    if state["inflight"] > 0 and state["bytes"] + q.bytes > self.budget:
                        if q.rid not in waited:
                            waited.add(q.rid)
                            self.budget_waits += 1
                        lock.wait()
                        continue
                    state["next"] += 1
                    state["bytes"] += q.bytes
                    state["inflight"] += 1
                    self.peak_bytes = max(self.peak_bytes, state["bytes"])
                    return q

        def release(q):
            with lock:
                state["bytes"] -= q.bytes
                state["inflight"] -= 1
                lock.notify_all()

        def worker():
            try:
                ctx = self.backend.open()
            except Exception as e:  # no device: report once, stop the run
                with lock:
                    errors.append(e)
                    lock.notify_all()
                return
            try:
                while True:
                    q = take()
                    if q is None:
                        return
                    start = clock()
                    arrival = q.arrival if realtime else 0.0
                    try:
                        it, conv, etot, ee = self.backend.solve(ctx, q)
                        done[q.rid] = Completed(q.rid, q.template, arrival, start, clock(), it, conv, etot, ee)
                    except X2GError as e:
                        # the request failed (a NaN, a device wait limit):
                        # recorded, and the slot serves the next one
                        nan = float("nan")
                        done[q.rid] = Completed(q.rid, q.template, arrival, start, clock(), 0, 0, nan,
                                                (nan,) * q.norb, error=str(e))
                    except Exception as e:
                        with lock:
                            errors.append(e)
                            lock.notify_all()
                    finally:
                        release(q)
            finally:
                self.backend.close(ctx)

        threads = [threading.Thread(target=worker, daemon=True) for _ in range(self.slots)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        if errors:
            raise errors[0]
        return [done[q.rid] for q in requests], clock()


def summary(completed, wall):
    """p50 / p99 latency, mean service time and solves/s of a run."""
    lat = sorted(c.latency for c in completed)
    svc = [c.end - c.start for c in completed]

    def pct(p):
        return lat[min(len(lat) - 1, int(round(p * (len(lat) - 1))))]

    return {"requests": len(completed), "solves_per_s": len(completed) / wall, "wall_s": wall,
            "latency_p50_s": pct(0.50), "latency_p99_s": pct(0.99), "service_mean_s": statistics.mean(svc),
            "converged": sum(1 for c in completed if c.converged),
            "converged_energy": sum(1 for c in completed if c.converged == 1),
            "converged_norm": sum(1 for c in completed if c.converged == 2),
            "unconverged": sum(1 for c in completed if not c.converged and not c.error),
            "failed": sum(1 for c in completed if c.error),
            "converged_solves_per_s": sum(1 for c in completed if c.converged) / wall}
