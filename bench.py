#!/usr/bin/env python
"""Benchmark: SCF solves/s of the x2dhf relaxation path on GB300.

Workloads (grids after the reference's n = 1 (mod 30) rounding):
  n2   closed-shell N2 (Z=7,7, R=2.068 bohr), 6 orbitals, 22 Coulomb+exchange
       potentials per SCF iteration, grid 337x481 -> 331x481, R_inf = 40
  h2   H2 (Z=1,1, R=1.4), grid 169x241 -> 151x241, R_inf = 40
One step = one full SCF solve from the hydrogenic start to the orbital-energy
threshold.  `value` is the mixed form (FP32 sweeps + FP64 defect
correction) in its batched mode: every Coulomb and exchange potential of an
SCF iteration relaxed in one launch, then every orbital in one launch, with
the state already resident in HBM.  Beside it: the plain FP64 form in the
reference's colour and relaxation order (the comparator), the mixed form in
the reference's order, and for N2 each form's |dE| against the full FP64
oracle solve in tests/golden.  `e2e` times the public API call a user makes
(host case description in, host orbitals out) including the host->device
upload of the grid tables and the device->host readback of every orbital.

--impl reference times the reference on the host cores: the reference's own C
relaxation backend (x2dhf src/c, built unmodified into oracle/_ref) under the
oracle's restatement of the SCF driver (no Fortran compiler exists here).
"""
import argparse
import faulthandler
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SCF solves/s & p99 latency at |dE|<1e-9 Eh: mixed vs FP64 MCSOR, 1 GB300"
UNIT = "SCF solves/s"
# algorithmic bytes per point-update: u read + u write + lhs + rhs
BYTES_PER_PT = {0: 32.0, 1: 16.0}
FLOPS_PER_PT = 54.0
# DRAM bytes (read + write) per point-update of the on-chip cluster sweep,
# from ncu (dram__bytes_read.sum + dram__bytes_write.sum = 2 765 824 + 0) of
# one single-job, 10-sweep launch on 331x481 (1 566 040 point-updates): the
# correction, residual and omega/lhs stay in shared memory, so DRAM sees only
# the band load (the u += e writeback was still in L2 when the launch ended)
CLUSTER_DRAM_BYTES_PER_PT = 2765824.0 / 1566040.0
# the same for the persistent-band sweep of grids beyond one cluster, from
# ncu of two 6-job, 10-sweep launches on 781x1201 (71.38 + 1.57 MB read + write
# per launch, 55 901 040 point-updates)
BAND_DRAM_BYTES_PER_PT = (71379200.0 + 1573120.0) / 55901040.0


def n2_deck(grid="337 481 40.0"):
    with open(os.path.join(ROOT, "tests", "golden", "n2_set01.input")) as f:
        deck = f.read()
    out = []
    for ln in deck.splitlines():
        key = ln.strip().lower()
        if key.startswith("grid"):
            ln = f"grid {grid}"
        elif key.startswith("scf"):
            ln = "scf 8000 0 12 14 1"
        elif key.startswith(("mmoments", "stop")):
            continue
        out.append(ln)
    out += ["mcsor", "mcsor-ce", "stop"]
    return "\n".join(out) + "\n"


def h2_deck():
    return """title H2
method hf
nuclei  1.0 1.0  1.4
config 0
  1 sigma g end
grid 169 241 40.0
orbpot hydrogen
lcao
 1.0 1 0 1.0   1.0   1 0  1.0
scf  4000 0 12 14 1
mcsor
mcsor-ce
stop
"""


def kf_deck():
    """KF (Z=19,9, R=4.1035 bohr; 3 pi + 8 sigma, 11 Coulomb + 61 exchange
    potentials per SCF iteration) from the reference's kf-elprop/set-01 input,
    on grid 793x1201 -> 781x1201, R_inf=60: the heteronuclear large-grid case."""
    with open(os.path.join(ROOT, "tests", "golden", "kf_set01.input")) as f:
        deck = f.read()
    out = []
    for ln in deck.splitlines():
        key = ln.strip().lower()
        if key.startswith("grid"):
            ln = "grid 793 1201 60.0"
        elif key.startswith(("mmoments", "conv", "stop", "!")):
            continue
        out.append(ln)
    out += ["mcsor", "mcsor-ce", "stop"]
    return "\n".join(out) + "\n"


WORKLOADS = {"n2": n2_deck, "h2": h2_deck, "kf": kf_deck, "kf-solve": kf_deck}
# workloads timed over a fixed number of SCF iterations per step (a full
# solve of the large grid takes thousands of iterations)
FIXED_ITERS = {"kf": 20}
# full-solve workloads whose warm-up steps run only the first SCF iterations
# (a warm-up full solve of the plain FP64 form would take minutes)
WARMUP_ITERS = {"kf-solve": 20}
WORKLOAD_TEXT = {
    "n2": "N2 closed-shell HF SCF, Z=7,7 R=2.068, 6 orbitals, 22 Poisson solves/iteration, grid 337x481 -> 331x481, "
          "R_inf=40",
    "h2": "H2 HF SCF, Z=1,1 R=1.4, grid 169x241 -> 151x241, R_inf=40",
    "kf": "KF HF SCF, Z=19,9 R=4.1035, 11 orbitals (3 pi, 8 sigma), 72 Poisson solves/iteration, grid 793x1201 -> "
          "781x1201, R_inf=60; first 20 SCF iterations from the hydrogenic start per step",
    "kf-solve": "KF HF SCF, Z=19,9 R=4.1035, 11 orbitals (3 pi, 8 sigma), 72 Poisson solves/iteration, grid "
                "793x1201 -> 781x1201, R_inf=60; one full SCF solve per step (warm-up steps: the first 20 "
                "iterations)",
}


def slater_sources(grid_h, nnu, nmu, r, batch, seed0=1234):
    """Seeded pairs of normalised Slater functions r^l e^(-zeta r) P_l^m(cos)
    on centre A or B (exponents U[0.5,8], l <= 3, m <= min(l,2)), evaluated on
    the plain grid: the sources psi_a psi_b of a batch of Poisson solves."""
    import numpy as np

    hni = np.pi / (nnu - 1)
    x = 2.0 * grid_h / r
    hmu = np.log(x + np.sqrt(x * x - 1.0)) / (nmu - 1)
    xi = np.cosh(np.arange(nmu) * hmu)[:, None]
    eta = np.cos(np.arange(nnu) * hni)[None, :]
    out = []
    for b in range(batch):
        rng = np.random.default_rng(seed0 + b)
        pair = []
        for _ in range(2):
            zeta = rng.uniform(0.5, 8.0)
            l = int(rng.integers(0, 4))
            m = int(rng.integers(0, min(l, 2) + 1))
            sign = 1.0 if rng.integers(0, 2) == 0 else -1.0
            rc = (r / 2.0) * (xi + sign * eta)          # distance from the centre
            cz = np.clip(sign * (1.0 + xi * eta) / np.maximum(xi + sign * eta, 1e-300), -1.0, 1.0)
            sz = np.sqrt(np.clip(1.0 - cz * cz, 0.0, None))
            f = rc ** l * np.exp(-zeta * rc) * (sz ** m) * (cz ** (l - m))
            pair.append((f / max(np.abs(f).max(), 1e-300), m))
        out.append(pair)
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.rows.append([x.strip() for x in ln.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if len(r) > 3 + k and r[3 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def flush_l2(torch, buf):
    buf.add_(1.0)  # writes 512 MiB > 129 MB L2


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def round_grid(n):
    """The reference's grid rounding (nnucalc/nmucalc, src/inputInterface.F90:
    2961-3095): n = 1 (mod 6) and n - 6 = 0 (mod 5) enforced alternately,
    always rounding down.  Plain Python, so that the reference arm loads
    nothing of this repository's GPU library."""
    if n < 7:
        return 0
    while True:
        while (n - 1) % 6 != 0:
            n -= 1
        nt = n
        while ((n - 6) // 5) * 5 != n - 6:
            n -= 1
        if n > 1 and n != nt:
            continue
        return n


def deck_grid(deck):
    """(N_nu, N_mu) of a deck whose grid card gives both counts, rounded."""
    for ln in deck.splitlines():
        t = ln.split("!")[0].split()
        if t and t[0].lower() == "grid":
            return round_grid(int(t[1])), round_grid(int(float(t[2])))
    raise ValueError("deck has no grid card")


def workload_config(name):
    """The `config` of a workload's JSON line, identical in both arms."""
    nnu, nmu = deck_grid(WORKLOADS[name]())
    return {"workload": f"{name}: " + WORKLOAD_TEXT[name],
            "convergence": "orbital-energy change < 1e-12 for 4 consecutive SCF iterations",
            "parallelism": "replicas only (independent SCF solves per GPU)",
            "grid": [nnu, nmu], "points_per_sweep": (nnu - 2) * (nmu - 5),
            "l2": "GPU arm: 512 MiB buffer written between timed steps (L2 flushed); CPU arm: host caches as they are"}


def max_over_ranks(values, world, device):
    """Element-wise maximum of per-rank timings over all ranks (replicas run
    the same work independently; no collective touches the data path)."""
    if world <= 1:
        return list(values)
    import torch
    import torch.distributed as dist

    t = torch.tensor(values, device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


# the N2 workload's full oracle solve (FP64, reference order), written by
# tests/golden/make_oracle_solves.py: the |dE| of every form against it
ORACLE_SOLVES = {"n2": os.path.join(ROOT, "tests", "golden", "n2_331x481_oracle.json")}
# SCF forms timed by the GPU arm: (name, precision 0 FP64 / 1 mixed, batch
# mode, MCSOR sweeps per relaxation: 0 the deck's own, else the mcsor card's
# maxsor for orbitals and potentials); the last leg, the batched mixed form,
# is the headline `value`
SCF_LEGS = (("fp64", 0, 0, 0), ("fp64_batched", 0, 2, 0), ("mixed_reference_order", 1, 0, 0),
            ("mixed_sweeps40", 1, 2, 40), ("mixed", 1, 2, 0))
# workloads that run the sweeps40 leg (a few-second full solve each)
SWEEPS_LEG_WORKLOADS = ("n2", "h2")


def deck_with_sweeps(deck, n):
    """The deck with n MCSOR sweeps per orbital and potential relaxation (the
    mcsor card's maxsor fields, inputInterface.F90:1910-2028); n = 0 keeps it."""
    if not n:
        return deck
    out = [ln for ln in deck.splitlines() if not ln.strip().lower().startswith(("mcsor", "stop"))]
    return "\n".join(out + [f"mcsor 0 {n} {n}", f"mcsor-ce 0 {n}", "stop"]) + "\n"


def oracle_reference(name):
    try:
        with open(ORACLE_SOLVES[name]) as f:
            d = json.load(f)
        return {"total_energy": d["total_energy"], "orbital_energies": d["orbital_energies"],
                "iterations": d["iterations"]}
    except (KeyError, OSError, ValueError):
        return None


def run_gpu(args):
    import torch
    import x2dhf_gb300 as xg
    from x2dhf_gb300 import build

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    build.build()
    torch.cuda.set_device(local)
    ctx = xg.Context(local)
    _configure(ctx, args)
    stream = torch.cuda.ExternalStream(xg.lib().x2g_stream(ctx.h))
    deck = WORKLOADS[args.workload]()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    fixed = FIXED_ITERS.get(args.workload, 1 << 30)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    copied = [0, 0, 0]  # host-to-device bytes, device-to-host bytes, timed e2e steps

    def timed_solves(prec, mode, k, warm, e2e=False, cap=None, warm_cap=None, sweeps=0):
        lat, res_last, iters = [], None, []
        leg_deck = deck_with_sweeps(deck, sweeps)
        for step in range(warm + k):
            if not e2e:
                case = xg.parse_deck(leg_deck, precision=prec, batch_mode=mode)
                scf = xg.SCF(ctx, case)  # initial guess uploaded: state resident in HBM
            flush_l2(torch, flush)
            barrier()
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0 = time.perf_counter()
            b0 = ctx.transfer_bytes()
            ev0.record(stream)
            if e2e:
                case = xg.parse_deck(leg_deck, precision=prec, batch_mode=mode)
                scf = xg.SCF(ctx, case)
            res = scf.run(cap if cap else (fixed if step >= warm else
                                           warm_cap or WARMUP_ITERS.get(args.workload, fixed)))
            if e2e:
                for i in range(1, case.norb + 1):
                    scf.orbital(i)
            ev1.record(stream)
            ev1.synchronize()
            wall = time.perf_counter() - t0
            dev = ev0.elapsed_time(ev1) / 1000.0
            if step >= warm:
                lat.append(max(dev, wall) if e2e else dev)
                iters.append(res.iterations)
                if e2e:
                    b1 = ctx.transfer_bytes()
                    copied[0] += b1[0] - b0[0]
                    copied[1] += b1[1] - b0[1]
                    copied[2] += 1
            res_last = res
            scf.close()
        return lat, res_last, iters

    legs = [lg for lg in SCF_LEGS if (args.legs == "all" and (not lg[3] or args.workload in SWEEPS_LEG_WORKLOADS))
            or lg[0] == args.legs]
    head = legs[-1]
    sampler = ClockSampler(local)
    lat, res, its = {}, {}, {}
    launches = 0
    ctx.profile(0, xg.FP64)  # the timed steps run without the library's per-launch events
    with sampler:
        for name, prec, mode, sweeps in legs:
            # the plain FP64 form is the slow comparator: a few timed solves
            k = args.steps if not name.startswith("fp64") or len(legs) == 1 else min(args.steps, args.fp64_steps)
            l0 = ctx.launches
            # the comparator's warm-up solves stop after 50 iterations (a full
            # plain-FP64 solve takes seconds and warms nothing more)
            lat[name], res[name], its[name] = timed_solves(prec, mode, k, args.warmup,
                                                           warm_cap=50 if name.startswith("fp64") else None,
                                                           sweeps=sweeps)
            if name == head[0]:
                # launches of the timed headline solves (the warm-up ones counted out)
                launches = int((ctx.launches - l0) * k / (k + args.warmup))
        late2e, rese2e, _ = timed_solves(head[1], head[2], max(1, args.steps // 2), 1, e2e=True, sweeps=head[3])
    # roofline figures: one more step of each form with the library's
    # per-launch CUDA events on (recorded on its own stream), not timed; a
    # long full-solve workload profiles its first iterations only
    prof = {}
    for name, prec, mode, sweeps in legs:
        if name in ("mixed_reference_order", "mixed_sweeps40"):
            continue
        ctx.profile(2, prec)
        timed_solves(prec, mode, 1, 0, cap=WARMUP_ITERS.get(args.workload))
        prof[name] = ctx.profile(-1, prec)
    ctx.profile(0, xg.FP64)
    # max over ranks: the slowest replica sets the pace
    names = list(lat)
    tot = max_over_ranks([sum(lat[n]) for n in names] + [sum(late2e)], world, f"cuda:{local}")
    tot, tote2e = dict(zip(names, tot[:-1])), tot[-1]
    if rank != 0:
        return None
    hbm, peak_kind = peaks()
    c = xg.parse_deck(deck)
    per_step = FIXED_ITERS.get(args.workload, 1)  # solves, or iterations for a fixed-iteration workload
    unit = "SCF iterations/s" if args.workload in FIXED_ITERS else UNIT
    metric = (f"SCF iterations/s over the first {per_step} iterations: mixed vs FP64 MCSOR, 1 GB300"
              if args.workload in FIXED_ITERS else METRIC)
    rate = {n: world * len(lat[n]) * per_step / tot[n] for n in names}
    value = rate[head[0]]
    e2e_value = world * len(late2e) * per_step / tote2e
    on_chip = xg.host_cluster_plan(c.nnu, c.nmu)[0] > 0
    occ = (0, 0)
    if on_chip:
        g = xg.Grid(ctx, c.nnu, c.nmu, c.r, c.rinf, c.z1, c.z2)
        occ = g.cluster_occupancy()
        g.close()
    hs = sorted(lat[head[0]])
    p99 = hs[min(len(hs) - 1, int(round(0.99 * (len(hs) - 1))))]
    # bytes the library copied per timed e2e step (grid tables up; per-iteration
    # scalars and the orbitals down), from its own transfer counters
    h2d = copied[0] // max(1, copied[2])
    d2h = copied[1] // max(1, copied[2])
    msmx, ptsmx, nmx = prof.get(head[0], (0.0, 0.0, 0)) if head[1] == 1 else (0.0, 0.0, 0)
    ms64, pts64, n64 = prof.get("fp64", (0.0, 0.0, 0))
    msb64, ptsb64, nb64 = prof.get("fp64_batched", (0.0, 0.0, 0))
    sweep_gbs_mx = ptsmx * BYTES_PER_PT[1] / (msmx / 1e3) / 1e9 if msmx > 0 else None
    sweep_gbs_64 = pts64 * BYTES_PER_PT[0] / (ms64 / 1e3) / 1e9 if ms64 > 0 else None
    pts_per_launch = ptsmx / nmx if nmx else None
    traffic = ((CLUSTER_DRAM_BYTES_PER_PT if on_chip else BAND_DRAM_BYTES_PER_PT) * pts_per_launch
               if pts_per_launch else None)
    oref = oracle_reference(args.workload)
    fp64_e = res["fp64"].total_energy if "fp64" in res else None

    def form(n):
        r = res[n]
        d = {"value": rate[n], "unit": unit, "iterations": its[n], "total_energy": r.total_energy,
             "orbital_energies": [r.ee[i] for i in range(c.norb)], "sweeps": r.sweeps,
             "latency_p50_s": statistics.median(lat[n]),
             "batch_mode": dict((x[0], x[2]) for x in SCF_LEGS)[n],
             "sweeps_per_relaxation": dict((x[0], x[3]) for x in SCF_LEGS)[n] or c.maxsor_orb}
        if fp64_e is not None and n != "fp64":
            d["dE_vs_fp64"] = abs(r.total_energy - fp64_e)
            d["max_dee_vs_fp64"] = max(abs(r.ee[i] - res["fp64"].ee[i]) for i in range(c.norb))
            d["speedup_vs_fp64"] = rate[n] / rate["fp64"]
        if "fp64_batched" in res and n.startswith("mixed"):
            d["speedup_vs_fp64_batched"] = rate[n] / rate["fp64_batched"]
        if oref and args.workload not in FIXED_ITERS:
            d["dE_vs_fp64_oracle"] = abs(r.total_energy - oref["total_energy"])
            d["max_dee_vs_fp64_oracle"] = max(abs(r.ee[i] - oref["orbital_energies"][i]) for i in range(c.norb))
        return d

    out = {
        "metric": metric,
        "value": value,
        "unit": unit,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * tot[head[0]] / len(lat[head[0]]),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 sweeps + f64 defect correction (value); f64 (fp64 leg)",
        "data": "synthetic: hydrogenic LCAO start of the reference's own input deck, no dataset",
        "config": workload_config(args.workload),
        "form": {"value": f"{head[0]}: FP32 MCSOR sweeps + FP64 defect correction, "
                          + ("every potential of an SCF iteration in one launch, then every orbital in one "
                             "launch (batch mode 2)" if head[2] == 2 else "the reference's relaxation order"),
                 "fp64": "plain form: FP64 MCSOR in the reference's colour order and relaxation order",
                 "fp64_batched": "plain form, FP64 MCSOR in the reference's colour order, batched like the "
                                 "headline (batch mode 2): the comparator with the same launch shape",
                 "mixed_sweeps40": "the headline form with 40 MCSOR sweeps per relaxation instead of the deck's "
                                   "10 (the mcsor card's maxsor): fewer SCF iterations, same fixed point"},
        "latency_s": {"p50": statistics.median(lat[head[0]]), "p99": p99},
        "e2e": {"value": e2e_value, "unit": unit, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "roofline": {
            "bound": "hbm",
            "kernel": ("k_mixed_cluster (mixed-form FP32 correction sweeps, one 16-CTA cluster per relaxation job, "
                       "band resident in shared memory)" if on_chip else
                       "k_mcsor_f32p (mixed-form FP32 correction sweeps, persistent-band cooperative kernel: "
                       "every block keeps one band of one job in shared memory for the whole launch, halos "
                       "exchanged through L2; the grid's bands do not fit one cluster's shared memory)"),
            "achieved": sweep_gbs_mx, "peak": hbm, "unit": "GB/s",
            "frac": (sweep_gbs_mx / hbm) if sweep_gbs_mx else None, "traffic": traffic,
            "peak_kind": peak_kind,
            "bytes_per_point_update": BYTES_PER_PT[1],
            "note": ("achieved = 16 algorithmic B per point-update / launch time; the correction lives in shared "
                     "memory during the sweeps, so DRAM traffic is far below it and the launch is bound by the "
                     "colour-phase latency (cluster barrier + shared-memory pipe), not by HBM" if on_chip else
                     "achieved = 16 algorithmic B per point-update / launch time; the correction stays in shared "
                     "memory for the whole launch, so DRAM traffic stays far below the algorithmic bytes and the "
                     "launch is bound by phase latency (neighbour wait, halo round trip, level chain), not by HBM"),
            "sweep_ms_total": msmx, "sweep_launches": nmx, "point_updates": ptsmx,
            "point_updates_per_launch": pts_per_launch,
            # SM-side utilisation of the on-chip sweep (ncu --set full, one launch of 16 potentials on
            # this grid; profiles/mixed_cluster_pot_sweep_poisson_b16_331x481.md): the kernel's bound
            "sm_side_ncu": ({"l1_shared_throughput_frac": 0.524, "issue_active_frac": 0.439,
                             "lsu_instruction_frac": 0.342, "fma_pipe_frac": 0.194,
                             "barrier_stalls_per_issue": 7.63} if on_chip else None),
            "clusters_co_resident": {"plain": occ[0], "potentials_variant": occ[1],
                                     "potentials_variant_mode": args.potential_clusters},
            "colouring": args.colouring,
            "residual_overlap": args.residual_overlap,
            "orthonormalise": args.orthonormalise,
            "fp64_kernel": {"kernel": "k_mcsor_f64", "achieved_gbs": sweep_gbs_64,
                            "frac_hbm": (sweep_gbs_64 / hbm) if sweep_gbs_64 else None,
                            "achieved_tflops": pts64 * FLOPS_PER_PT / (ms64 / 1e3) / 1e12 if ms64 > 0 else None,
                            "bound": "fp64 ALU (1.19 TFLOP/s measured on this GB300)",
                            "sweep_ms_total": ms64, "sweep_launches": n64,
                            "batched": {"achieved_tflops": (ptsb64 * FLOPS_PER_PT / (msb64 / 1e3) / 1e12
                                                            if msb64 > 0 else None),
                                        "sweep_ms_total": msb64, "sweep_launches": nb64,
                                        "point_updates_per_launch": ptsb64 / nb64 if nb64 else None}},
        },
        "clocks": sampler.summary(),
    }
    for n in names:
        out[n] = form(n)
    if oref:
        out["fp64_oracle"] = dict(oref, source="tests/golden/n2_331x481_oracle.json (FP64 oracle, reference order)")
    if not args.no_cpu_baseline:
        nthreads = min(16, os.cpu_count() or 1)
        out["cpu_baseline"] = cpu_baseline(args.workload, deck,
                                           min(args.cpu_iters, 4) if args.workload in FIXED_ITERS else args.cpu_iters,
                                           nthreads)
    return out


POISSON_BATCHES = (16, 64, 256)


def run_poisson(args):
    """Batched Poisson relaxation (survey config 2: R=2.0, 337x481 ->
    331x481, R_inf=40): B independent potentials with sources psi_a psi_b g
    from seeded Slater functions, one relaxation call of 10 MCSOR sweeps
    each, every B in {16, 64, 256} in the plain FP64 form and in the mixed
    form (FP32 sweeps + FP64 defect correction).  A step is one relaxation
    call over the whole batch; reports point-updates/s per (B, form), the
    sweep kernels' algorithmic GB/s from a separate profiled step, and the
    mixed form's largest deviation from the FP64 result relative to the
    change the call made."""
    import numpy as np
    import torch
    import x2dhf_gb300 as xg
    from x2dhf_gb300 import build

    build.build()
    ctx = xg.Context(0)
    _configure(ctx, args)
    nnu, nmu, r, rinf = 331, 481, 2.0, 40.0
    grid = xg.Grid(ctx, nnu, nmu, r, rinf, 1.0, 1.0)
    dev = torch.device("cuda:0")
    n8, m8 = nnu + 8, nmu + 8
    omega_orb, omega_pot = C_double_pair(xg, nnu, nmu)
    stream = torch.cuda.ExternalStream(xg.lib().x2g_stream(ctx.h))
    batches = [args.batch] if args.batch else list(POISSON_BATCHES)
    forms = [args.precision] if args.precision else ["fp64", "mixed"]
    hbm, peak_kind = peaks()
    runs = []
    sampler = ClockSampler(0)
    with sampler:
        for B in batches:
            src = slater_sources(rinf, nnu, nmu, r, B)
            keep, start = [], []
            for pa, pb in src:
                ua = torch.zeros(m8, n8, dtype=torch.float64, device=dev)
                ub = torch.zeros_like(ua)
                ua[4:nmu + 4, 4:nnu + 4] = torch.from_numpy(pa[0])
                ub[4:nmu + 4, 4:nnu + 4] = torch.from_numpy(pb[0])
                keep += [ua, ub]
                start.append((ua, ub, abs(pa[1] - pb[1])))
            results = {}
            for form in forms:
                prec = xg.MIXED if form == "mixed" else xg.FP64
                us = [torch.zeros(m8, n8, dtype=torch.float64, device=dev) for _ in start]
                jobs = [xg.Job(u=u.data_ptr(), psa=ua.data_ptr(), psb=ub.data_ptr(), omega=omega_pot,
                               isym=1 if idel % 2 == 0 else -1, idel=idel, kind=1)
                        for u, (ua, ub, idel) in zip(us, start)]
                torch.cuda.synchronize()
                # the first call from zero is the result compared between the forms
                xg.relax(ctx, grid, jobs, 10, prec)
                ctx.synchronize()
                results[form] = [u.clone() for u in us]
                for _ in range(args.warmup):
                    xg.relax(ctx, grid, jobs, 10, prec)
                ctx.synchronize()
                ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                ev0.record(stream)
                for _ in range(args.steps):
                    xg.relax(ctx, grid, jobs, 10, prec)
                ev1.record(stream)
                ctx.synchronize()
                ms = ev0.elapsed_time(ev1) / args.steps
                ctx.profile(2, prec)
                xg.relax(ctx, grid, jobs, 10, prec)
                ctx.synchronize()
                kms, pts, nl = ctx.profile(-1, prec)
                ctx.profile(0, prec)
                pts_step = B * (nnu - 2) * (nmu - 5) * 10
                bpp = BYTES_PER_PT[1 if prec == xg.MIXED else 0]
                gbs = pts * bpp / (kms / 1e3) / 1e9
                runs.append({"batch": B, "form": form, "point_updates_per_s": pts_step / (ms / 1e3), "ms_per_call": ms,
                             "sweep_kernel_gbs": gbs, "frac": gbs / hbm, "sweep_kernel_ms": kms,
                             "sweep_launches": nl,
                             "fp64_tflops": (pts * FLOPS_PER_PT / (kms / 1e3) / 1e12) if prec == xg.FP64 else None})
            if "fp64" in results and "mixed" in results:
                worst = 0.0
                for a, b in zip(results["fp64"], results["mixed"]):
                    worst = max(worst, float((a - b).abs().max() / a.abs().max()))
                for run in runs:
                    if run["batch"] == B and run["form"] == "mixed":
                        run["max_rel_dev_vs_fp64"] = worst
            del keep
    head = [x for x in runs if x["form"] == forms[-1]][-1]
    return {"metric": "point-updates/s (batched Poisson MCSOR)", "value": head["point_updates_per_s"],
            "unit": "point-updates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": head["ms_per_call"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 sweeps + f64 defect correction (mixed); f64 (fp64)", "data": "synthetic: seeded Slater sources",
            "config": {"workload": f"poisson: B={batches} Slater-product sources (exponents U[0.5,8], l<=3, m<=2), "
                                   "331x481, R=2.0, R_inf=40, 10 MCSOR sweeps per solve, FP64 and mixed",
                       "l2": "not flushed: the B=16 batch (~64 MB) fits in L2, B=64 and B=256 (~0.26 and ~1 GB) "
                             "exceed it"},
            "runs": runs,
            "roofline": {"bound": "hbm", "achieved": head["sweep_kernel_gbs"], "peak": hbm, "unit": "GB/s",
                         "frac": head["frac"], "peak_kind": peak_kind, "traffic": None,
                         "kernel": f"{head['form']} sweep kernel at B={head['batch']}"},
            "clocks": sampler.summary()}


def run_serve(args):
    """Serving loop (survey config 5): seeded Poisson arrivals of closed-shell
    diatomic HF solves (H2, LiH, FH, CO, N2 decks of the reference; bond
    length U[1.5, 5.0] bohr within [0.8, 1.5] x the deck's; grids 169..505 x
    241..721 before rounding, R_inf=40), `--slots` concurrent solves on one
    GPU, each in the batched mode; the mixed form and the FP64 form on the
    same request stream, and the mixed form again under an HBM budget of 1.2
    times the largest request, which admits one large solve at a time."""
    import x2dhf_gb300 as xg
    from x2dhf_gb300 import build, serve

    build.build()
    templates = {}
    for n in ("h2", "lih", "fh", "co", "n2"):
        with open(os.path.join(ROOT, "tests", "golden", n + "_set01.input")) as f:
            templates[n] = f.read()
    reqs = serve.make_requests(templates, args.requests, rate=args.rate, seed=42)
    # warm-up: one request per template, not timed
    warm = [q for i, q in enumerate(reqs) if q.template not in {r.template for r in reqs[:i]}]
    tight = int(1.2 * max(q.bytes for q in reqs))
    out = {}
    sampler = ClockSampler(0)
    with sampler:
        for name, prec, budget in (("mixed", xg.MIXED, 64 << 30), ("fp64", xg.FP64, 64 << 30),
                                   ("mixed_tight_budget", xg.MIXED, tight)):
            srv = serve.Server(slots=args.slots, precision=prec, hbm_budget=budget)
            srv.run(warm, realtime=False)
            done, wall = srv.run(reqs)
            out[name] = dict(serve.summary(done, wall), peak_footprint_bytes=srv.peak_bytes, hbm_budget_bytes=budget,
                             budget_waits=srv.budget_waits)
            out[name + "_energies"] = [c.total_energy for c in done]
            out[name + "_converged"] = [c.converged for c in done]
            if name == "mixed":
                # every request: template, grid, bond length, SCF iterations, exit (0: the iteration cap
                # or stagnation, 1: energy threshold, 2: norm threshold), and the error of a failed one
                out[name]["per_request"] = [[q.template, q.nnu, q.nmu, round(q.r, 4), c.iterations, c.converged]
                                            + ([c.error] if c.error else []) for q, c in zip(reqs, done)]
        # the mixed form at other arrival rates (the same seeded stream,
        # arrival times scaled): throughput and latency against the load
        sweep = []
        for rate in [float(x) for x in args.rates.split(",") if x.strip()] if args.rates else []:
            rq = serve.make_requests(templates, args.requests, rate=rate, seed=42)
            srv = serve.Server(slots=args.slots, precision=xg.MIXED)
            done, wall = srv.run(rq)
            sm = serve.summary(done, wall)
            sweep.append({"rate": rate, "solves_per_s": sm["solves_per_s"], "latency_p50_s": sm["latency_p50_s"],
                          "latency_p99_s": sm["latency_p99_s"], "converged": sm["converged"]})
    # failed requests (recorded with NaN energies and their error) are left out
    de = max((abs(a - b) for a, b in zip(out["mixed_energies"], out["fp64_energies"]) if a == a and b == b),
             default=None)
    both = [i for i, (a, b) in enumerate(zip(out["mixed_converged"], out["fp64_converged"])) if a and b]
    de_conv = max((abs(out["mixed_energies"][i] - out["fp64_energies"][i]) for i in both), default=None)
    same = out["mixed_energies"] == out["mixed_tight_budget_energies"]
    mx, f64 = out["mixed"], out["fp64"]
    return {"metric": "served SCF solves/s and p99 latency (Poisson arrivals), mixed vs FP64", "value":
            mx["solves_per_s"], "unit": "SCF solves/s", "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": 1e3 * mx["wall_s"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 sweeps + f64 defect correction", "data": "synthetic: seeded request stream",
            "config": {"workload": f"serve: {args.requests} requests, rate {args.rate}/s, {args.slots} slots, "
                                   "H2/LiH/FH/CO/N2, R in U[1.5,5.0] within [0.8,1.5] x R_eq, grids 169..505 x "
                                   "241..721 -> 151..481 x 241..721, R_inf=40, batched SCF mode"},
            "latency_s": {"p50": mx["latency_p50_s"], "p99": mx["latency_p99_s"],
                          "fp64_p50": f64["latency_p50_s"], "fp64_p99": f64["latency_p99_s"]},
            "mixed": mx, "fp64": f64, "mixed_tight_budget": out["mixed_tight_budget"],
            "max_dE_mixed_vs_fp64": de, "max_dE_mixed_vs_fp64_both_converged": de_conv,
            "both_converged": len(both), "tight_budget_energies_identical": same, "rate_sweep": sweep,
            "clocks": sampler.summary()}


def C_double_pair(xg, nnu, nmu):
    import ctypes as C
    a, b = C.c_double(), C.c_double()
    xg.lib().x2g_default_omega(nnu, nmu, 1.0, 1.0, C.byref(a), C.byref(b))
    return a.value, b.value


# Full solves by the reference's own C relaxation kernels under the
# oracle's SCF driver, written by oracle/ref_solves.py: the iteration count
# that scales a bounded sample of SCF iterations to one solve
REF_SOLVES = os.path.join(ROOT, "oracle", "ref_solves.json")
# workloads whose full solve on the host cores fits one bench step
REF_FULL_SOLVE = {"h2"}


def ref_solve_record(name):
    """The full reference solve of a workload (None when there is none: a
    solve of the largest grid on the host cores would take hours)."""
    try:
        with open(REF_SOLVES) as f:
            return json.load(f).get(name)
    except (OSError, ValueError):
        return None


def _ref_backend(deck, nthreads):
    """The reference's own C relaxation backend (oracle/_ref, built from the
    x2dhf sources) under the oracle's SCF driver; the oracle port when the
    reference sources could not be built."""
    from oracle import pyoracle, pyref

    pyoracle.build()
    if pyref.available():
        return pyref.ReferenceSCF(deck, nthreads=nthreads), "reference"
    return pyoracle.Case(deck), "port"


def cpu_sample(deck, sample_iters, nthreads):
    """prepSCF + 1 iteration, then `sample_iters` timed SCF iterations:
    (setup seconds, seconds per iteration, backend kind)."""
    t0 = time.perf_counter()
    c, kind = _ref_backend(deck, nthreads)
    c.steps(1)
    t1 = time.perf_counter()
    c.steps(sample_iters)
    t2 = time.perf_counter()
    return (t1 - t0), (t2 - t1) / sample_iters, kind


def cpu_full_solve(deck, nthreads):
    """One full SCF solve to the driver's convergence exit: (seconds, iterations, kind)."""
    t0 = time.perf_counter()
    c, kind = _ref_backend(deck, nthreads)
    c.steps(1 << 30)
    recs = c.records()
    return time.perf_counter() - t0, (recs[-1][0] if recs else 0), kind


def host_cpu():
    model = platform.processor() or platform.machine()
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith(("model name", "cpu part")):
                    model = ln.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    return {"nproc": os.cpu_count(), "model": model, "machine": platform.machine()}


def cpu_kernel_rates(names, max_threads, reps=3):
    """Sweeps/s of the reference's own C kernels on each workload's grid
    (survey measurement plan): sorpt_ on one thread over the "middle" list
    (list-order SOR of a potential, src/c/sorpt.c:11-121) and on the colour
    lists, and mcsor_pthread_ (src/c/mcsor_pthread.c:32) on 1, 2, 4, ...
    threads for an orbital.  One call is maxsor2 = 10 sweeps."""
    import numpy as np
    from oracle import pyoracle, pyref

    pyoracle.build()
    if not pyref.available():
        return None
    out = []
    for name in names:
        oc = pyoracle.Case(WORKLOADS[name]())
        rk = pyref.RefKernels(oc)
        npts = (oc.nni - 2) * (oc.nmu - 5)
        f1, f2 = oc.fock(1)
        lhs_o, rhs_o = f1 + oc.coeffs()[5], f2
        u_o = oc.putin(1, oc.orbital(1))
        in1, in2, idel, isym = oc.pot_info(1, 1)
        lhs_p = oc.suppl(7)
        rhs_p = oc.orbital(in1) * oc.orbital(in2) * oc.suppl(9)
        u_p = oc.putin(isym, oc.pot(1, 1))
        oo, op = oc.omega()

        def rate(fn):
            fn()
            t0 = time.perf_counter()
            for _ in range(reps):
                fn()
            return 10 * reps / (time.perf_counter() - t0)

        row = {"workload": name, "grid": [oc.nni, oc.nmu], "points_per_sweep": npts,
               "sorpt_sor_1t_sweeps_per_s": rate(lambda: rk.sorpt(isym, op, u_p, lhs_p, rhs_p, False)),
               "sorpt_colour_1t_sweeps_per_s": rate(lambda: rk.sorpt(isym, op, u_p, lhs_p, rhs_p, True)),
               "mcsor_pthread_sweeps_per_s": {}}
        t = 1
        while t <= max_threads:
            row["mcsor_pthread_sweeps_per_s"][str(t)] = rate(lambda: rk.mcsor(1, t, oo, u_o, lhs_o, rhs_o))
            t *= 2
        best = max(row["mcsor_pthread_sweeps_per_s"].values())
        row["best_point_updates_per_s"] = best * npts
        out.append(row)
        del rk, oc
    return out


CPU_KERNEL_GRIDS = ("h2", "n2", "kf")


def cpu_baseline(name, deck, sample_iters, nthreads, kernels=True):
    """The reference's C relaxation kernels (one thread per potential,
    mcsor_pthread_ on `nthreads` threads) under the oracle's SCF driver on a
    bounded sample of the same workload, plus the per-kernel sweep rates."""
    if name in FIXED_ITERS or (name not in REF_FULL_SOLVE and ref_solve_record(name) is None):
        setup, per_iter, kind = cpu_sample(deck, sample_iters, nthreads)
        out = {"value": 1.0 / per_iter, "unit": "SCF iterations/s", "cores": nthreads, "kind": kind,
               "sample": f"setup + prepSCF + 1 iteration ({setup:.2f} s), then {sample_iters} timed SCF "
                         f"iterations ({per_iter:.3f} s/iteration) on {nthreads} threads"}
    elif name in REF_FULL_SOLVE:
        wall, iters, kind = cpu_full_solve(deck, nthreads)
        out = {"value": 1.0 / wall, "unit": UNIT, "cores": nthreads, "kind": kind,
               "sample": f"one full SCF solve ({iters} iterations, {wall:.2f} s) on {nthreads} threads"}
    else:
        rec = ref_solve_record(name)
        setup, per_iter, kind = cpu_sample(deck, sample_iters, nthreads)
        solve_s = setup + per_iter * (rec["iterations"] - 1)
        out = {"value": 1.0 / solve_s, "unit": UNIT, "cores": nthreads, "kind": kind,
               "sample": f"setup + prepSCF + 1 iteration ({setup:.2f} s), then {sample_iters} SCF iterations "
                         f"({per_iter:.3f} s/iteration) on {nthreads} threads; scaled to the "
                         f"{rec['iterations']} iterations of a full reference solve (oracle/ref_solves.json)",
               "extrapolated": True}
    out["host"] = host_cpu()
    if kernels:
        out["kernels"] = cpu_kernel_rates(CPU_KERNEL_GRIDS, nthreads)
    return out


def run_reference(args):
    """The reference's own CPU implementation of the path on the host cores,
    on the GPU arm's workload, metric, unit and config.  A step is one full
    SCF solve where that fits (h2), else a bounded sample of SCF iterations
    whose rate is scaled to one solve by the iteration count of a full
    reference solve (oracle/ref_solves.json); ms_per_step is always the
    time the step actually took."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    name = args.workload
    if name not in FIXED_ITERS and name not in REF_FULL_SOLVE and ref_solve_record(name) is None:
        return {"impl": "reference", "unavailable": "no full reference solve of this workload is on record (hours on "
                                                    "the host cores); the kf workload times its SCF iterations"}
    deck = WORKLOADS[name]()
    nthreads = min(16, os.cpu_count() or 1)
    walls, vals, kind, note = [], [], "port", ""
    for step in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        if name in FIXED_ITERS:
            setup, per_iter, kind = cpu_sample(deck, min(args.cpu_iters, 4), nthreads)
            v = 1.0 / per_iter
            note = (f"per step: setup + prepSCF + 1 iteration, then {min(args.cpu_iters, 4)} timed SCF iterations "
                    f"on {nthreads} threads")
        elif name in REF_FULL_SOLVE:
            wall, iters, kind = cpu_full_solve(deck, nthreads)
            v = 1.0 / wall
            note = f"per step: one full SCF solve ({iters} iterations) on {nthreads} threads"
        else:
            rec = ref_solve_record(name)
            setup, per_iter, kind = cpu_sample(deck, args.cpu_iters, nthreads)
            assert rec is not None
            v = 1.0 / (setup + per_iter * (rec["iterations"] - 1))
            note = (f"per step: setup + prepSCF + {1 + args.cpu_iters} SCF iterations on {nthreads} threads; the "
                    f"solve rate scales the timed iterations to the {rec['iterations']} iterations of a full "
                    f"reference solve (oracle/ref_solves.json)")
        if step >= args.warmup:
            walls.append(time.perf_counter() - t0)
            vals.append(v)
    unit = "SCF iterations/s" if name in FIXED_ITERS else UNIT
    metric = (f"SCF iterations/s over the first {FIXED_ITERS[name]} iterations: mixed vs FP64 MCSOR, 1 GB300"
              if name in FIXED_ITERS else METRIC)
    value = (args.steps / sum(walls)) if name in REF_FULL_SOLVE else statistics.median(vals)
    out = {
        # n_gpus: the N this arm was launched for, as the GPU arm's line; the work runs on host cores
        "metric": metric, "value": value, "unit": unit, "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(walls) / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic: hydrogenic LCAO start of the reference's input",
        "impl": "reference", "config": workload_config(name),
        "cpu_baseline": {"value": value, "unit": unit, "cores": nthreads, "kind": kind, "sample": note,
                         "host": host_cpu()},
        "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if name not in FIXED_ITERS and name not in REF_FULL_SOLVE:
        out["extrapolated"] = {"from": "timed SCF iterations of each step", "iterations_per_solve":
                               ref_solve_record(name)["iterations"], "source": "oracle/ref_solves.json"}
    return out


def run_window(args):
    """Profiling window of an SCF workload's headline form: `warm` SCF
    iterations, then `n` more inside a CUDA profiler range (for
    ncu --profile-from-start off); prints the library's launches per
    iteration in the window.  Not a bench line."""
    import torch
    import x2dhf_gb300 as xg
    from x2dhf_gb300 import build

    warm, n = (int(x) for x in args.window.split(","))
    name, prec, mode, sweeps = [lg for lg in SCF_LEGS if args.legs == "all" or lg[0] == args.legs][-1]
    build.build()
    ctx = xg.Context(0)
    _configure(ctx, args)
    s = xg.SCF(ctx, xg.parse_deck(deck_with_sweeps(WORKLOADS[args.workload](), sweeps), precision=prec,
                                  batch_mode=mode))
    s.run(warm)
    ctx.synchronize()
    l0 = ctx.launches
    torch.cuda.profiler.start()
    s.run(n)
    ctx.synchronize()
    torch.cuda.profiler.stop()
    print(json.dumps({"window": f"{args.workload} {name}: iterations {warm + 1}..{warm + n}",
                      "launches_per_iteration": (ctx.launches - l0) / n}))
    return None


def _configure(ctx, args):
    """Context options the command line sets."""
    mode = getattr(args, "potential_clusters", "auto")
    ctx.set_potential_clusters("auto" if mode == "auto" else mode == "on")
    ctx.set_mixed_colouring(getattr(args, "colouring", "reference"))
    ctx.set_residual_overlap(getattr(args, "residual_overlap", "on") == "on")
    ctx.set_gram_orthonormalise(getattr(args, "orthonormalise", "rounds") == "gram")


def main():
    faulthandler.enable()  # a fatal signal prints the Python stack to stderr
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="n2", choices=sorted(WORKLOADS) + ["poisson", "serve"])
    ap.add_argument("--requests", type=int, default=48, help="serve workload: requests in the stream")
    ap.add_argument("--rate", type=float, default=4.0, help="serve workload: mean arrivals per second")
    ap.add_argument("--slots", type=int, default=4, help="serve workload: concurrent solves")
    ap.add_argument("--rates", default="", help="serve workload: comma-separated further arrival rates for the "
                                                "mixed form (a load sweep)")
    ap.add_argument("--cpu-iters", type=int, default=12)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--legs", default="all", choices=["all"] + [lg[0] for lg in SCF_LEGS],
                    help="SCF workloads: time every form (default) or one (for profiling runs)")
    ap.add_argument("--fp64-steps", type=int, default=2,
                    help="SCF workloads: timed solves of the slow plain FP64 comparator")
    ap.add_argument("--batch", type=int, default=0,
                    help="poisson workload: one batch size (default: every size of the configuration)")
    ap.add_argument("--precision", default="", choices=["", "mixed", "fp64"],
                    help="poisson workload: one form (default: both)")
    ap.add_argument("--potential-clusters", default="auto", choices=["auto", "on", "off"],
                    help="mixed form: cluster sweep of potential batches at two CTAs per SM "
                         "(default: for batches above the plain kernel's co-resident clusters)")
    ap.add_argument("--residual-overlap", default="on", choices=["on", "off"],
                    help="mixed form: second-wave potentials' FP64 residual beside the first wave's sweep")
    ap.add_argument("--orthonormalise", default="rounds", choices=["rounds", "gram"],
                    help="batch mode 2: orthonormalisation in rounds (the loop's sums) or through the Gram matrix")
    ap.add_argument("--colouring", default="reference", choices=["reference", "free"],
                    help="mixed form: colouring of the on-chip cluster sweep")
    ap.add_argument("--window", default="", help="WARM,N: profile SCF iterations WARM+1..WARM+N of the headline form "
                                                 "inside a CUDA profiler range (no bench line)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.window:
        out = run_window(args)
    elif args.workload == "poisson":
        out = run_poisson(args)
    elif args.workload == "serve":
        out = run_serve(args) if args.impl != "reference" else {
            "impl": "reference", "unavailable": "the reference has no serving loop (config 5 is GPU-side only)"}
    else:
        out = run_reference(args) if args.impl == "reference" else run_gpu(args)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
