"""bench.py helpers that run without a GPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def test_workload_config_names_grid_and_points():
    """Both bench arms print the same workload config: the workload's text,
    its grid after the reference's rounding and its points per sweep."""
    import bench

    c = bench.workload_config("n2")
    assert c["workload"].startswith("n2: ")
    assert c["grid"] == [331, 481] and c["points_per_sweep"] == 329 * 476
    k = bench.workload_config("kf")
    assert k["grid"] == [781, 1201] and k["points_per_sweep"] == 931684
    assert bench.workload_config("h2")["grid"] == [151, 241]


def test_bench_grid_rounding_equals_library():
    """The bench's plain-Python grid rounding (used by the reference arm,
    which must not load the GPU library) equals the library's."""
    import bench
    import x2dhf_gb300 as xg

    for n in range(7, 1400):
        assert bench.round_grid(n) == xg.round_grid(n), n


def test_reference_arm_runs_without_the_gpu_library():
    """--impl reference times real full H2 solves of the reference's C
    kernels, prints the GPU arm's config, and never loads libx2dhf_gpu.so."""
    code = (
        "import runpy, sys\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--workload', 'h2', '--steps', '1', '--warmup', '3']\n"
        "runpy.run_path('bench.py', run_name='__main__')\n"
        "maps = open('/proc/self/maps').read()\n"
        "print('LOADED', int('x2dhf_gb300' in sys.modules), int('libx2dhf_gpu' in maps))\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = r.stdout.strip().splitlines()
    assert lines[-1] == "LOADED 0 0", lines[-1]
    out = json.loads(lines[-2])
    import bench

    assert out["impl"] == "reference" and out["unit"] == bench.UNIT and out["metric"] == bench.METRIC
    assert out["config"] == bench.workload_config("h2")
    assert out["steps"] == 1 and out["warmup"] == 3
    # a full solve per step: the rate is the inverse of the step time
    assert abs(out["value"] * out["ms_per_step"] / 1e3 - 1.0) < 1e-9
    assert out["cpu_baseline"]["kind"] == "reference"


def test_reference_solve_fixture_present():
    """The iteration counts that scale the reference arm's N2 sample come from
    oracle/ref_solves.py's full solves, not from a constant."""
    with open(os.path.join(ROOT, "oracle", "ref_solves.json")) as f:
        d = json.load(f)
    for name, grid in (("h2", [151, 241]), ("n2", [331, 481])):
        assert d[name]["grid"] == grid and d[name]["iterations"] > 100
        assert d[name]["total_energy"] < 0


def test_sweeps_leg_deck_sets_maxsor():
    """The 40-sweep leg rewrites the deck's mcsor / mcsor-ce cards only: the
    MCSOR schemes stay and both sweep counts become 40; 0 keeps the deck."""
    import bench
    import x2dhf_gb300 as xg

    deck = bench.n2_deck()
    assert bench.deck_with_sweeps(deck, 0) == deck
    c0, c40 = xg.parse_deck(deck), xg.parse_deck(bench.deck_with_sweeps(deck, 40))
    assert (c0.maxsor_orb, c0.maxsor_pot) == (10, 10)
    assert (c40.maxsor_orb, c40.maxsor_pot) == (40, 40)
    assert (c40.orb_scheme, c40.pot_scheme) == (c0.orb_scheme, c0.pot_scheme) == (1, 1)
    assert (c40.nnu, c40.nmu, c40.r) == (c0.nnu, c0.nmu, c0.r)
