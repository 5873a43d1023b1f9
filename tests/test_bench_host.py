"""bench.py helpers that run without a GPU."""
import os
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
