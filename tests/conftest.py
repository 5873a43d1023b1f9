import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than ~20 s on one CPU core")


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_deck(name):
    with open(os.path.join(GOLDEN, name + ".input")) as f:
        return f.read()


def golden_json(name):
    import json
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        return json.load(f)
