import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.json")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 host)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Compile libwbpr and the oracle once per session (no-op when current)."""
    from wbpr_gb300 import build as wb
    from oracle.build_oracle import build_oracle

    wb.build()
    build_oracle()


@pytest.fixture(scope="session")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)["cases"]


@pytest.fixture(scope="session")
def has_gpu():
    import wbpr_gb300 as W

    return W.device_count() > 0


def graph_of(case):
    import numpy as np
    import wbpr_gb300 as W

    arcs = np.asarray(case["arcs"], dtype=np.int64).reshape(-1, 3)
    return W.Graph.from_arcs(case["n"], arcs[:, 0], arcs[:, 1], arcs[:, 2], case["s"], case["t"])
